// link.cu -- linking the centerpoint vertices into centerline trees: the back
// half of runNewCenterlineAlg (parallelCenterlineExtraction.cpp:911-1332) with
// the kernels linkLengths, compact, linkCenterpoints, removeDuplicateEdges,
// graphComponentLabeling, calculateTreeLength and removeSmallTrees
// (kernels.cl:327-559) and the 2-D histogram-pyramid enumeration of the edge
// image (kernels.cl:100-142, 229-325).
//
// Per vertex a, the candidate partners are the vertices b with
// 0 < |a - b| < max-distance; a links to the pair (b, c) that minimises
// round|ab| + round|ac| subject to an angle of at least 2 rad between ab and ac
// and a mean TDF >= min-mean-tdf along both segments (sampled at 0..round|ab|
// with the linear sampler).  The reference appends candidates with atomics
// (nondeterministic order, which decides ties of equal distance sums); here
// they are listed in ascending vertex order, one warp per vertex with a
// ballot, so the result is deterministic.
//
// Edges: tuple (a, b) for each chosen partner; (a, b) with a > b is dropped
// when (b, a) exists (removeDuplicateEdges).  The reference enumerates the
// tuple image with a 2-D pyramid whose children are visited (0,0), (0,1),
// (1,0), (1,1) -- i.e. in ascending order of the key interleaving the bits of
// (a, b) with b as the low bit -- so the tuples are sorted by that key (one
// CTA, bitonic sort in shared memory).
//
// Labels: graphComponentLabeling propagates the smaller label across every
// edge until nothing changes; whatever the order of its atomics it ends with
// every vertex labelled by the smallest index in its component, which one CTA
// computes in shared memory here; calculateTreeLength counts the component
// sizes.  removeSmallTrees rasterises the edges of components of at least
// min-tree-length vertices.
#include "tdf_common.cuh"

namespace tsf {

constexpr int kLinkMaxVertices = 16384;   // the candidate stage keeps fewer (parallelCenterlineExtraction.cpp:895-899)

__device__ __forceinline__ float vdist(const int *v, int a, int b) {
    const float dx = (float)v[3 * a] - (float)v[3 * b];
    const float dy = (float)v[3 * a + 1] - (float)v[3 * b + 1];
    const float dz = (float)v[3 * a + 2] - (float)v[3 * b + 2];
    return sqrtf((dx * dx + dy * dy) + dz * dz);
}

// linkLengths + compact: row a lists (length, b) for 0 < |ab| < maxd, b ascending
__global__ void link_lists_kernel(const int *__restrict__ v, int n, float maxd, float2 *__restrict__ lists,
                                  int *__restrict__ counts) {
    const int a = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (a >= n) return;
    int base = 0;
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int b = b0 + lane;
        const float d = b < n ? vdist(v, a, b) : 0.0f;
        const bool ok = b < n && d < maxd && d > 0.0f;
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (ok) lists[(int64_t)a * n + base + __popc(m & ((1u << lane) - 1u))] = make_float2(d, (float)b);
        base += __popc(m);
    }
    if (lane == 0) counts[a] = base;
}

// the TDF (float or unorm16) through the linear sampler, clamp to edge
__device__ __forceinline__ float tdf_texel(const void *T, int unorm, int64_t i) {
    return unorm ? (float)reinterpret_cast<const uint16_t *>(T)[i] / 65535.0f : reinterpret_cast<const float *>(T)[i];
}

__device__ float sample_tdf(const void *T, int unorm, int X, int Y, int Z, float u, float v, float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const int i1 = clampi(i0 + 1, X), j1 = clampi(j0 + 1, Y), k1 = clampi(k0 + 1, Z);
    i0 = clampi(i0, X); j0 = clampi(j0, Y); k0 = clampi(k0, Z);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    float o = ((ia * ib) * ic) * tdf_texel(T, unorm, lin(i0, j0, k0, X, Y));
    o = o + ((a * ib) * ic) * tdf_texel(T, unorm, lin(i1, j0, k0, X, Y));
    o = o + ((ia * b) * ic) * tdf_texel(T, unorm, lin(i0, j1, k0, X, Y));
    o = o + ((a * b) * ic) * tdf_texel(T, unorm, lin(i1, j1, k0, X, Y));
    o = o + ((ia * ib) * c) * tdf_texel(T, unorm, lin(i0, j0, k1, X, Y));
    o = o + ((a * ib) * c) * tdf_texel(T, unorm, lin(i1, j0, k1, X, Y));
    o = o + ((ia * b) * c) * tdf_texel(T, unorm, lin(i0, j1, k1, X, Y));
    o = o + ((a * b) * c) * tdf_texel(T, unorm, lin(i1, j1, k1, X, Y));
    return o;
}

// mean TDF at xa + s * k / d, k = 0..d
__device__ float mean_tdf(const void *T, int unorm, int X, int Y, int Z, const float xa[3], const float s[3], int d) {
    float sum = 0.0f;
    for (int k = 0; k <= d; k++) {
        const float alpha = (float)k / (float)d;
        sum = sum + sample_tdf(T, unorm, X, Y, Z, xa[0] + s[0] * alpha, xa[1] + s[1] * alpha, xa[2] + s[2] * alpha);
    }
    return sum / (float)(d + 1);
}

// acos(d) < 2  <=>  d > cos(2); -0.41614684f is the float just below cos(2)
__device__ __forceinline__ bool angle_below_2(float d) { return d > -0.41614684f; }

// linkCenterpoints (kernels.cl:353-475), one thread per vertex
__global__ void link_kernel(const int *__restrict__ v, int n, const float2 *__restrict__ lists,
                            const int *__restrict__ counts, const void *T, int unorm, int X, int Y, int Z,
                            float min_avg, float maxd, int *__restrict__ partner) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const float xa[3] = {(float)v[3 * a], (float)v[3 * a + 1], (float)v[3 * a + 2]};
    const float2 *row = lists + (int64_t)a * n;
    const int cnt = counts[a];
    float shortest = maxd * 2.0f;
    int best_b = -1, best_c = -1;
    for (int i = 0; i < cnt; i++) {
        const float2 cb = row[i];
        const int b = (int)cb.y;
        const int db = (int)roundf(cb.x);
        if ((float)db >= shortest) continue;
        const float ab[3] = {(float)v[3 * b] - xa[0], (float)v[3 * b + 1] - xa[1], (float)v[3 * b + 2] - xa[2]};
        for (int j = 0; j < i; j++) {
            const float2 cc = row[j];
            const int c = (int)cc.y;
            if (c == b) continue;
            const int dc = (int)roundf(cc.x);
            if (!((float)(db + dc) < shortest)) continue;
            const float ac[3] = {(float)v[3 * c] - xa[0], (float)v[3 * c + 1] - xa[1], (float)v[3 * c + 2] - xa[2]};
            const float lb = sqrtf((ab[0] * ab[0] + ab[1] * ab[1]) + ab[2] * ab[2]);
            const float lc = sqrtf((ac[0] * ac[0] + ac[1] * ac[1]) + ac[2] * ac[2]);
            const float dot = ((ab[0] / lb) * (ac[0] / lc) + (ab[1] / lb) * (ac[1] / lc)) + (ab[2] / lb) * (ac[2] / lc);
            if (angle_below_2(dot)) continue;
            if (mean_tdf(T, unorm, X, Y, Z, xa, ab, db) < min_avg) continue;
            if (mean_tdf(T, unorm, X, Y, Z, xa, ac, dc) < min_avg) continue;
            best_b = b;
            best_c = c;
            shortest = (float)(db + dc);
        }
    }
    partner[2 * a] = best_b;
    partner[2 * a + 1] = best_c;
}

// the key of tuple (x, y) in the 2-D pyramid's enumeration order
__device__ __forceinline__ unsigned hp2d_key(unsigned x, unsigned y) {
    unsigned k = 0;
#pragma unroll
    for (int bit = 0; bit < 16; bit++) k |= (((y >> bit) & 1u) | (((x >> bit) & 1u) << 1)) << (2 * bit);
    return k;
}
__device__ __forceinline__ void hp2d_unkey(unsigned k, int &x, int &y) {
    unsigned xx = 0, yy = 0;
#pragma unroll
    for (int bit = 0; bit < 16; bit++) {
        yy |= ((k >> (2 * bit)) & 1u) << bit;
        xx |= ((k >> (2 * bit + 1)) & 1u) << bit;
    }
    x = (int)xx;
    y = (int)yy;
}

__device__ __forceinline__ bool chose(const int *partner, int a, int b) {
    return partner[2 * a] == b || partner[2 * a + 1] == b;
}

// removeDuplicateEdges (kernels.cl:536-557) as keys; dropped tuples get ~0u
__global__ void edge_keys_kernel(const int *__restrict__ partner, int n, unsigned *__restrict__ keys, int m) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    unsigned key = 0xffffffffu;
    if (t < 2 * n) {
        const int a = t >> 1, b = partner[t];
        if (b >= 0 && (a <= b || !chose(partner, b, a))) key = hp2d_key((unsigned)a, (unsigned)b);
    }
    keys[t] = key;
}

// one CTA: bitonic sort of m (power of two) keys in shared memory, then the
// edge list (x, y) and its length
__global__ void __launch_bounds__(1024) sort_edges_kernel(const unsigned *__restrict__ keys_in, int m,
                                                          int *__restrict__ edges, int *__restrict__ n_edges) {
    extern __shared__ unsigned sk[];
    __shared__ int total;
    if (threadIdx.x == 0) total = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) sk[i] = keys_in[i];
    __syncthreads();
    for (int size = 2; size <= m; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < m / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const unsigned a = sk[lo], b = sk[hi];
                if ((a > b) == up) {
                    sk[lo] = b;
                    sk[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    int cnt = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const unsigned k = sk[i];
        if (k != 0xffffffffu) {
            int x, y;
            hp2d_unkey(k, x, y);
            edges[2 * i] = x;
            edges[2 * i + 1] = y;
            cnt++;
        }
    }
    if (cnt) atomicAdd(&total, cnt);
    __syncthreads();
    if (threadIdx.x == 0) *n_edges = total;
}

// graphComponentLabeling + calculateTreeLength (kernels.cl:477-508): one CTA,
// labels and sizes in shared memory; status 1 if propagation did not settle
// within n + 1 rounds (it always settles within n)
__global__ void __launch_bounds__(1024) label_kernel(const int *__restrict__ edges, const int *__restrict__ n_edges_p,
                                                     int n, int *__restrict__ labels, int *__restrict__ sizes,
                                                     int *__restrict__ status) {
    extern __shared__ int sm[];
    int *C = sm, *S = sm + n;
    const int ne = *n_edges_p;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        C[i] = i;
        S[i] = 0;
    }
    __syncthreads();
    int rounds = 0;
    for (;;) {
        int changed = 0;
        for (int e = threadIdx.x; e < ne; e += blockDim.x) {
            const int a = edges[2 * e], b = edges[2 * e + 1];
            const int ca = C[a], cb = C[b];
            if (ca < cb) {
                atomicMin(&C[b], ca);
                changed = 1;
            } else if (cb < ca) {
                atomicMin(&C[a], cb);
                changed = 1;
            }
        }
        if (!__syncthreads_or(changed)) break;
        if (++rounds > n + 1) {
            if (threadIdx.x == 0) *status = 1;
            break;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&S[C[i]], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        labels[i] = C[i];
        sizes[i] = S[i];
    }
}

// removeSmallTrees (kernels.cl:510-534): rasterise the edges of large trees
__global__ void raster_kernel(const int *__restrict__ v, const int *__restrict__ edges, int ne,
                              const int *__restrict__ labels, const int *__restrict__ sizes, int min_tree,
                              int8_t *__restrict__ out, int X, int Y, int Z) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int a = edges[2 * e], b = edges[2 * e + 1];
    if (sizes[labels[a]] < min_tree) return;
    const float xa[3] = {(float)v[3 * a], (float)v[3 * a + 1], (float)v[3 * a + 2]};
    const float d[3] = {(float)v[3 * b] - xa[0], (float)v[3 * b + 1] - xa[1], (float)v[3 * b + 2] - xa[2]};
    const int l = (int)roundf(sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]));
    for (int i = 0; i < l; i++) {
        const float alpha = (float)i / (float)l;
        const int x = (int)roundf(xa[0] + d[0] * alpha), y = (int)roundf(xa[1] + d[1] * alpha),
                  z = (int)roundf(xa[2] + d[2] * alpha);
        if (x >= 0 && y >= 0 && z >= 0 && x < X && y < Y && z < Z) out[lin(x, y, z, X, Y)] = 1;
    }
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }
static int pow2_at_least(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

struct LinkLayout {
    size_t lists, counts, partner, keys, status, bytes;
    int m;
};
static LinkLayout link_layout(int n) {
    LinkLayout L;
    L.m = pow2_at_least(2 * n > 2 ? 2 * n : 2);
    size_t off = 0;
    L.lists = off; off = al256(off + sizeof(float2) * (size_t)n * n);
    L.counts = off; off = al256(off + sizeof(int) * (size_t)n);
    L.partner = off; off = al256(off + sizeof(int) * 2 * (size_t)n);
    L.keys = off; off = al256(off + sizeof(unsigned) * (size_t)L.m);
    L.status = off; off = al256(off + 2 * sizeof(int));
    L.bytes = off;
    return L;
}

size_t link_workspace_size(int n) { return n > 0 ? link_layout(n).bytes : 0; }

int run_link(const int *d_v, int n, const void *d_T, int unorm, int X, int Y, int Z, float min_avg, float maxd,
             int *d_edges, int *n_edges, int *d_labels, int *d_sizes, void *ws, size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (n <= 0 || n > kLinkMaxVertices) return fail(TSF_ERR_INVALID_ARG, "vertex count must be in [1, 16384]");
    if (!d_v || !d_T || !d_edges || !n_edges || !d_labels || !d_sizes)
        return fail(TSF_ERR_INVALID_ARG, "null buffer");
    const LinkLayout L = link_layout(n);
    if (!ws || ws_bytes < L.bytes) return fail(TSF_ERR_WORKSPACE, "linking workspace too small");
    char *w = (char *)ws;
    float2 *lists = (float2 *)(w + L.lists);
    int *counts = (int *)(w + L.counts), *partner = (int *)(w + L.partner);
    unsigned *keys = (unsigned *)(w + L.keys);
    int *status = (int *)(w + L.status);
    TSF_TRY_CUDA(cudaMemsetAsync(status, 0, 2 * sizeof(int), s));
    link_lists_kernel<<<(n + 7) / 8, 256, 0, s>>>(d_v, n, maxd, lists, counts);
    link_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_v, n, lists, counts, d_T, unorm, X, Y, Z, min_avg, maxd, partner);
    edge_keys_kernel<<<(L.m + 255) / 256, 256, 0, s>>>(partner, n, keys, L.m);
    TSF_CHECK_LAUNCHES("link kernels", 3);
    TSF_TRY_CUDA(cudaFuncSetAttribute(sort_edges_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(L.m * sizeof(unsigned))));
    sort_edges_kernel<<<1, 1024, L.m * sizeof(unsigned), s>>>(keys, L.m, d_edges, status + 1);
    TSF_CHECK_LAUNCH("sort_edges_kernel");
    int ne = 0;
    TSF_TRY_CUDA(cudaMemcpyAsync(&ne, status + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    TSF_TRY_CUDA(cudaStreamSynchronize(s));
    *n_edges = ne;
    if (ne == 0) return fail(TSF_ERR_COUNT_RANGE, "No edges were found");
    TSF_TRY_CUDA(cudaFuncSetAttribute(label_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(2 * n * sizeof(int))));
    label_kernel<<<1, 1024, 2 * n * sizeof(int), s>>>(d_edges, status + 1, n, d_labels, d_sizes, status);
    TSF_CHECK_LAUNCH("label_kernel");
    int st = 0;
    TSF_TRY_CUDA(cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    TSF_TRY_CUDA(cudaStreamSynchronize(s));
    if (st) return fail(TSF_ERR_NOT_CONVERGED, "graph component labelling did not settle");
    return TSF_OK;
}

int run_rasterize_trees(const int *d_v, const int *d_edges, int ne, const int *d_labels, const int *d_sizes,
                        int min_tree, int8_t *d_out, int X, int Y, int Z, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_v || !d_edges || !d_labels || !d_sizes || !d_out || ne < 0)
        return fail(TSF_ERR_INVALID_ARG, "invalid rasterisation arguments");
    if (ne == 0) return TSF_OK;
    raster_kernel<<<(ne + 127) / 128, 128, 0, s>>>(d_v, d_edges, ne, d_labels, d_sizes, min_tree, d_out, X, Y, Z);
    TSF_CHECK_LAUNCH("raster_kernel");
    return TSF_OK;
}

// createCenterlineVoxels' device side (parallelCenterlineExtraction.cpp:
// 287-321): the host lists the cells the kept edges visit; these read the
// radius there and write the centerline mark and the smoothed radius back.
// Cells outside [0, X*Y*Z) are skipped.
__global__ void gather_cells_kernel(const float *__restrict__ vol, int64_t nvox, const int64_t *__restrict__ cells,
                                    int64_t n, float *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p = cells[i];
    out[i] = (p >= 0 && p < nvox) ? vol[p] : 0.0f;
}

__global__ void centerline_apply_kernel(int8_t *__restrict__ cl, float *__restrict__ radius, int64_t nvox,
                                        const int64_t *__restrict__ cells, const float *__restrict__ values,
                                        int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p = cells[i];
    if (p < 0 || p >= nvox) return;
    cl[p] = 1;
    if (radius) radius[p] = values[i];
}

int run_gather_cells(const float *d_vol, int X, int Y, int Z, const int64_t *d_cells, int64_t n, float *d_out,
                     cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (n < 0 || (n > 0 && (!d_vol || !d_cells || !d_out))) return fail(TSF_ERR_INVALID_ARG, "invalid gather arguments");
    if (n == 0) return TSF_OK;
    gather_cells_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_vol, (int64_t)X * Y * Z, d_cells, n, d_out);
    TSF_CHECK_LAUNCH("gather_cells_kernel");
    return TSF_OK;
}

int run_centerline_apply(int8_t *d_cl, float *d_radius, int X, int Y, int Z, const int64_t *d_cells,
                         const float *d_values, int64_t n, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (n < 0 || (n > 0 && (!d_cl || !d_cells || (d_radius && !d_values))))
        return fail(TSF_ERR_INVALID_ARG, "invalid centerline arguments");
    if (n == 0) return TSF_OK;
    centerline_apply_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d_cl, d_radius, (int64_t)X * Y * Z, d_cells,
                                                                       d_values, n);
    TSF_CHECK_LAUNCH("centerline_apply_kernel");
    return TSF_OK;
}

}  // namespace tsf

extern "C" int tsf_gather_cells(const float *d_volume, int X, int Y, int Z, const int64_t *d_cells, int64_t n_cells,
                                float *d_values, void *stream) {
    return tsf::run_gather_cells(d_volume, X, Y, Z, d_cells, n_cells, d_values,
                                 reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_centerline_apply(int8_t *d_centerlines, float *d_radius, int X, int Y, int Z,
                                    const int64_t *d_cells, const float *d_values, int64_t n_cells, void *stream) {
    return tsf::run_centerline_apply(d_centerlines, d_radius, X, Y, Z, d_cells, d_values, n_cells,
                                     reinterpret_cast<cudaStream_t>(stream));
}

extern "C" size_t tsf_link_workspace_size(int n_vertices) { return tsf::link_workspace_size(n_vertices); }

extern "C" int tsf_link_centerpoints(const int *d_vertices, int n_vertices, const void *d_T, int tdf_unorm16, int X,
                                     int Y, int Z, float min_mean_tdf, float max_distance, int *d_edges,
                                     int *n_edges, int *d_labels, int *d_tree_sizes, void *d_workspace,
                                     size_t workspace_bytes, void *stream) {
    return tsf::run_link(d_vertices, n_vertices, d_T, tdf_unorm16, X, Y, Z, min_mean_tdf, max_distance, d_edges,
                         n_edges, d_labels, d_tree_sizes, d_workspace, workspace_bytes,
                         reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_rasterize_trees(const int *d_vertices, const int *d_edges, int n_edges, const int *d_labels,
                                   const int *d_tree_sizes, int min_tree_length, int8_t *d_centerlines, int X, int Y,
                                   int Z, void *stream) {
    return tsf::run_rasterize_trees(d_vertices, d_edges, n_edges, d_labels, d_tree_sizes, min_tree_length,
                                    d_centerlines, X, Y, Z, reinterpret_cast<cudaStream_t>(stream));
}
