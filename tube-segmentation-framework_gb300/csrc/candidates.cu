// candidates.cu -- candidate centerpoints: threshold, compaction in
// histogram-pyramid order, cross-section non-maximum filter and per-cube
// arg-max (reference runNewCenterlineAlg front half,
// parallelCenterlineExtraction.cpp:667-899; kernels findCandidateCenterpoints,
// findCandidateCenterpoints2, dd, constructHPLevel3D / traverseHP3D /
// createPositions3D in kernels.cl).
//
// Compaction.  The reference builds a histogram pyramid (a sum pyramid of
// 2x2x2 cells) and enumerates rank t -> voxel by walking it top-down, visiting
// the 8 children in the order (0,0,0),(1,0,0),(0,0,1),(1,0,1),(0,1,0),(1,1,0),
// (0,1,1),(1,1,1) (kernels.cl:70-79).  The enumeration is therefore the sort
// of the selected voxels by the key K = sum_b (x_b | z_b<<1 | y_b<<2) << 3b.
// Here the volume is cut into 8^3 bricks; an aligned brick is a contiguous K
// range, so the list is produced by (1) counting each brick's selected voxels,
// (2) an exclusive scan of the counts in brick-key order and (3) a pass in
// which every brick ranks its voxels in local key order with warp ballots and
// writes them at its offset.  The result is the reference's list, without
// building or walking a pyramid.
#include "eigen3.cuh"
#include "tsf_common.cuh"

namespace tsf {

enum { FLAG_TDF_F32 = 0, FLAG_TDF_U16 = 1, FLAG_MASK = 2 };

struct BrickGrid {
    int nbx, nby, nbz;  // bricks per axis (ceil(extent / 8))
    int pbits;          // log2 of the enclosing power-of-two brick cube
};

static BrickGrid brick_grid(int X, int Y, int Z) {
    BrickGrid g;
    g.nbx = (X + 7) / 8; g.nby = (Y + 7) / 8; g.nbz = (Z + 7) / 8;
    int m = g.nbx > g.nby ? g.nbx : g.nby;
    if (g.nbz > m) m = g.nbz;
    g.pbits = 0;
    while ((1 << g.pbits) < m) g.pbits++;
    return g;
}

static int64_t brick_keys(const BrickGrid &g) { return (int64_t)1 << (3 * g.pbits); }

// key bits (x0 z0 y0 x1 z1 y1 ...) -> coordinates
__device__ __forceinline__ void decode_key(uint64_t k, int bits, int &x, int &y, int &z) {
    x = y = z = 0;
    for (int b = 0; b < bits; b++) {
        x |= (int)((k >> (3 * b)) & 1) << b;
        z |= (int)((k >> (3 * b + 1)) & 1) << b;
        y |= (int)((k >> (3 * b + 2)) & 1) << b;
    }
}

template <int MODE>
__device__ __forceinline__ int flag_at(const void *src, int64_t i, float thr) {
    if (MODE == FLAG_TDF_F32) return reinterpret_cast<const float *>(src)[i] < thr ? 0 : 1;
    if (MODE == FLAG_TDF_U16) return from_unorm16(reinterpret_cast<const uint16_t *>(src)[i]) < thr ? 0 : 1;
    return reinterpret_cast<const int8_t *>(src)[i] != 0 ? 1 : 0;
}

// Loads one 8^3 brick's flags into shared memory (x fastest) and returns the
// brick origin; false if the brick key lies outside the brick grid.
template <int MODE>
__device__ __forceinline__ bool load_brick(const void *src, float thr, int X, int Y, int Z, BrickGrid g, uint8_t *sflag,
                                           int &ox, int &oy, int &oz) {
    int bx, by, bz;
    decode_key(blockIdx.x, g.pbits, bx, by, bz);
    if (bx >= g.nbx || by >= g.nby || bz >= g.nbz) return false;
    ox = bx * 8; oy = by * 8; oz = bz * 8;
    const int t = threadIdx.x;
    const int lx = t & 7, ly = (t >> 3) & 7, lz = t >> 6;
    const int x = ox + lx, y = oy + ly, z = oz + lz;
    int f = 0;
    if (x < X && y < Y && z < Z) f = flag_at<MODE>(src, lin(x, y, z, X, Y), thr);
    sflag[t] = (uint8_t)f;
    return true;
}

template <int MODE>
__global__ void __launch_bounds__(512) brick_count_kernel(const void *src, float thr, int X, int Y, int Z, BrickGrid g,
                                                          int32_t *counts) {
    __shared__ uint8_t sflag[512];
    int ox, oy, oz;
    const bool in = load_brick<MODE>(src, thr, X, Y, Z, g, sflag, ox, oy, oz);
    if (!in) {                           // uniform over the block
        if (threadIdx.x == 0) counts[blockIdx.x] = 0;
        return;
    }
    const int c = __syncthreads_count(sflag[threadIdx.x]);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// Exclusive scan of n int32 counts into int64 offsets; total -> *total.
// One CTA of 1024 threads, each owning a contiguous segment.
__global__ void __launch_bounds__(1024) scan_counts_kernel(const int32_t *counts, int64_t n, int64_t *offsets,
                                                           int64_t *total) {
    __shared__ int64_t warp_sums[32];
    const int t = threadIdx.x;
    const int64_t seg = (n + 1023) / 1024;
    const int64_t b = (int64_t)t * seg, e = (b + seg < n) ? b + seg : n;
    int64_t s = 0;
    for (int64_t i = b; i < e; i++) s += counts[i];
    // inclusive scan of s over the block
    int64_t v = s;
    const int lane = t & 31, w = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_sums[w] = v;
    __syncthreads();
    if (w == 0) {
        int64_t ws = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += u;
        }
        warp_sums[lane] = ws;
    }
    __syncthreads();
    int64_t run = v - s + (w > 0 ? warp_sums[w - 1] : 0);
    for (int64_t i = b; i < e; i++) {
        offsets[i] = run;
        run += counts[i];
    }
    if (t == 1023) *total = warp_sums[31];
}

template <int MODE>
__global__ void __launch_bounds__(512) brick_write_kernel(const void *src, float thr, int X, int Y, int Z, BrickGrid g,
                                                          const int64_t *offsets, int32_t *pos, int64_t cap) {
    __shared__ uint8_t sflag[512];
    __shared__ int warp_cnt[16];
    int ox, oy, oz;
    const bool in = load_brick<MODE>(src, thr, X, Y, Z, g, sflag, ox, oy, oz);
    if (!in) return;
    __syncthreads();
    const int t = threadIdx.x;                  // local key
    int lx, ly, lz;
    decode_key((uint64_t)t, 3, lx, ly, lz);
    const int f = sflag[lx + 8 * ly + 64 * lz];
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int lane = t & 31, w = t >> 5;
    if (lane == 0) warp_cnt[w] = __popc(bal);
    __syncthreads();
    int before = 0;
    for (int i = 0; i < w; i++) before += warp_cnt[i];
    if (f) {
        const int64_t r = offsets[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u));
        if (r < cap) {
            pos[3 * r + 0] = ox + lx;
            pos[3 * r + 1] = oy + ly;
            pos[3 * r + 2] = oz + lz;
        }
    }
}

// ---------------------------------------------------------------------------
// findCandidateCenterpoints2 (kernels.cl:1309-1390): one warp per candidate.
// ---------------------------------------------------------------------------
template <int ST>
__global__ void __launch_bounds__(256) candidates2_kernel(const float *__restrict__ R, const void *__restrict__ F,
                                                          int X, int Y, int Z, const int32_t *__restrict__ pos,
                                                          int64_t count, float cos_lim, int8_t *mask_out) {
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= count) return;                     // uniform per warp
    const int x = pos[3 * wid], y = pos[3 * wid + 1], z = pos[3 * wid + 2];
    float rr = roundf(R[lin(x, y, z, X, Y)]);
    rr = fminf(rr, 8.0f);
    rr = fmaxf(rr, 1.0f);
    const int maxD = (int)rr;
    // Hessian of the normalised field and its eigenvectors; e1 = tube direction
    const float4 xp = Vec4Load<ST>::load(F, lin(clampi(x + 1, X), y, z, X, Y));
    const float4 xm = Vec4Load<ST>::load(F, lin(clampi(x - 1, X), y, z, X, Y));
    const float4 yp = Vec4Load<ST>::load(F, lin(x, clampi(y + 1, Y), z, X, Y));
    const float4 ym = Vec4Load<ST>::load(F, lin(x, clampi(y - 1, Y), z, X, Y));
    const float4 zp = Vec4Load<ST>::load(F, lin(x, y, clampi(z + 1, Z), X, Y));
    const float4 zm = Vec4Load<ST>::load(F, lin(x, y, clampi(z - 1, Z), X, Y));
    float H[3][3], V[3][3], d[3];
    H[0][0] = 0.5f * (xp.x / xp.w - xm.x / xm.w);
    H[1][0] = H[0][1] = 0.5f * (xp.y / xp.w - xm.y / xm.w);
    H[1][1] = 0.5f * (yp.y / yp.w - ym.y / ym.w);
    H[2][0] = H[0][2] = 0.5f * (xp.z / xp.w - xm.z / xm.w);
    H[2][1] = H[1][2] = 0.5f * (yp.z / yp.w - ym.z / ym.w);
    H[2][2] = 0.5f * (zp.z / zp.w - zm.z / zm.w);
    eig3<float>(H, V, d);
    const float e0 = V[0][0], e1 = V[1][0], e2 = V[2][0];
    const float mag0 = Vec4Load<ST>::load(F, lin(x, y, z, X, Y)).w;
    const int S = 2 * maxD + 1, S3 = S * S * S;
    bool invalid = false;
    for (int o = lane; o < S3; o += 32) {
        const int a = o / (S * S) - maxD, b = (o / S) % S - maxD, c = o % S - maxD;
        if ((a | b | c) == 0) continue;
        if (a * a + b * b + c * c >= maxD * maxD) continue;
        const float r0 = (float)a, r1 = (float)b, r2 = (float)c;
        const float dp = (e0 * r0 + e1 * r1) + e2 * r2;
        const float p0 = r0 - e0 * dp, p1 = r1 - e1 * dp, p2 = r2 - e2 * dp;
        const float lr = sqrtf((r0 * r0 + r1 * r1) + r2 * r2);
        const float lp = sqrtf((p0 * p0 + p1 * p1) + p2 * p2);
        const float dd = ((r0 / lr) * (p0 / lp) + (r1 / lr) * (p1 / lp)) + (r2 / lr) * (p2 / lp);
        if (!(dd >= cos_lim && dd <= 1.0f)) continue;
        const float mag = Vec4Load<ST>::load(F, lin(clampi(x + a, X), clampi(y + b, Y), clampi(z + c, Z), X, Y)).w;
        if (mag < mag0) invalid = true;
    }
    invalid = __any_sync(0xffffffffu, invalid);
    if (lane == 0) mask_out[lin(x, y, z, X, Y)] = invalid ? 0 : 1;
}

// ---------------------------------------------------------------------------
// dd (kernels.cl:1260-1292): one thread per cube of cs^3 voxels.
// ---------------------------------------------------------------------------
template <bool UNORM>
__global__ void dd_kernel(const void *__restrict__ T, const int8_t *__restrict__ cand, int X, int Y, int Z, int cs,
                          int GX, int GY, int GZ, int8_t *out) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (int64_t)GX * GY * GZ) return;
    const int gx = (int)(id % GX), gy = (int)((id / GX) % GY), gz = (int)(id / ((int64_t)GX * GY));
    float best = 0.0f;
    bool found = false;
    int bx = 0, by = 0, bz = 0;
    for (int a = 0; a < cs; a++)
        for (int b = 0; b < cs; b++)
            for (int c = 0; c < cs; c++) {
                const int x = gx * cs + a, y = gy * cs + b, z = gz * cs + c;
                const int64_t i = lin(clampi(x, X), clampi(y, Y), clampi(z, Z), X, Y);
                if (cand[i] == 1) {
                    const float g = UNORM ? from_unorm16(reinterpret_cast<const uint16_t *>(T)[i])
                                          : reinterpret_cast<const float *>(T)[i];
                    if (g > best) {
                        found = true;
                        best = g;
                        bx = x; by = y; bz = z;
                    }
                }
            }
    if (found && bx < X && by < Y && bz < Z) out[lin(bx, by, bz, X, Y)] = 1;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

struct CandWs {
    int32_t *counts;
    int64_t *offsets;
    int64_t *total;
    int8_t *mask2;
    int8_t *mask3;
    int32_t *list;
    int64_t list_cap;
    size_t bytes;
};

static CandWs cand_ws_layout(void *base, int X, int Y, int Z) {
    const BrickGrid g = brick_grid(X, Y, Z);
    const int64_t nk = brick_keys(g);
    const int64_t n = (int64_t)X * Y * Z;
    CandWs w;
    char *p = (char *)base;
    size_t off = 0;
    w.counts = (int32_t *)(p + off); off = align256(off + sizeof(int32_t) * nk);
    w.offsets = (int64_t *)(p + off); off = align256(off + sizeof(int64_t) * nk);
    w.total = (int64_t *)(p + off); off = align256(off + sizeof(int64_t) * 2);
    w.mask2 = (int8_t *)(p + off); off = align256(off + (size_t)n);
    w.mask3 = (int8_t *)(p + off); off = align256(off + (size_t)n);
    w.list_cap = n / 2 + 1;
    w.list = (int32_t *)(p + off); off = align256(off + sizeof(int32_t) * 3 * (size_t)w.list_cap);
    w.bytes = off;
    return w;
}

size_t candidates_workspace_size(int X, int Y, int Z) { return cand_ws_layout(nullptr, X, Y, Z).bytes; }

size_t compact_workspace_size(int X, int Y, int Z) {
    const int64_t nk = brick_keys(brick_grid(X, Y, Z));
    return align256(sizeof(int32_t) * nk) + align256(sizeof(int64_t) * nk) + align256(sizeof(int64_t) * 2);
}

// count + scan + (optional) write; returns the number of selected voxels in *count.
static int compact(int mode, const void *src, float thr, int X, int Y, int Z, int32_t *counts, int64_t *offsets,
                   int64_t *d_total, int32_t *pos, int64_t cap, int64_t *count, cudaStream_t s) {
    const BrickGrid g = brick_grid(X, Y, Z);
    const int64_t nk = brick_keys(g);
    if (nk > 0x7fffffffLL) return fail(TSF_ERR_INVALID_ARG, "volume too large for compaction");
    const unsigned blocks = (unsigned)nk;
    switch (mode) {
    case FLAG_TDF_F32: brick_count_kernel<FLAG_TDF_F32><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, counts); break;
    case FLAG_TDF_U16: brick_count_kernel<FLAG_TDF_U16><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, counts); break;
    default: brick_count_kernel<FLAG_MASK><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, counts); break;
    }
    TSF_CHECK_LAUNCH("brick_count_kernel");
    scan_counts_kernel<<<1, 1024, 0, s>>>(counts, nk, offsets, d_total);
    TSF_CHECK_LAUNCH("scan_counts_kernel");
    int64_t total = 0;
    TSF_TRY_CUDA(cudaMemcpyAsync(&total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TSF_TRY_CUDA(cudaStreamSynchronize(s));
    *count = total;
    if (pos && total > 0 && cap > 0) {
        switch (mode) {
        case FLAG_TDF_F32: brick_write_kernel<FLAG_TDF_F32><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, offsets, pos, cap); break;
        case FLAG_TDF_U16: brick_write_kernel<FLAG_TDF_U16><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, offsets, pos, cap); break;
        default: brick_write_kernel<FLAG_MASK><<<blocks, 512, 0, s>>>(src, thr, X, Y, Z, g, offsets, pos, cap); break;
        }
        TSF_CHECK_LAUNCH("brick_write_kernel");
    }
    return TSF_OK;
}

int run_compact_mask(const int8_t *mask, int X, int Y, int Z, int32_t *pos, int64_t cap, int64_t *count, void *ws,
                     size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!mask || !count) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!ws || ws_bytes < compact_workspace_size(X, Y, Z)) return fail(TSF_ERR_WORKSPACE, "compaction workspace too small");
    const BrickGrid g = brick_grid(X, Y, Z);
    const int64_t nk = brick_keys(g);
    char *p = (char *)ws;
    int32_t *counts = (int32_t *)p;
    int64_t *offsets = (int64_t *)(p + align256(sizeof(int32_t) * nk));
    int64_t *tot = (int64_t *)(p + align256(sizeof(int32_t) * nk) + align256(sizeof(int64_t) * nk));
    r = compact(FLAG_MASK, mask, 0.0f, X, Y, Z, counts, offsets, tot, pos, cap, count, s);
    if (r) return r;
    if (pos && *count > cap) return fail(TSF_ERR_CAPACITY, "position buffer too small");
    return TSF_OK;
}

// smallest float strictly above cos(0.5): acos(d) < 0.5 <=> d >= this (d <= 1)
static float cos_half_limit() {
    float c = (float)cos(0.5);
    if ((double)c <= cos(0.5)) c = nextafterf(c, 2.0f);
    return c;
}

int run_candidates(const void *T, int unorm, const float *R, const void *F, int st, int X, int Y, int Z,
                   float tdf_high, int cube_size, int32_t *vertices, int64_t max_vertices, int8_t *centerpoints,
                   int32_t *cand_out, int64_t max_cand, int64_t *n_cand, int64_t *n_vert, void *ws, size_t ws_bytes,
                   cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!T || !R || !F || !n_cand || !n_vert) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (cube_size < 1) return fail(TSF_ERR_INVALID_ARG, "cube-size must be >= 1");
    const CandWs w = cand_ws_layout(ws, X, Y, Z);
    if (!ws || ws_bytes < w.bytes) return fail(TSF_ERR_WORKSPACE, "candidate workspace too small");
    const int64_t n = (int64_t)X * Y * Z;
    *n_cand = 0;
    *n_vert = 0;

    // C1 + C2: threshold and compaction in pyramid order
    int64_t cnt = 0;
    int32_t *list = w.list;
    int64_t cap = w.list_cap;
    r = compact(unorm ? FLAG_TDF_U16 : FLAG_TDF_F32, T, tdf_high, X, Y, Z, w.counts, w.offsets, w.total, list, cap,
                &cnt, s);
    if (r) return r;
    *n_cand = cnt;
    if (cnt <= 0 || (double)cnt > 0.5 * (double)n)
        return fail(TSF_ERR_COUNT_RANGE,
                    "The number of candidate voxels is too low or too high. Something went wrong... Wrong parameters?");
    if (cand_out && max_cand > 0) {
        const int64_t k = cnt < max_cand ? cnt : max_cand;
        TSF_TRY_CUDA(cudaMemcpyAsync(cand_out, list, sizeof(int32_t) * 3 * (size_t)k, cudaMemcpyDeviceToDevice, s));
    }

    // C3: cross-section filter, one warp per candidate
    TSF_TRY_CUDA(cudaMemsetAsync(w.mask2, 0, (size_t)n, s));
    {
        const int threads = 256;
        const int64_t blocks64 = (cnt * 32 + threads - 1) / threads;
        if (blocks64 > 0x7fffffffLL) return fail(TSF_ERR_INVALID_ARG, "too many candidates");
        const float cl = cos_half_limit();
        TSF_DISPATCH_STORAGE(st, ST,
            candidates2_kernel<ST><<<(unsigned)blocks64, threads, 0, s>>>(R, F, X, Y, Z, list, cnt, cl, w.mask2));
        TSF_CHECK_LAUNCH("candidates2_kernel");
    }
    if (centerpoints) TSF_TRY_CUDA(cudaMemcpyAsync(centerpoints, w.mask2, (size_t)n, cudaMemcpyDeviceToDevice, s));

    // C4: per-cube arg-max
    TSF_TRY_CUDA(cudaMemsetAsync(w.mask3, 0, (size_t)n, s));
    {
        const int GX = (X + cube_size - 1) / cube_size, GY = (Y + cube_size - 1) / cube_size,
                  GZ = (Z + cube_size - 1) / cube_size;
        const int64_t cubes = (int64_t)GX * GY * GZ;
        const unsigned blocks = (unsigned)((cubes + 127) / 128);
        if (unorm) dd_kernel<true><<<blocks, 128, 0, s>>>(T, w.mask2, X, Y, Z, cube_size, GX, GY, GZ, w.mask3);
        else dd_kernel<false><<<blocks, 128, 0, s>>>(T, w.mask2, X, Y, Z, cube_size, GX, GY, GZ, w.mask3);
        TSF_CHECK_LAUNCH("dd_kernel");
    }

    // second compaction: the vertex list
    int64_t nv = 0;
    r = compact(FLAG_MASK, w.mask3, 0.0f, X, Y, Z, w.counts, w.offsets, w.total, vertices, max_vertices, &nv, s);
    if (r) return r;
    *n_vert = nv;
    if (nv < 8) return fail(TSF_ERR_COUNT_RANGE, "Too few centerpoints detected. Revise parameters.");
    if (nv >= 16384)
        return fail(TSF_ERR_COUNT_RANGE, "Too many centerpoints detected. More cropping of dataset is probably needed.");
    if (vertices && nv > max_vertices) return fail(TSF_ERR_CAPACITY, "vertex buffer too small");
    return TSF_OK;
}

}  // namespace tsf
