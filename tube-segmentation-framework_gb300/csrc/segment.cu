// segment.cu -- segmentation from the centerlines: inverse-gradient region
// growing (runInverseGradientSegmentation, segmentation.cpp:5-205; kernels
// initGrowing, grow, dilate, erode) and sphere segmentation
// (runSphereSegmentation, segmentation.cpp:207-307; kernel
// sphereSegmentation).  The kernels follow the buffer variants the reference
// compiles on devices without 3-D image writes, NVIDIA's included
// (kernels_no_3d_write.cl:1100-1235, 1370-1412; tube-segmentation.cpp:88-111):
// writes outside the volume are dropped, reads clamp to the edge.
//
// Growing.  State per voxel: 1 accepted, 2 to check, 0 neither.  The start is
// the centerline (1) with every non-centerline voxel within
// N = min(max(1, round(r/2)), 4) of a centerline voxel set to 2 (r its
// radius).  An iteration checks every voxel X at 2: for each neighbour Y of
// its 26 with state != 1 and |v(Y)| > |v(X)|, the direction among Y's 26
// neighbours that best matches v(Y)/|v(Y)| (largest dot product, first in
// x, y, z loop order) is found; if it points back at X and Y lies inside the
// volume, X is accepted and Y is set to 2.  X at 2 that accepts nothing drops
// to 0.  The reference lets these writes race within an iteration (a voxel's
// own thread writes 1 or 0 while an accepting neighbour writes 2), so its
// result depends on thread order; here an iteration first decides (which X
// accept, which Y they mark) and then applies with the precedence accepted >
// to check > dropped.  Iterations stop when nothing is accepted.  The grown
// mask (state 1) is then closed: dilated by the 3x3x3 cube, then eroded by it.
#include <algorithm>
#include <cmath>

#include "tsf_common.cuh"

namespace tsf {

// the 26 unit directions (a, b, c) / |(a, b, c)| in the reference's loop order
struct Dirs26 {
    float d[26][3];
    int o[26][3];
};

static Dirs26 host_dirs26() {
    Dirs26 t;
    int k = 0;
    for (int a = -1; a < 2; a++)
        for (int b = -1; b < 2; b++)
            for (int c = -1; c < 2; c++) {
                if (a == 0 && b == 0 && c == 0) continue;
                const float l = std::sqrt((float)(a * a + b * b + c * c));
                t.d[k][0] = (float)a / l;
                t.d[k][1] = (float)b / l;
                t.d[k][2] = (float)c / l;
                t.o[k][0] = a;
                t.o[k][1] = b;
                t.o[k][2] = c;
                k++;
            }
    return t;
}

#define SEG_XYZ(X, Y, Z)                                            \
    const int x = blockIdx.x * blockDim.x + threadIdx.x;            \
    const int y = blockIdx.y * blockDim.y + threadIdx.y;            \
    const int z = blockIdx.z * blockDim.z + threadIdx.z;            \
    if (x >= (X) || y >= (Y) || z >= (Z)) return;

// initGrowing: state = centerline, then 2 around every centerline voxel
__global__ void seg_init_kernel(const int8_t *__restrict__ cl, const float *__restrict__ radius, int8_t *state,
                                int X, int Y, int Z) {
    SEG_XYZ(X, Y, Z);
    const int64_t i = lin(x, y, z, X, Y);
    if (cl[i] != 1) return;
    const int N = min(max(1, (int)roundf(radius[i] / 2.0f)), 4);
    for (int a = -N; a <= N; a++)
        for (int b = -N; b <= N; b++)
            for (int c = -N; c <= N; c++) {
                const int nx = x + a, ny = y + b, nz = z + c;
                if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z) continue;
                const int64_t j = lin(nx, ny, nz, X, Y);
                if (cl[j] == 0) state[j] = 2;
            }
}

// The voxels at 2 form the front, kept as a list of linear indices so that an
// iteration costs the front, not the volume.  Front entries are unique: the
// initial list is a compaction of the state, and a voxel enters the next list
// only with the first mark it receives (an atomic OR on the mark byte's word).

// Warp-aggregated append of index i (when `take`) to list / *cnt.
__device__ __forceinline__ void seg_append(bool take, int64_t i, int64_t *list, unsigned long long *cnt) {
    const unsigned full = 0xffffffffu;
    const unsigned m = __ballot_sync(full, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(cnt, (unsigned long long)__popc(m));
    base = __shfl_sync(full, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// the initial front: every voxel at 2, in any order
__global__ void seg_front_init_kernel(const int8_t *__restrict__ state, int64_t n, int64_t *__restrict__ front,
                                      unsigned long long *__restrict__ cnt) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // whole warps stay in the loop so that the ballots see every lane
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x; b < n; b += stride) {
        const int64_t i = b + threadIdx.x;
        seg_append(i < n && state[i] == 2, i, front, cnt);
    }
}

// grow, deciding half, one warp per front voxel X, lane k < 26 its neighbour
// k: acc[X] = 1 if X accepts; each marked neighbour Y gets mark[Y] = 1 and,
// on its first mark, a place in the next front; *any = 1 if anything was
// accepted.  Decisions read only the iteration's starting state, so the order
// of the list changes nothing.
template <int ST>
__global__ void seg_front_decide_kernel(const int8_t *__restrict__ state, const void *__restrict__ F,
                                        const Dirs26 dirs, int8_t *__restrict__ acc, int8_t *mark,
                                        const int64_t *__restrict__ front, const unsigned long long *__restrict__ nfront,
                                        int64_t *__restrict__ next, unsigned long long *__restrict__ nnext,
                                        int *__restrict__ any, int X, int Y, int Z) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nf = (int64_t)*nfront;
    const int64_t plane = (int64_t)X * Y;
    for (int64_t f = (((int64_t)blockIdx.x * blockDim.x) + threadIdx.x) >> 5; f < nf; f += warps) {
        const int64_t i = front[f];
        if (state[i] != 2) continue;                       // warp-uniform
        const int z = (int)(i / plane), y = (int)((i - (int64_t)z * plane) / X), x = (int)(i - (int64_t)z * plane - (int64_t)y * X);
        const float wx = Vec4Load<ST>::load(F, i).w;
        bool grew = false, marked_first = false;
        int64_t yj = 0;
        if (lane < 26) {
            const int k = lane;
            const int yx = x + dirs.o[k][0], yy = y + dirs.o[k][1], yz = z + dirs.o[k][2];
            const int64_t j = lin(clampi(yx, X), clampi(yy, Y), clampi(yz, Z), X, Y);
            if (state[j] != 1) {
                float4 fy = Vec4Load<ST>::load(F, j);
                fy.x /= fy.w;
                fy.y /= fy.w;
                fy.z /= fy.w;
                if (fy.w > wx) {
                    float best = -2.0f;
                    int bk = 0;
                    for (int m = 0; m < 26; m++) {
                        const float v = (fy.x * dirs.d[m][0] + fy.y * dirs.d[m][1]) + fy.z * dirs.d[m][2];
                        if (v > best) {
                            best = v;
                            bk = m;
                        }
                    }
                    // Z = Y + o[bk] is X  <=>  o[bk] = -o[k]; accepted only through Y inside
                    if (bk == 25 - k && yx >= 0 && yy >= 0 && yz >= 0 && yx < X && yy < Y && yz < Z) {
                        grew = true;
                        yj = lin(yx, yy, yz, X, Y);
                        unsigned *word = reinterpret_cast<unsigned *>(mark + (yj & ~(int64_t)3));
                        const unsigned bit = 1u << (8 * (int)(yj & 3));
                        marked_first = (atomicOr(word, bit) & bit) == 0;
                    }
                }
            }
        }
        seg_append(marked_first, yj, next, nnext);
        if (__ballot_sync(full, grew) && lane == 0) {
            acc[i] = 1;
            *any = 1;
        }
    }
}

// grow, applying half 1: the front's own verdicts (accepted -> 1, else 0)
__global__ void seg_front_apply_kernel(int8_t *__restrict__ state, int8_t *__restrict__ acc,
                                       const int64_t *__restrict__ front, const unsigned long long *__restrict__ nfront) {
    const int64_t nf = (int64_t)*nfront;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = front[f];
        if (state[i] != 2) continue;
        state[i] = acc[i] ? 1 : 0;
        acc[i] = 0;
    }
}

// grow, applying half 2: the marked voxels go to 2 unless accepted (the
// precedence accepted > to check > dropped); their list is the next front.
// Clears the marks, and the count of the front just applied (that list holds
// the next iteration's marks).
__global__ void seg_mark_apply_kernel(int8_t *__restrict__ state, int8_t *mark, const int64_t *__restrict__ next,
                                      const unsigned long long *__restrict__ nnext,
                                      unsigned long long *__restrict__ nfront) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *nfront = 0;
    const int64_t nn = (int64_t)*nnext;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nn; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = next[g];
        mark[j] = 0;
        if (state[j] != 1) state[j] = 2;
    }
}

// dilate: out (zeroed) = 1 on the 3x3x3 neighbourhood of every voxel at 1
__global__ void seg_dilate_kernel(const int8_t *__restrict__ in, int8_t *__restrict__ out, int X, int Y, int Z) {
    SEG_XYZ(X, Y, Z);
    if (in[lin(x, y, z, X, Y)] != 1) return;
    for (int a = -1; a < 2; a++)
        for (int b = -1; b < 2; b++)
            for (int c = -1; c < 2; c++) {
                const int nx = x + a, ny = y + b, nz = z + c;
                if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z) continue;
                out[lin(nx, ny, nz, X, Y)] = 1;
            }
}

// erode: 1 where the voxel and its 26 neighbours (clamped to the edge) are 1
__global__ void seg_erode_kernel(const int8_t *__restrict__ in, int8_t *__restrict__ out, int X, int Y, int Z) {
    SEG_XYZ(X, Y, Z);
    const int64_t i = lin(x, y, z, X, Y);
    bool keep = in[i] == 1;
    for (int a = -1; a < 2 && keep; a++)
        for (int b = -1; b < 2 && keep; b++)
            for (int c = -1; c < 2 && keep; c++)
                keep = in[lin(clampi(x + a, X), clampi(y + b, Y), clampi(z + c, Z), X, Y)] == 1;
    out[i] = keep ? 1 : 0;
}

// sphereSegmentation: 1 within distance < r of every centerline voxel
__global__ void seg_sphere_kernel(const int8_t *__restrict__ cl, const float *__restrict__ radius,
                                  int8_t *__restrict__ out, int X, int Y, int Z) {
    SEG_XYZ(X, Y, Z);
    const int64_t i = lin(x, y, z, X, Y);
    if (cl[i] == 0) return;
    const float r = radius[i];
    if (!(r > 0.0f)) return;   // no offset has length < r (r <= 0 or NaN)
    // offsets beyond the largest extent leave the volume: bounding the loop
    // there changes nothing and keeps a huge radius finite
    const int N = (int)ceilf(fminf(r, (float)max(X, max(Y, Z))));
    for (int a = -N; a <= N; a++)
        for (int b = -N; b <= N; b++)
            for (int c = -N; c <= N; c++) {
                const float l = sqrtf((float)(a * a) + (float)(b * b) + (float)(c * c));
                if (!(l < r)) continue;
                const int nx = x + a, ny = y + b, nz = z + c;
                if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z) continue;
                out[lin(nx, ny, nz, X, Y)] = 1;
            }
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Grow iterations launched between two reads of the accept flags.  An
// iteration that accepts nothing leaves no voxel at 2, so the iterations after
// it in the same batch change nothing.
constexpr int kGrowBatch = 8;

size_t segment_workspace_size(int X, int Y, int Z) {
    const size_t n = (size_t)X * Y * Z;
    // state, acc, mark (int8); two front lists (int64); two counts; the batch's accept flags
    return 3 * al256(n) + 2 * al256(n * sizeof(int64_t)) + 256 + al256(kGrowBatch * sizeof(int));
}

static dim3 seg_block() { return dim3(32, 4, 2); }
static dim3 seg_grid(int X, int Y, int Z) { return dim3((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2); }

int run_segment_inverse_gradient(const int8_t *cl, const void *F, int st, const float *radius, int X, int Y, int Z,
                                 int8_t *out, int *iterations, void *ws, size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!cl || !F || !radius || !out) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!ws || ws_bytes < segment_workspace_size(X, Y, Z))
        return fail(TSF_ERR_WORKSPACE, "segmentation workspace too small");
    if ((reinterpret_cast<uintptr_t>(ws) & 7) != 0) return fail(TSF_ERR_INVALID_ARG, "workspace must be 8-byte aligned");
    const int64_t n = (int64_t)X * Y * Z;
    char *w = (char *)ws;
    int8_t *state = (int8_t *)w, *acc = (int8_t *)(w + al256(n)), *mark = (int8_t *)(w + 2 * al256(n));
    int64_t *lists[2] = {(int64_t *)(w + 3 * al256(n)),
                         (int64_t *)(w + 3 * al256(n) + al256(n * sizeof(int64_t)))};
    unsigned long long *cnt = (unsigned long long *)(w + 3 * al256(n) + 2 * al256(n * sizeof(int64_t)));
    int *flags = (int *)((char *)cnt + 256);
    const Dirs26 dirs = host_dirs26();
    TSF_TRY_CUDA(cudaMemcpyAsync(state, cl, (size_t)n, cudaMemcpyDeviceToDevice, s));
    TSF_TRY_CUDA(cudaMemsetAsync(acc, 0, 2 * al256(n), s));
    TSF_TRY_CUDA(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), s));
    seg_init_kernel<<<seg_grid(X, Y, Z), seg_block(), 0, s>>>(cl, radius, state, X, Y, Z);
    const unsigned gblocks = 8 * 152;
    seg_front_init_kernel<<<gblocks, 256, 0, s>>>(state, n, lists[0], cnt);
    TSF_CHECK_LAUNCHES("seg_init/front_init", 2);
    int p = 0;                                            // lists[p] holds the front
    int64_t it = 0;
    for (;;) {
        TSF_TRY_CUDA(cudaMemsetAsync(flags, 0, kGrowBatch * sizeof(int), s));
        for (int b = 0; b < kGrowBatch; b++) {
            TSF_DISPATCH_STORAGE(st, ST, {
                seg_front_decide_kernel<ST><<<gblocks, 256, 0, s>>>(state, F, dirs, acc, mark, lists[p], cnt + p,
                                                                    lists[1 - p], cnt + (1 - p), flags + b, X, Y, Z);
            });
            seg_front_apply_kernel<<<gblocks, 256, 0, s>>>(state, acc, lists[p], cnt + p);
            seg_mark_apply_kernel<<<gblocks, 256, 0, s>>>(state, mark, lists[1 - p], cnt + (1 - p), cnt + p);
            TSF_CHECK_LAUNCHES("seg_decide/apply", 3);
            p = 1 - p;
        }
        int h[kGrowBatch];
        TSF_TRY_CUDA(cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, s));
        TSF_TRY_CUDA(cudaStreamSynchronize(s));
        int b = 0;
        while (b < kGrowBatch && h[b]) b++;
        if (b < kGrowBatch) {
            it += b + 1;
            break;
        }
        it += kGrowBatch;
        // every productive iteration accepts at least one more voxel
        if (it > n + 1) return fail(TSF_ERR_NOT_CONVERGED, "segmentation growing did not settle");
    }
    if (iterations) *iterations = (int)std::min<int64_t>(it, INT32_MAX);
    // close the grown mask: dilate into acc (zeroed), erode into out
    TSF_TRY_CUDA(cudaMemsetAsync(acc, 0, (size_t)n, s));
    seg_dilate_kernel<<<seg_grid(X, Y, Z), seg_block(), 0, s>>>(state, acc, X, Y, Z);
    seg_erode_kernel<<<seg_grid(X, Y, Z), seg_block(), 0, s>>>(acc, out, X, Y, Z);
    TSF_CHECK_LAUNCHES("seg_dilate/erode", 2);
    return TSF_OK;
}

int run_segment_spheres(const int8_t *cl, const float *radius, int X, int Y, int Z, int8_t *out, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!cl || !radius || !out) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    TSF_TRY_CUDA(cudaMemsetAsync(out, 0, (size_t)X * Y * Z, s));
    seg_sphere_kernel<<<seg_grid(X, Y, Z), seg_block(), 0, s>>>(cl, radius, out, X, Y, Z);
    TSF_CHECK_LAUNCH("seg_sphere_kernel");
    return TSF_OK;
}

}  // namespace tsf

extern "C" size_t tsf_segment_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return tsf::segment_workspace_size(X, Y, Z);
}

extern "C" int tsf_segment_inverse_gradient(const int8_t *d_centerlines, const void *d_field4, int storage,
                                            const float *d_radius, int X, int Y, int Z, int8_t *d_segmentation,
                                            int *iterations, void *d_workspace, size_t workspace_bytes,
                                            void *stream) {
    return tsf::run_segment_inverse_gradient(d_centerlines, d_field4, storage, d_radius, X, Y, Z, d_segmentation,
                                             iterations, d_workspace, workspace_bytes,
                                             reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_segment_spheres(const int8_t *d_centerlines, const float *d_radius, int X, int Y, int Z,
                                   int8_t *d_segmentation, void *stream) {
    return tsf::run_segment_spheres(d_centerlines, d_radius, X, Y, Z, d_segmentation,
                                    reinterpret_cast<cudaStream_t>(stream));
}
