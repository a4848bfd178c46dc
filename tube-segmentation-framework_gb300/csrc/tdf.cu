// tdf.cu -- the circle-fitting tube detection filter fused with the Hessian
// and its eigen-decomposition (reference circleFittingTDF, kernels.cl:1065-1157;
// driver runCircleFittingTDF, tubeDetectionFilters.cpp:57-73; combine,
// kernels.cl:561-572).
//
// One thread per voxel.  The thread reads the six face neighbours of the
// field4 image (one 16 B or 8 B vector load each), builds the Hessian,
// decomposes it in registers (eigen3.cuh), then sweeps the radii: per radius
// 32 points on the circle spanned by e2 and e3, each a trilinear read of the
// x,y,z channels with OpenCL's unnormalised-coordinate convention
// (i0 = floor(u - 0.5), clamp to edge).  The sweep stops at the first radius
// that does not raise the mean response.  Algorithmic HBM traffic is the
// field read once (4s B/voxel) plus T and R written (8 B or 6 B/voxel); the
// trilinear gathers are served by L1/L2.
#include "tdf_common.cuh"

namespace tsf {

// Upper bound on the number of radii one voxel evaluates (a radius step of 0
// would otherwise repeat the same radius until the response stops growing).
constexpr int kMaxRadii = 4096;

template <int ST, bool NORM, bool UNORM>
__global__ void __launch_bounds__(256) tdf_circle_kernel(const void *__restrict__ F, int X, int Y, int Z, float rmin,
                                                         float rmax, float rstep, const CircleTable tab, void *T,
                                                         float *__restrict__ Rout) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    float H[3][3], V[3][3], d[3];
    hessian<ST, NORM>(F, X, Y, Z, x, y, z, H);
    eig3<float>(H, V, d);
    const float e2x = V[0][1], e2y = V[1][1], e2z = V[2][1];
    const float e3x = V[0][2], e3y = V[1][2], e3z = V[2][2];
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    float maxSum = 0.0f, maxRadius = 0.0f;
    int nr = 0;
    for (float radius = rmin; radius <= rmax && nr < kMaxRadii; radius = radius + rstep, nr++) {
        float rs = 0.0f;
#pragma unroll 4
        for (int j = 0; j < 32; j++) {
            const float c = tab.c[j], s = tab.s[j];
            const float va0 = c * e3x + s * e2x;
            const float va1 = c * e3y + s * e2y;
            const float va2 = c * e3z + s * e2z;
            const float3 smp = sample_linear<ST>(F, X, Y, Z, fx + radius * va0, fy + radius * va1, fz + radius * va2);
            const float dt = ((-smp.x) * va0 + (-smp.y) * va1) + (-smp.z) * va2;
            rs = rs + dt;
        }
        rs = rs / 32.0f;
        if (rs > maxSum) {
            maxSum = rs;
            maxRadius = radius;
        } else {
            break;
        }
    }
    const int64_t i = lin(x, y, z, X, Y);
    if (UNORM) {
        reinterpret_cast<uint16_t *>(T)[i] = to_unorm16(maxSum);
    } else {
        reinterpret_cast<float *>(T)[i] = maxSum;
    }
    Rout[i] = maxRadius;
}

// Same filter with the radius sweeps load-balanced inside each warp.
//
// With one voxel per lane, a warp runs as many radii as its slowest voxel
// needs (about half the voxels stop at the first radius, others go on to 3-6),
// which left ~60 % of the lanes idle.  Here a warp owns kSeg = 128 voxels: it
// first decomposes all their Hessians (one voxel per lane, 4 rounds) into
// shared memory, then treats each voxel's sweep as a task: a lane evaluates
// one radius (its 32 samples, in order) per round and, when its voxel's sweep
// ends, takes the next unstarted voxel, in lane order.  Lanes stay busy until
// the queue drains, and each voxel's arithmetic is exactly that of
// tdf_circle_kernel.
//
// Locality: a warp's voxels form an 8 x 4 x 4 block and a CTA's four warps an
// 8 x 8 x 8 brick, so the circles sampled by a CTA stay within a
// (8 + 2 rmax)^3 neighbourhood that L1 can hold (row segments of 128 voxels
// touched ~5x more distinct lines and missed L1 for about a quarter of the
// trilinear corners).
constexpr int kSeg = 128;
constexpr int kTdfWarps = 4;

// PAIR: interior samples read the x-paired copy P of a 16-bit field (one
// 16-byte load per corner row, sample_linear_pair_in) instead of F.
template <int ST, bool NORM, bool UNORM, bool PAIR>
__global__ void __launch_bounds__(32 * kTdfWarps) tdf_queue_kernel(const void *__restrict__ F, int X, int Y, int Z,
                                                                    float rmin, float rmax, float rstep,
                                                                    const CircleTable tab, void *T,
                                                                    float *__restrict__ Rout, int fast_ok,
                                                                    const uint4 *__restrict__ P) {
    static_assert(kTdfWarps == 4 && kSeg == 128, "a CTA is an 8x8x8 brick of four 8x4x4 warp blocks");
    __shared__ float se[kTdfWarps][6][kSeg];
    __shared__ unsigned char sin_[kTdfWarps][kSeg];      // samples stay inside: unclamped sampler
    const int XY = X * Y, margin = sample_margin(rmax);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // brick of this CTA, block of this warp: task t -> (t & 7, (t >> 3) & 3, t >> 5)
    const int nbx = (X + 7) >> 3, nby = (Y + 7) >> 3;
    const int b = blockIdx.x;
    const int bx0 = (b % nbx) * 8, by0 = ((b / nbx) % nby) * 8 + (w & 1) * 4;
    const int bz0 = (b / (nbx * nby)) * 8 + (w >> 1) * 4;
    const int ntask = kSeg;
    auto tx = [&](int t) { return bx0 + (t & 7); };
    auto ty = [&](int t) { return by0 + ((t >> 3) & 3); };
    auto tz = [&](int t) { return bz0 + (t >> 5); };
    auto inside = [&](int t) { return tx(t) < X && ty(t) < Y && tz(t) < Z; };
    // phase 1: eigenvectors of the block's voxels
    for (int t = lane; t < ntask; t += 32) {
        if (!inside(t)) continue;
        float H[3][3], V[3][3], d[3];
        hessian<ST, NORM>(F, X, Y, Z, tx(t), ty(t), tz(t), H);
        eig3<float>(H, V, d);
        se[w][0][t] = V[0][1]; se[w][1][t] = V[1][1]; se[w][2][t] = V[2][1];
        se[w][3][t] = V[0][2]; se[w][4][t] = V[1][2]; se[w][5][t] = V[2][2];
        const float e2[3] = {V[0][1], V[1][1], V[2][1]}, e3[3] = {V[0][2], V[1][2], V[2][2]};
        sin_[w][t] = fast_ok && samples_inside(tx(t), ty(t), tz(t), X, Y, Z, margin, e2, e3);
    }
    __syncwarp();
    // phase 2: radius sweeps as tasks
    const unsigned full = 0xffffffffu;
    int task = lane < ntask ? lane : -1;
    int next = 32;                                   // next unstarted task (same in every lane)
    float radius = rmin, maxSum = 0.0f, maxRadius = 0.0f;
    int nr = 0;
    while (__any_sync(full, task >= 0)) {
        bool done = true;
        if (task >= 0 && inside(task)) {
            const float e2x = se[w][0][task], e2y = se[w][1][task], e2z = se[w][2][task];
            const float e3x = se[w][3][task], e3y = se[w][4][task], e3z = se[w][5][task];
            const float fx = (float)tx(task), fy = (float)ty(task), fz = (float)tz(task);
            if (radius <= rmax && nr < kMaxRadii) {
                float rs = 0.0f;
                if (sin_[w][task]) {
#pragma unroll 4
                    for (int j = 0; j < 32; j++) {
                        const float c = tab.c[j], s = tab.s[j];
                        const float va0 = c * e3x + s * e2x;
                        const float va1 = c * e3y + s * e2y;
                        const float va2 = c * e3z + s * e2z;
                        float3 smp;
                        if constexpr (PAIR)
                            smp = sample_linear_pair_in<ST>(P, X, XY, fx + radius * va0, fy + radius * va1,
                                                            fz + radius * va2);
                        else
                            smp = sample_linear_in<ST>(F, X, XY, fx + radius * va0, fy + radius * va1,
                                                       fz + radius * va2);
                        const float dt = ((-smp.x) * va0 + (-smp.y) * va1) + (-smp.z) * va2;
                        rs = rs + dt;
                    }
                } else {
#pragma unroll 4
                    for (int j = 0; j < 32; j++) {
                        const float c = tab.c[j], s = tab.s[j];
                        const float va0 = c * e3x + s * e2x;
                        const float va1 = c * e3y + s * e2y;
                        const float va2 = c * e3z + s * e2z;
                        const float3 smp =
                            sample_linear<ST>(F, X, Y, Z, fx + radius * va0, fy + radius * va1, fz + radius * va2);
                        const float dt = ((-smp.x) * va0 + (-smp.y) * va1) + (-smp.z) * va2;
                        rs = rs + dt;
                    }
                }
                rs = rs / 32.0f;
                if (rs > maxSum) {
                    maxSum = rs;
                    maxRadius = radius;
                    radius = radius + rstep;
                    nr++;
                    done = false;
                }
            }
            if (done) {
                const int64_t i = lin(tx(task), ty(task), tz(task), X, Y);
                if (UNORM) reinterpret_cast<uint16_t *>(T)[i] = to_unorm16(maxSum);
                else reinterpret_cast<float *>(T)[i] = maxSum;
                Rout[i] = maxRadius;
            }
        }
        // lanes whose sweep ended take the next tasks, in lane order
        const unsigned want = __ballot_sync(full, task >= 0 && done) | __ballot_sync(full, task < 0 && next < ntask);
        if ((want >> lane) & 1u) {
            const int k = next + __popc(want & ((1u << lane) - 1u));
            task = k < ntask ? k : -1;
            radius = rmin;
            maxSum = 0.0f;
            maxRadius = 0.0f;
            nr = 0;
        }
        next += __popc(want);
    }
}

// The x-paired copy of a 16-bit field4 image: P[i] = (texel i, texel of the
// next x, clamped at the last column), 16 bytes per voxel.
__global__ void tdf_pair_kernel(const uint2 *__restrict__ F, uint4 *__restrict__ P, int X, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % X);
    const uint2 a = __ldg(F + i), b = __ldg(F + i + (x + 1 < X ? 1 : 0));
    P[i] = make_uint4(a.x, a.y, b.x, b.y);
}

size_t tdf_workspace_size(int X, int Y, int Z, int st) {
    if (X <= 0 || Y <= 0 || Z <= 0 || !valid_storage(st) || st == TSF_STORE_F32) return 0;
    return (size_t)X * Y * Z * sizeof(uint4);
}

template <bool UNORM>
__global__ void combine_kernel(const void *__restrict__ Ts, const float *__restrict__ Rs, void *Tl, float *Rl, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (UNORM) {
        const uint16_t s = reinterpret_cast<const uint16_t *>(Ts)[i];
        uint16_t *L = reinterpret_cast<uint16_t *>(Tl);
        if (L[i] < s) { L[i] = s; Rl[i] = Rs[i]; }
    } else {
        const float s = reinterpret_cast<const float *>(Ts)[i];
        float *L = reinterpret_cast<float *>(Tl);
        if (L[i] < s) { L[i] = s; Rl[i] = Rs[i]; }
    }
}

// tdf_mode: 0 = default (load-balanced sweeps), 1 = one voxel per lane.
// ws / ws_bytes: room for the x-paired copy of a 16-bit field (tdf_workspace_size);
// without it, or for FP32 storage, the samples read the field itself.
int launch_tdf_circle(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                      void *d_T, int unorm, float *d_R, cudaStream_t s, int tdf_mode, void *ws, size_t ws_bytes) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_field4 || !d_T || !d_R) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!(rstep >= 0.0f) || !(rmin >= 0.0f)) return fail(TSF_ERR_INVALID_ARG, "invalid radius range");
    const CircleTable tab = host_circle_table();
    const dim3 b(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    const bool norm = !(rmax < 4.0f);   // kernels.cl:1083-1091
    const unsigned qblocks = (unsigned)(((X + 7) / 8) * ((Y + 7) / 8) * ((Z + 7) / 8));   // 8^3 bricks
    const bool queue = tdf_mode != 1;
    const int fast_ok = (int64_t)X * Y * Z < ((int64_t)1 << 31) - 1;   // 32-bit texel offsets
    const int64_t n = (int64_t)X * Y * Z;
    const size_t need = tdf_workspace_size(X, Y, Z, st);
    const bool pair = queue && fast_ok && need > 0 && ws && ws_bytes >= need &&
                      (reinterpret_cast<uintptr_t>(ws) & 15) == 0 && (reinterpret_cast<uintptr_t>(d_field4) & 7) == 0;
    uint4 *P = pair ? static_cast<uint4 *>(ws) : nullptr;
    if (pair) {
        tdf_pair_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const uint2 *>(d_field4), P, X, n);
        TSF_CHECK_LAUNCH("tdf_pair_kernel");
    }
#define TSF_TDF_LAUNCH(ST, NORM, UN)                                                                                 \
    do {                                                                                                             \
        if (queue && pair)                                                                                           \
            tdf_queue_kernel<ST, NORM, UN, ST != TSF_STORE_F32><<<qblocks, 32 * kTdfWarps, 0, s>>>(                 \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, P);                                    \
        else if (queue)                                                                                              \
            tdf_queue_kernel<ST, NORM, UN, false><<<qblocks, 32 * kTdfWarps, 0, s>>>(                               \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, nullptr);                              \
        else                                                                                                         \
            tdf_circle_kernel<ST, NORM, UN><<<g, b, 0, s>>>(d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R);    \
    } while (0)
    TSF_DISPATCH_STORAGE(st, ST, {
        if (norm) {
            if (unorm) TSF_TDF_LAUNCH(ST, true, true); else TSF_TDF_LAUNCH(ST, true, false);
        } else {
            if (unorm) TSF_TDF_LAUNCH(ST, false, true); else TSF_TDF_LAUNCH(ST, false, false);
        }
    });
#undef TSF_TDF_LAUNCH
    TSF_CHECK_LAUNCH("tdf_circle_kernel");
    return TSF_OK;
}

int launch_tdf_combine(const void *Ts, const float *Rs, void *Tl, float *Rl, int64_t n, int unorm, cudaStream_t s) {
    if (!Ts || !Rs || !Tl || !Rl || n <= 0) return fail(TSF_ERR_INVALID_ARG, "invalid combine arguments");
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if (unorm) combine_kernel<true><<<blocks, threads, 0, s>>>(Ts, Rs, Tl, Rl, n);
    else combine_kernel<false><<<blocks, threads, 0, s>>>(Ts, Rs, Tl, Rl, n);
    TSF_CHECK_LAUNCH("combine_kernel");
    return TSF_OK;
}

}  // namespace tsf
