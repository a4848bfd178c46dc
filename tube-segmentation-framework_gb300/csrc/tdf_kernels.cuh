// tdf_kernels.cuh -- the circle-fitting tube detection filter fused with the
// Hessian and its eigen-decomposition (reference circleFittingTDF,
// kernels.cl:1065-1157; driver runCircleFittingTDF,
// tubeDetectionFilters.cpp:57-73): the kernel templates and their launcher,
// instantiated for the reference's tred2 + tql2 (eigen mode 0, tdf.cu) and for
// the closed-form eigensolver (eigen mode 1, tdf_closed.cu) in separate
// translation units so the two compile in parallel.
//
// One thread per voxel (tdf_circle_kernel) or load-balanced sweeps over
// bricks (tdf_queue_kernel).  The thread reads the six face neighbours of the
// field4 image (one 16 B or 8 B vector load each), builds the Hessian,
// decomposes it in registers, then sweeps the radii: per radius tab.n points
// on the circle spanned by e2 and e3 (32 in the reference, kernels.cl:1122;
// the table holds entries j * stride of the reference's cos / sin table), each
// a trilinear read of the x,y,z channels with OpenCL's
// unnormalised-coordinate convention (i0 = floor(u - 0.5), clamp to edge).
// The sweep stops at the first radius that does not raise the mean response.
// Algorithmic HBM traffic is the field read once (4s B/voxel) plus T and R
// written (8 B or 6 B/voxel); the trilinear gathers are served by L1/L2.
#pragma once

#include "eigen_closed.cuh"
#include "tdf_common.cuh"

namespace tsf {

// Eigenvectors e2, e3 (columns 1, 2) of the Hessian H: the reference's
// tred2 + tql2 (EIG 0) or the closed form (EIG 1).
template <int EIG> __device__ __forceinline__ void tdf_eigen(const float H[3][3], float V[3][3]) {
    float d[3];
    if constexpr (EIG == 0) eig3<float>(H, V, d);
    else eig3_closed(H, V, d);
}

// Upper bound on the number of radii one voxel evaluates (a radius step of 0
// would otherwise repeat the same radius until the response stops growing).
constexpr int kMaxRadii = 4096;

template <int ST, bool NORM, bool UNORM, int EIG>
__global__ void __launch_bounds__(256) tdf_circle_kernel(const void *__restrict__ F, int X, int Y, int Z, float rmin,
                                                         float rmax, float rstep, const CircleTable tab, void *T,
                                                         float *__restrict__ Rout) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    float H[3][3], V[3][3];
    hessian<ST, NORM>(F, X, Y, Z, x, y, z, H);
    tdf_eigen<EIG>(H, V);
    const float e2x = V[0][1], e2y = V[1][1], e2z = V[2][1];
    const float e3x = V[0][2], e3y = V[1][2], e3z = V[2][2];
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    float maxSum = 0.0f, maxRadius = 0.0f;
    int nr = 0;
    for (float radius = rmin; radius <= rmax && nr < kMaxRadii; radius = radius + rstep, nr++) {
        float rs = 0.0f;
#pragma unroll 2
        for (int j = 0; j < tab.n; j++) {
            const float3 va = circle_dir(tab.c[j], tab.s[j], e2x, e2y, e2z, e3x, e3y, e3z);
            const float3 u = circle_point(fx, fy, fz, radius, va);
            const float3 smp = sample_linear<ST>(F, X, Y, Z, u.x, u.y, u.z);
            rs = rs + radial_term(smp, va);
        }
        rs = rs / (float)tab.n;
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
// the queue drains; after that, once few sweeps are left (tdf_tail), the warp
// runs them one voxel at a time with lane j computing sample j and every lane
// summing the 32 staged samples in sample order.  Each voxel's arithmetic is
// exactly that of tdf_circle_kernel.
//
// Locality: a warp's voxels form an 8 x 4 x 4 block and a CTA's four warps an
// 8 x 8 x 8 brick, so the circles sampled by a CTA stay within a
// (8 + 2 rmax)^3 neighbourhood that L1 can hold (row segments of 128 voxels
// touched ~5x more distinct lines and missed L1 for about a quarter of the
// trilinear corners).
constexpr int kSeg = 128;
constexpr int kTdfWarps = 4;
// Sweeps left when the load-balanced kernel switches to one sample per lane,
// as measured at 256^3: 16-bit fields 24 for the large-radius pass
// (normalised Hessian, radii to 7: 8.21 -> 7.93 ms) and 8 for the small-radius
// one (6.37 -> 6.24 ms); FP32 fields 8 for the small pass (9.64 -> 9.47 ms) and
// none for the large one, where the switch cost time (13.57 -> 14.10 ms).
template <int ST, bool NORM> constexpr int tdf_tail() {
    return NORM ? (ST == TSF_STORE_F32 ? 0 : 24) : 8;
}

// PAIR: interior samples read the x-paired copy P of a 16-bit field (one
// 16-byte load per corner row, sample_linear_pair_in) instead of F.
template <int ST, bool NORM, bool UNORM, bool PAIR, int EIG>
__global__ void __launch_bounds__(32 * kTdfWarps, 6) tdf_queue_kernel(const void *__restrict__ F, int X, int Y, int Z,
                                                                    float rmin, float rmax, float rstep,
                                                                    const CircleTable tab, void *T,
                                                                    float *__restrict__ Rout, int fast_ok,
                                                                    const uint4 *__restrict__ P) {
    static_assert(kTdfWarps == 4 && kSeg == 128, "a CTA is an 8x8x8 brick of four 8x4x4 warp blocks");
    __shared__ float se[kTdfWarps][6][kSeg];
    __shared__ unsigned char room[kTdfWarps][kSeg];      // sample_room: unclamped sampler while the margin fits
    __shared__ float stage[kTdfWarps][32];               // the tail's samples of one voxel-radius
    const int XY = X * Y;
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
        float H[3][3], V[3][3];
        hessian<ST, NORM>(F, X, Y, Z, tx(t), ty(t), tz(t), H);
        tdf_eigen<EIG>(H, V);
        se[w][0][t] = V[0][1]; se[w][1][t] = V[1][1]; se[w][2][t] = V[2][1];
        se[w][3][t] = V[0][2]; se[w][4][t] = V[1][2]; se[w][5][t] = V[2][2];
        const float e2[3] = {V[0][1], V[1][1], V[2][1]}, e3[3] = {V[0][2], V[1][2], V[2][2]};
        room[w][t] = fast_ok ? sample_room(tx(t), ty(t), tz(t), X, Y, Z, e2, e3) : 0;
    }
    __syncwarp();
    // phase 2: radius sweeps as tasks
    const unsigned full = 0xffffffffu;
    int task = lane < ntask ? lane : -1;
    int next = 32;                                   // next unstarted task (same in every lane)
    float radius = rmin, maxSum = 0.0f, maxRadius = 0.0f;
    int nr = 0;
    while (__any_sync(full, task >= 0)) {
        if (next >= ntask) {
            // The queue is empty: once few sweeps are left, the warp finishes
            // them one voxel at a time, lane j computing sample j of each
            // radius (the same samples; the owner's sum in sample order), so
            // that the lanes whose sweeps ended do not idle while the longest
            // ones run.
            unsigned act = __ballot_sync(full, task >= 0 && inside(task));
            if (__popc(act) <= tdf_tail<ST, NORM>()) {
                while (act) {
                    const int o = __ffs(act) - 1;
                    act &= act - 1u;
                    const int t = __shfl_sync(full, task, o);
                    float r = __shfl_sync(full, radius, o), ms = __shfl_sync(full, maxSum, o);
                    float mr = __shfl_sync(full, maxRadius, o);
                    int n = __shfl_sync(full, nr, o);
                    const float e2x = se[w][0][t], e2y = se[w][1][t], e2z = se[w][2][t];
                    const float e3x = se[w][3][t], e3y = se[w][4][t], e3z = se[w][5][t];
                    const float fx = (float)tx(t), fy = (float)ty(t), fz = (float)tz(t);
                    const int rm = room[w][t];
                    while (r <= rmax && n < kMaxRadii) {
                        float term = 0.0f;
                        if (lane < tab.n) {
                            const float3 va = circle_dir(tab.c[lane], tab.s[lane], e2x, e2y, e2z, e3x, e3y, e3z);
                            const float3 u = circle_point(fx, fy, fz, r, va);
                            float3 smp;
                            if (sample_margin(r) <= rm) {
                                if constexpr (PAIR)
                                    smp = sample_linear_pair_in<ST>(P, X, XY, u.x, u.y, u.z);
                                else
                                    smp = sample_linear_in<ST>(F, X, XY, u.x, u.y, u.z);
                            } else {
                                if constexpr (PAIR)
                                    smp = sample_linear_pair_clamped<ST>(P, X, Y, Z, u.x, u.y, u.z);
                                else
                                    smp = sample_linear<ST>(F, X, Y, Z, u.x, u.y, u.z);
                            }
                            term = radial_term(smp, va);
                        }
                        stage[w][lane] = term;
                        __syncwarp();
                        float rs = 0.0f;
                        for (int j = 0; j < tab.n; j++) rs = rs + stage[w][j];
                        __syncwarp();
                        rs = rs / (float)tab.n;
                        if (!(rs > ms)) break;
                        ms = rs;
                        mr = r;
                        r = r + rstep;
                        n++;
                    }
                    if (lane == 0) {
                        const int64_t i = lin(tx(t), ty(t), tz(t), X, Y);
                        if (UNORM) reinterpret_cast<uint16_t *>(T)[i] = to_unorm16(ms);
                        else reinterpret_cast<float *>(T)[i] = ms;
                        Rout[i] = mr;
                    }
                }
                return;
            }
        }
        bool done = true;
        if (task >= 0 && inside(task)) {
            const float e2x = se[w][0][task], e2y = se[w][1][task], e2z = se[w][2][task];
            const float e3x = se[w][3][task], e3y = se[w][4][task], e3z = se[w][5][task];
            const float fx = (float)tx(task), fy = (float)ty(task), fz = (float)tz(task);
            if (radius <= rmax && nr < kMaxRadii) {
                float rs = 0.0f;
                if (sample_margin(radius) <= room[w][task]) {
#pragma unroll 2
                    for (int j = 0; j < tab.n; j++) {
                        const float3 va = circle_dir(tab.c[j], tab.s[j], e2x, e2y, e2z, e3x, e3y, e3z);
                        const float3 u = circle_point(fx, fy, fz, radius, va);
                        float3 smp;
                        if constexpr (PAIR)
                            smp = sample_linear_pair_in<ST>(P, X, XY, u.x, u.y, u.z);
                        else
                            smp = sample_linear_in<ST>(F, X, XY, u.x, u.y, u.z);
                        rs = rs + radial_term(smp, va);
                    }
                } else {
#pragma unroll 2
                    for (int j = 0; j < tab.n; j++) {
                        const float3 va = circle_dir(tab.c[j], tab.s[j], e2x, e2y, e2z, e3x, e3y, e3z);
                        const float3 u = circle_point(fx, fy, fz, radius, va);
                        float3 smp;
                        if constexpr (PAIR)
                            smp = sample_linear_pair_clamped<ST>(P, X, Y, Z, u.x, u.y, u.z);
                        else
                            smp = sample_linear<ST>(F, X, Y, Z, u.x, u.y, u.z);
                        rs = rs + radial_term(smp, va);
                    }
                }
                rs = rs / (float)tab.n;
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


// Same filter with one circle sample per lane.
//
// The load-balanced sweeps above leave lanes idle at the end of each warp's
// queue (a voxel whose sweep runs to ten radii keeps its lane busy while the
// others have nothing left) and where a warp mixes voxels near the volume's
// faces (clamped sampler) with interior ones: about 29 % of the lanes idled
// in the sweeps.  Here a warp evaluates one voxel-radius at a time with lane j
// computing sample j of the circle, so every lane has work as long as any
// voxel-radius is left, and all lanes take the same sampler path.  A batch
// takes the current radius of every voxel held in the warp's 32 slots (slot v
// owned by lane v, refilled from the 128-voxel block in lane order as
// sweeps end); the 32 samples of each voxel-radius go to shared memory and
// the owning lane then sums them in sample order, so each voxel's arithmetic
// -- samples, their order of summation, the division, the comparison that
// ends the sweep -- is exactly tdf_circle_kernel's.
template <int ST, bool NORM, bool UNORM, bool PAIR, int EIG>
__global__ void __launch_bounds__(32 * kTdfWarps) tdf_lane_kernel(const void *__restrict__ F, int X, int Y, int Z,
                                                                   float rmin, float rmax, float rstep,
                                                                   const CircleTable tab, void *T,
                                                                   float *__restrict__ Rout, int fast_ok,
                                                                   const uint4 *__restrict__ P) {
    static_assert(kTdfWarps == 4 && kSeg == 128, "a CTA is an 8x8x8 brick of four 8x4x4 warp blocks");
    __shared__ float se[kTdfWarps][6][kSeg];
    __shared__ unsigned char room[kTdfWarps][kSeg];
    constexpr int kRows = 8;                               // voxel-radii per chunk of a batch
    __shared__ float dtb[kTdfWarps][kRows][33];            // [row][sample], padded row
    const int XY = X * Y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nbx = (X + 7) >> 3, nby = (Y + 7) >> 3;
    const int b = blockIdx.x;
    const int bx0 = (b % nbx) * 8, by0 = ((b / nbx) % nby) * 8 + (w & 1) * 4;
    const int bz0 = (b / (nbx * nby)) * 8 + (w >> 1) * 4;
    const int ntask = kSeg;
    auto tx = [&](int t) { return bx0 + (t & 7); };
    auto ty = [&](int t) { return by0 + ((t >> 3) & 3); };
    auto tz = [&](int t) { return bz0 + (t >> 5); };
    auto inside = [&](int t) { return tx(t) < X && ty(t) < Y && tz(t) < Z; };
    // phase 1: eigenvectors of the block's voxels (one voxel per lane)
    for (int t = lane; t < ntask; t += 32) {
        if (!inside(t)) continue;
        float H[3][3], V[3][3];
        hessian<ST, NORM>(F, X, Y, Z, tx(t), ty(t), tz(t), H);
        tdf_eigen<EIG>(H, V);
        se[w][0][t] = V[0][1]; se[w][1][t] = V[1][1]; se[w][2][t] = V[2][1];
        se[w][3][t] = V[0][2]; se[w][4][t] = V[1][2]; se[w][5][t] = V[2][2];
        const float e2[3] = {V[0][1], V[1][1], V[2][1]}, e3[3] = {V[0][2], V[1][2], V[2][2]};
        room[w][t] = fast_ok ? sample_room(tx(t), ty(t), tz(t), X, Y, Z, e2, e3) : 0;
    }
    __syncwarp();
    // phase 2: batches of voxel-radii, one sample per lane
    const unsigned full = 0xffffffffu;
    const int ns = tab.n;
    const float cj = tab.c[lane], sj = tab.s[lane];       // this lane's sample direction (lane < ns)
    int task = lane < ntask ? lane : -1;
    int next = 32;
    float radius = rmin, maxSum = 0.0f, maxRadius = 0.0f;
    int nr = 0;
    while (__any_sync(full, task >= 0)) {
        const bool eval = task >= 0 && inside(task) && radius <= rmax && nr < kMaxRadii;
        const unsigned M = __ballot_sync(full, eval);
        // chunks of up to kRows voxel-radii: their samples go to the rows of
        // dtb (row = rank of the owning slot in the chunk), then each owner sums
        // its row in sample order (a small staging buffer leaves L1 its room)
        float rs_own = 0.0f;
        for (unsigned m = M; m;) {
            unsigned rest = m;
            for (int q = 0; q < kRows && rest; q++) rest &= rest - 1;
            const unsigned chunk = m & ~rest;
            m = rest;
            int row = 0;
            for (unsigned c = chunk; c; c &= c - 1, row++) {
                const int v = __ffs(c) - 1;
                const int tv = __shfl_sync(full, task, v);
                const float rv = __shfl_sync(full, radius, v);
                const float e2x = se[w][0][tv], e2y = se[w][1][tv], e2z = se[w][2][tv];
                const float e3x = se[w][3][tv], e3y = se[w][4][tv], e3z = se[w][5][tv];
                const float fx = (float)tx(tv), fy = (float)ty(tv), fz = (float)tz(tv);
                float dt = 0.0f;
                if (lane < ns) {
                    const float3 va = circle_dir(cj, sj, e2x, e2y, e2z, e3x, e3y, e3z);
                    const float3 u = circle_point(fx, fy, fz, rv, va);
                    float3 smp;
                    if (sample_margin(rv) <= room[w][tv]) {
                        if constexpr (PAIR)
                            smp = sample_linear_pair_in<ST>(P, X, XY, u.x, u.y, u.z);
                        else
                            smp = sample_linear_in<ST>(F, X, XY, u.x, u.y, u.z);
                    } else {
                        if constexpr (PAIR)
                            smp = sample_linear_pair_clamped<ST>(P, X, Y, Z, u.x, u.y, u.z);
                        else
                            smp = sample_linear<ST>(F, X, Y, Z, u.x, u.y, u.z);
                    }
                    dt = radial_term(smp, va);
                }
                dtb[w][row][lane] = dt;
            }
            __syncwarp();
            if ((chunk >> lane) & 1u) {
                const int myrow = __popc(chunk & ((1u << lane) - 1u));
                float rs = 0.0f;
                for (int j = 0; j < ns; j++) rs = rs + dtb[w][myrow][j];
                rs_own = rs;
            }
            __syncwarp();
        }
        bool done = true;
        if (eval) {
            const float rs = rs_own / (float)ns;
            if (rs > maxSum) {
                maxSum = rs;
                maxRadius = radius;
                radius = radius + rstep;
                nr++;
                done = false;
            }
        }
        __syncwarp();
        if (task >= 0 && done && inside(task)) {
            const int64_t i = lin(tx(task), ty(task), tz(task), X, Y);
            if (UNORM) reinterpret_cast<uint16_t *>(T)[i] = to_unorm16(maxSum);
            else reinterpret_cast<float *>(T)[i] = maxSum;
            Rout[i] = maxRadius;
        }
        // lanes whose sweep ended take the next voxels, in lane order
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

// Launches the sweep kernel of eigen mode EIG.  kernel: 0 = the faster of the
// two brick kernels for the format (one sample per lane for snorm16, whose
// decode-heavy samples gain most from full lanes -- 256^3, radii 1-3: 7.9
// against 10.2 ms; the load-balanced sweeps for the others -- f16, radii
// 1-3: 7.2 against 7.3 ms, radii 2.5-7: 9.5 against 10.0 ms), 1 = one voxel
// per lane (tdf_circle_kernel), 2 = one
// sample per lane (tdf_lane_kernel), 3 = load-balanced sweeps
// (tdf_queue_kernel); P: the x-paired 16-bit copy of the field (brick kernels)
// or null.  All give the same bits.
template <int EIG>
int launch_tdf_kernels(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                       const CircleTable &tab, void *d_T, int unorm, float *d_R, cudaStream_t s, int kernel,
                       const uint4 *P, int fast_ok) {
    if (kernel == 0) kernel = st == TSF_STORE_SNORM16 ? 2 : 3;
    const bool queue = kernel == 3;
    const dim3 b(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    const bool norm = !(rmax < 4.0f);   // kernels.cl:1083-1091
    const unsigned qblocks = (unsigned)(((X + 7) / 8) * ((Y + 7) / 8) * ((Z + 7) / 8));   // 8^3 bricks
#define TSF_TDF_LAUNCH(ST, NORM, UN)                                                                                 \
    do {                                                                                                             \
        if (kernel == 2 && P)                                                                                        \
            tdf_lane_kernel<ST, NORM, UN, ST != TSF_STORE_F32, EIG><<<qblocks, 32 * kTdfWarps, 0, s>>>(             \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, P);                                    \
        else if (kernel == 2)                                                                                        \
            tdf_lane_kernel<ST, NORM, UN, false, EIG><<<qblocks, 32 * kTdfWarps, 0, s>>>(                           \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, nullptr);                              \
        else if (queue && P)                                                                                         \
            tdf_queue_kernel<ST, NORM, UN, ST != TSF_STORE_F32, EIG><<<qblocks, 32 * kTdfWarps, 0, s>>>(            \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, P);                                    \
        else if (queue)                                                                                              \
            tdf_queue_kernel<ST, NORM, UN, false, EIG><<<qblocks, 32 * kTdfWarps, 0, s>>>(                          \
                d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R, fast_ok, nullptr);                              \
        else                                                                                                         \
            tdf_circle_kernel<ST, NORM, UN, EIG><<<g, b, 0, s>>>(d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T,     \
                                                                 d_R);                                               \
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

}  // namespace tsf
