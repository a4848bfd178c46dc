// gvf.cu -- gradient vector flow, Jacobi form (reference GVF3DIteration /
// GVF3DFinish, kernels.cl:1464-1515; host loop gradientVectorFlow.cpp:1007-1172).
//
// Layout in HBM: the field v and the data term f0 are planar (three planes of
// N stored components each), so every access is a unit-stride run and a
// voxel-iteration moves exactly 9 stored components: v (3) and f0 (3) read,
// v (3) written -- 36 B in FP32, 18 B in the 16-bit formats.  |f0|^2 is
// recomputed from the stored f0 each time, exactly like the reference (which
// keeps f0z in v.w and f0x,f0y in an RG image).
//
// Three kernels compute the same iteration, bit for bit:
//  * gvf_zs_kernel (gvf_zs.cu): z-streaming with TMA copies into a shared
//    memory ring of planes; the default wherever rows are a multiple of 16
//    bytes and the buffers 16-byte aligned.
//  * gvf_vec_kernel: one thread per 8- or 16-byte vector of a row, all loads
//    held in registers; rows that split into such vectors.
//  * gvf_plain_kernel: one thread per voxel; any shape.
#include "packed.cuh"

namespace tsf {

// ---------------------------------------------------------------------------
// one iteration per launch
// ---------------------------------------------------------------------------
template <int ST>
__global__ void __launch_bounds__(256) gvf_plain_kernel(const typename Store<ST>::T *__restrict__ f,
                                                        const typename Store<ST>::T *__restrict__ src,
                                                        typename Store<ST>::T *__restrict__ dst,
                                                        int X, int Y, int Z, float mu) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    const int64_t n = (int64_t)X * Y * Z;
    const int px = mirror(x, X), py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t p = lin(px, py, pz, X, Y);
    const int64_t sx = 1, sy = X, sz = (int64_t)X * Y;
    const float fx = Store<ST>::load(__ldg(f + p));
    const float fy = Store<ST>::load(__ldg(f + n + p));
    const float fz = Store<ST>::load(__ldg(f + 2 * n + p));
    const float sqr = (fx * fx + fy * fy) + fz * fz;
    const int64_t o = lin(x, y, z, X, Y);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const typename Store<ST>::T *s = src + c * n;
        const float v = Store<ST>::load(__ldg(s + p));
        float lap = -6.0f * v;
        lap = lap + Store<ST>::load(__ldg(s + p + sx));
        lap = lap + Store<ST>::load(__ldg(s + p - sx));
        lap = lap + Store<ST>::load(__ldg(s + p + sy));
        lap = lap + Store<ST>::load(__ldg(s + p - sy));
        lap = lap + Store<ST>::load(__ldg(s + p + sz));
        lap = lap + Store<ST>::load(__ldg(s + p - sz));
        const float fc = c == 0 ? fx : (c == 1 ? fy : fz);
        const float upd = mu * lap - (v - fc) * sqr;
        dst[c * n + o] = Store<ST>::store(v + upd);
    }
}

// ---------------------------------------------------------------------------
// one iteration per launch, z-streaming, VX voxels per thread along x
//
// A warp covers 32*VX consecutive voxels of one row; each thread walks a chunk
// of ZC planes keeping the planes z-1, z, z+1 of its VX columns in registers,
// so every stored component of v is fetched from HBM once (as the "next"
// plane); the y-neighbour rows come from L1 (the adjacent warps of the block
// fetch them) and the x-neighbours from the neighbouring lanes by shuffles.
// The mirror boundary rule is applied as: rows compute at mirror(y); the
// vector holding x = 0 / X-1 copies the result of x = 2 / X-3; the thread that
// computes plane 2 / Z-3 also writes plane 0 / Z-1 (chunks are >= 3 planes
// and the last chunk is shifted to end at Z, so those pairs never straddle a
// chunk).  Per voxel the arithmetic is exactly gvf_plain_kernel's.
// ---------------------------------------------------------------------------
// One thread = the VX voxels of one vector (BYTES bytes) of one row of one
// plane.  All loads of a thread are independent and issued together -- per
// component the centre vector and its y+-1 and z+-1 neighbours, plus the f0
// vectors -- and stay packed in registers until used.  The neighbour vectors
// are other threads' centre vectors, served by L1/L2, so HBM sees each stored
// component once.  x-neighbours come from the adjacent lanes by shuffles (the
// first / last lane of a warp reads its one outside neighbour itself).  FULL:
// every lane of every warp holds a vector (X / VX a multiple of 32), so no
// per-lane activity test is needed.  Mirror rule: rows and planes are computed
// at mirror(y), mirror(z); the vector holding x = 0 / X-1 copies the result of
// x = 2 / X-3.  Per voxel the arithmetic is exactly gvf_plain_kernel's.
template <int ST, int BYTES, bool FULL>
__global__ void __launch_bounds__(256) gvf_vec_kernel(const typename Store<ST>::T *__restrict__ f,
                                                      const typename Store<ST>::T *__restrict__ src,
                                                      typename Store<ST>::T *__restrict__ dst, int X, int Y, int Z,
                                                      float mu) {
    using T = typename Store<ST>::T;
    using P = PackedV<ST, BYTES>;
    using Raw = typename P::Raw;
    constexpr int VX = P::VX;
    static_assert(VX >= 4, "the x-boundary copy needs x = 2 in the first vector");
    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (y >= Y) return;                              // whole warp
    const int x0 = (blockIdx.x * 32 + lane) * VX;
    const bool act = FULL || x0 < X;
    const int py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    const int64_t p = (int64_t)pz * plane + (int64_t)py * X + x0;
    const unsigned full = 0xffffffffu;

    Raw rf[3], rc[3], ryp[3], rym[3], rzp[3], rzm[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T *sp = src + c * n + p;
        if (act) {
            rf[c] = P::load(f + c * n + p);
            rc[c] = P::load(sp);
            ryp[c] = P::load(sp + X);
            rym[c] = P::load(sp - X);
            rzp[c] = P::load(sp + plane);
            rzm[c] = P::load(sp - plane);
        } else {
            rf[c] = rc[c] = ryp[c] = rym[c] = rzp[c] = rzm[c] = P::zero();
        }
    }
    float sqr[VX];
    {
        float f0[VX], f1[VX], f2[VX];
        P::unpack(rf[0], f0);
        P::unpack(rf[1], f1);
        P::unpack(rf[2], f2);
#pragma unroll
        for (int i = 0; i < VX; i++) sqr[i] = (f0[i] * f0[i] + f1[i] * f1[i]) + f2[i] * f2[i];
    }
    const int64_t o = (int64_t)z * plane + (int64_t)y * X + x0;
    // the lanes at a warp's edge read their outside x-neighbour themselves
    const bool left_out = lane == 0 && act && x0 > 0;
    const bool right_out = lane == 31 && act && x0 + VX < X;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T *sp = src + c * n + p;
        const float xl_edge = left_out ? Store<ST>::load(sp[-1]) : 0.0f;
        const float xr_edge = right_out ? Store<ST>::load(sp[VX]) : 0.0f;
        float cc[VX], yp[VX], ym[VX], zp[VX], zm[VX], fc[VX];
        P::unpack(rc[c], cc);
        P::unpack(ryp[c], yp);
        P::unpack(rym[c], ym);
        P::unpack(rzp[c], zp);
        P::unpack(rzm[c], zm);
        P::unpack(rf[c], fc);
        float xl = __shfl_up_sync(full, cc[VX - 1], 1);
        float xr = __shfl_down_sync(full, cc[0], 1);
        xl = lane == 0 ? xl_edge : xl;
        xr = lane == 31 ? xr_edge : xr;
        float res[VX];
#pragma unroll
        for (int i = 0; i < VX; i++) {
            const float v = cc[i];
            float lap = -6.0f * v;
            lap = lap + (i == VX - 1 ? xr : cc[i + 1 < VX ? i + 1 : i]);
            lap = lap + (i == 0 ? xl : cc[i > 0 ? i - 1 : 0]);
            lap = lap + yp[i];
            lap = lap + ym[i];
            lap = lap + zp[i];
            lap = lap + zm[i];
            const float upd = mu * lap - (v - fc[i]) * sqr[i];
            res[i] = v + upd;                        // rounded to storage by the store
        }
        if (x0 == 0) res[0] = res[2];
        if (x0 + VX == X) res[VX - 1] = res[VX - 3];
        if (act) P::store(dst + c * n + o, res);
    }
}

// ---------------------------------------------------------------------------
// GVF3DFinish: planar -> field4 with w = |v| (1 if 0)
// ---------------------------------------------------------------------------
template <int ST>
__global__ void gvf_finish_kernel(const typename Store<ST>::T *__restrict__ v, void *field4, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = Store<ST>::load(v[i]), y = Store<ST>::load(v[n + i]), z = Store<ST>::load(v[2 * n + i]);
    const float l = sqrtf((x * x + y * y) + z * z);
    store4<ST>(field4, i, x, y, z, l > 0.0f ? l : 1.0f);
}

bool gvf_zs_eligible(int st, const void *d_f0, const void *a, const void *b, int X, int Y, int Z);
int launch_gvf_zs(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu,
                  cudaStream_t s, int rev = 0);

size_t gvf_workspace_size(int X, int Y, int Z, int st) {
    return (size_t)3 * (size_t)X * (size_t)Y * (size_t)Z * storage_bytes(st);
}

constexpr int kVecBY = 8;

template <int ST, int BYTES>
static void launch_vec(const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu, cudaStream_t s) {
    using T = typename Store<ST>::T;
    constexpr int VX = PackedV<ST, BYTES>::VX;
    const int nvec = X / VX;
    dim3 b(32, kVecBY), g((nvec + 31) / 32, (Y + kVecBY - 1) / kVecBY, Z);
    if (nvec % 32 == 0)
        gvf_vec_kernel<ST, BYTES, true><<<g, b, 0, s>>>((const T *)d_f0, (const T *)src, (T *)dst, X, Y, Z, mu);
    else
        gvf_vec_kernel<ST, BYTES, false><<<g, b, 0, s>>>((const T *)d_f0, (const T *)src, (T *)dst, X, Y, Z, mu);
}

static int launch_gvf_plain(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z,
                            float mu, cudaStream_t s) {
    // 16-byte vectors when the row splits into them, else 8-byte ones (FP32
    // 8-byte vectors hold 2 voxels, too few for the in-vector boundary copy)
    const int es = (int)storage_bytes(st);
    const int vx16 = 16 / es, vx8 = 8 / es;
    if (X % vx16 == 0 && X >= 2 * vx16) {
        TSF_DISPATCH_STORAGE(st, ST, launch_vec<ST, 16>(d_f0, src, dst, X, Y, Z, mu, s));
        TSF_CHECK_LAUNCH("gvf_vec_kernel");
        return TSF_OK;
    }
    if (es == 2 && X % vx8 == 0 && X >= 2 * vx8) {
        switch (st) {
        case TSF_STORE_F16: launch_vec<TSF_STORE_F16, 8>(d_f0, src, dst, X, Y, Z, mu, s); break;
        case TSF_STORE_BF16: launch_vec<TSF_STORE_BF16, 8>(d_f0, src, dst, X, Y, Z, mu, s); break;
        default: launch_vec<TSF_STORE_SNORM16, 8>(d_f0, src, dst, X, Y, Z, mu, s); break;
        }
        TSF_CHECK_LAUNCH("gvf_vec_kernel");
        return TSF_OK;
    }
    dim3 b(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    TSF_DISPATCH_STORAGE(st, ST, {
        using T = typename Store<ST>::T;
        gvf_plain_kernel<ST><<<g, b, 0, s>>>((const T *)d_f0, (const T *)src, (T *)dst, X, Y, Z, mu);
    });
    TSF_CHECK_LAUNCH("gvf_plain_kernel");
    return TSF_OK;
}

// One iteration from src to dst (distinct buffers); the streaming kernel
// where it applies.
int gvf_step(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu, cudaStream_t s) {
    if (gvf_zs_eligible(st, d_f0, src, dst, X, Y, Z)) return launch_gvf_zs(st, d_f0, src, dst, X, Y, Z, mu, s);
    return launch_gvf_plain(st, d_f0, src, dst, X, Y, Z, mu, s);
}

// Runs `iterations` Jacobi iterations in place on d_v, one iteration per
// launch, ping-ponging with the workspace.  mode: 0 = default (the streaming
// kernel gvf_zs_kernel where it applies, else gvf_vec_kernel), 1 = the
// register-vector kernels only, 2 = same as 0.  All give identical results.
bool gvf_tb2_eligible(int st, const void *d_f0, const void *a, const void *b, int X, int Y, int Z);
int launch_gvf_tb2(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu,
                   cudaStream_t s);

int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st,
            void *ws, size_t ws_bytes, int mode, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_v) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (iterations < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    if (mode < 0 || mode > 3) return fail(TSF_ERR_INVALID_ARG, "unknown GVF mode");
    if (iterations == 0) return TSF_OK;
    const size_t need = gvf_workspace_size(X, Y, Z, st);
    if (!ws || ws_bytes < need) return fail(TSF_ERR_WORKSPACE, "GVF workspace too small");
    void *a = d_v, *b = ws;
    const bool zs = mode != 1 && gvf_zs_eligible(st, d_f0, a, b, X, Y, Z);
    int left = iterations;
    if (mode == 3 && gvf_tb2_eligible(st, d_f0, a, b, X, Y, Z)) {
        // two iterations per launch; an odd count ends with one of the
        // one-iteration kernel
        for (; left >= 2; left -= 2) {
            r = launch_gvf_tb2(st, d_f0, a, b, X, Y, Z, mu, s);
            if (r) return r;
            void *t = a; a = b; b = t;
        }
    }
    for (; left > 0; left--) {
        // alternate the streaming direction: each iteration starts on the
        // planes the previous one wrote last, which are still in L2
        const int rev = mode == 2 ? 0 : (iterations - left) & 1;
        r = zs ? launch_gvf_zs(st, d_f0, a, b, X, Y, Z, mu, s, rev) : launch_gvf_plain(st, d_f0, a, b, X, Y, Z, mu, s);
        if (r) return r;
        void *t = a; a = b; b = t;
    }
    if (a != d_v) {
        TSF_TRY_CUDA(cudaMemcpyAsync(d_v, a, need, cudaMemcpyDeviceToDevice, s));
    }
    return TSF_OK;
}

int launch_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int st, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_v || !d_field4) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    const int64_t n = (int64_t)X * Y * Z;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    TSF_DISPATCH_STORAGE(st, ST, {
        using T = typename Store<ST>::T;
        gvf_finish_kernel<ST><<<blocks, threads, 0, s>>>((const T *)d_v, d_field4, n);
    });
    TSF_CHECK_LAUNCH("gvf_finish_kernel");
    return TSF_OK;
}

}  // namespace tsf
