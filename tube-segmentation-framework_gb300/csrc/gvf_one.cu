// gvf_one.cu -- the reference's low-memory GVF, one component at a time
// (runLowMemoryGVF, gradientVectorFlow.cpp:1172-1300; kernels
// GVF3DInit_one_component / GVF3DIteration_one_component /
// GVF3DFinish_one_component, kernels.cl:1392-1462 and
// kernels_no_3d_write.cl:1669-1741).
//
// Per component c the reference keeps v_c and an init pair (f0_c, |f0|^2)
// stored in the field's format, iterates
//   v_c <- v_c + (mu L(v_c) - (v_c - f0_c) * sq)
// K times with the mirror boundary rule, and after the three components
// writes the field4 image with w = |v| (1 if 0).  The only arithmetic
// difference from the three-component iteration (gvf_zs_kernel and friends)
// is that |f0|^2 is stored: in 16-bit formats it is rounded to the format
// before use.  With FP32 storage both give the same bits.
//
// Layout in the workspace (6 N stored values): the three result planes
// (planar v, as tsf_gvf leaves it), a ping-pong plane, the f0_c plane and the
// sq plane.  Rows that split into 16-byte vectors take gvf_one_vec_kernel
// (one thread per vector, x-neighbours from the adjacent lanes by shuffles,
// the y / z neighbour vectors through L1); other rows take gvf_one_kernel (one
// thread per voxel).  Both evaluate each voxel with the same operations.
#include "packed.cuh"

namespace tsf {

int launch_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int st, cudaStream_t s);

// GVF3DInit_one_component: v_c = f0_c, init = (f0_c, |f0|^2), both in storage
template <int ST>
__global__ void gvf_one_init_kernel(const void *__restrict__ field4, int64_t n, int comp,
                                    typename Store<ST>::T *__restrict__ v, typename Store<ST>::T *__restrict__ f,
                                    typename Store<ST>::T *__restrict__ sq) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = Vec4Load<ST>::load(field4, i);
    const float s = (a.x * a.x + a.y * a.y) + a.z * a.z;
    const typename Store<ST>::T q = Store<ST>::store(comp == 0 ? a.x : (comp == 1 ? a.y : a.z));
    v[i] = q;
    f[i] = q;
    sq[i] = Store<ST>::store(s);
}

// GVF3DIteration_one_component: one iteration src -> dst of one component
template <int ST>
__global__ void __launch_bounds__(256) gvf_one_kernel(const typename Store<ST>::T *__restrict__ f,
                                                      const typename Store<ST>::T *__restrict__ sq,
                                                      const typename Store<ST>::T *__restrict__ src,
                                                      typename Store<ST>::T *__restrict__ dst, int X, int Y, int Z,
                                                      float mu) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= X) return;
    // extents >= 4, so mirrored positions lie in [1, size-2] and their
    // neighbours inside the volume
    const int px = mirror(x, X), py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t p = lin(px, py, pz, X, Y);
    const int64_t sy = X, sz = (int64_t)X * Y;
    const float v = Store<ST>::load(__ldg(src + p));
    float lap = -6.0f * v;
    lap = lap + Store<ST>::load(__ldg(src + p + 1));
    lap = lap + Store<ST>::load(__ldg(src + p - 1));
    lap = lap + Store<ST>::load(__ldg(src + p + sy));
    lap = lap + Store<ST>::load(__ldg(src + p - sy));
    lap = lap + Store<ST>::load(__ldg(src + p + sz));
    lap = lap + Store<ST>::load(__ldg(src + p - sz));
    const float f0 = Store<ST>::load(__ldg(f + p)), s = Store<ST>::load(__ldg(sq + p));
    const float upd = mu * lap - (v - f0) * s;
    dst[lin(x, y, z, X, Y)] = Store<ST>::store(v + upd);
}

// GVF3DIteration_one_component, one thread per BYTES-byte vector of a row.
// FULL: every lane holds a vector (the row's vector count a multiple of 32).
template <int ST, int BYTES, bool FULL>
__global__ void __launch_bounds__(256) gvf_one_vec_kernel(const typename Store<ST>::T *__restrict__ f,
                                                          const typename Store<ST>::T *__restrict__ sq,
                                                          const typename Store<ST>::T *__restrict__ src,
                                                          typename Store<ST>::T *__restrict__ dst, int X, int Y,
                                                          int Z, float mu) {
    using P = PackedV<ST, BYTES>;
    constexpr int VX = P::VX;
    static_assert(VX >= 4, "the x-boundary copy needs x = 2 in the first vector");
    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (y >= Y) return;                              // whole warp
    const int x0 = (blockIdx.x * 32 + lane) * VX;
    const bool act = FULL || x0 < X;
    const int py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t plane = (int64_t)X * Y;
    const int64_t p = (int64_t)pz * plane + (int64_t)py * X + (act ? x0 : 0);
    const typename Store<ST>::T *sp = src + p;
    float c[VX], yp[VX], ym[VX], zp[VX], zm[VX], fc[VX], qc[VX];
    P::unpack(act ? P::load(sp) : P::zero(), c);
    P::unpack(act ? P::load(sp + X) : P::zero(), yp);
    P::unpack(act ? P::load(sp - X) : P::zero(), ym);
    P::unpack(act ? P::load(sp + plane) : P::zero(), zp);
    P::unpack(act ? P::load(sp - plane) : P::zero(), zm);
    P::unpack(act ? P::load(f + p) : P::zero(), fc);
    P::unpack(act ? P::load(sq + p) : P::zero(), qc);
    const unsigned full = 0xffffffffu;
    const float xl_edge = (lane == 0 && act && x0 > 0) ? Store<ST>::load(sp[-1]) : 0.0f;
    const float xr_edge = (lane == 31 && act && x0 + VX < X) ? Store<ST>::load(sp[VX]) : 0.0f;
    float xl = __shfl_up_sync(full, c[VX - 1], 1);
    float xr = __shfl_down_sync(full, c[0], 1);
    xl = lane == 0 ? xl_edge : xl;
    xr = lane == 31 ? xr_edge : xr;
    if (!FULL && x0 + VX >= X) xr = xr_edge;          // last vector of a row
    float res[VX];
#pragma unroll
    for (int i = 0; i < VX; i++) {
        const float v = c[i];
        float lap = -6.0f * v;
        lap = lap + (i == VX - 1 ? xr : c[i + 1 < VX ? i + 1 : i]);
        lap = lap + (i == 0 ? xl : c[i > 0 ? i - 1 : 0]);
        lap = lap + yp[i];
        lap = lap + ym[i];
        lap = lap + zp[i];
        lap = lap + zm[i];
        const float upd = mu * lap - (v - fc[i]) * qc[i];
        res[i] = v + upd;
    }
    if (x0 == 0) res[0] = res[2];
    if (x0 + VX == X) res[VX - 1] = res[VX - 3];
    if (act) P::store(dst + (int64_t)z * plane + (int64_t)y * X + x0, res);
}

template <int ST>
static void launch_one_iteration(const typename Store<ST>::T *F, const typename Store<ST>::T *Q,
                                 const typename Store<ST>::T *src, typename Store<ST>::T *dst, int X, int Y, int Z,
                                 float mu, cudaStream_t s) {
    constexpr int VX = PackedV<ST, 16>::VX;
    if (X % VX == 0 && X >= 2 * VX) {
        const int nvec = X / VX;
        const dim3 b(32, 8), g((unsigned)((nvec + 31) / 32), (unsigned)((Y + 7) / 8), (unsigned)Z);
        if (nvec % 32 == 0)
            gvf_one_vec_kernel<ST, 16, true><<<g, b, 0, s>>>(F, Q, src, dst, X, Y, Z, mu);
        else
            gvf_one_vec_kernel<ST, 16, false><<<g, b, 0, s>>>(F, Q, src, dst, X, Y, Z, mu);
    } else {
        const dim3 b(256), g((unsigned)((X + 255) / 256), (unsigned)Y, (unsigned)Z);
        gvf_one_kernel<ST><<<g, b, 0, s>>>(F, Q, src, dst, X, Y, Z, mu);
    }
}

size_t gvf_one_workspace_size(int X, int Y, int Z, int st) {
    return (size_t)6 * (size_t)X * (size_t)Y * (size_t)Z * storage_bytes(st);
}

int run_gvf_one_component(const void *d_field4_in, int X, int Y, int Z, float mu, int iterations, int st,
                          void *d_field4_out, void *ws, size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_field4_in || !d_field4_out) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (iterations < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    if (Y > 65535 || Z > 65535) return fail(TSF_ERR_INVALID_ARG, "Y and Z must be <= 65535 for the low-memory GVF");
    if (!ws || ws_bytes < gvf_one_workspace_size(X, Y, Z, st))
        return fail(TSF_ERR_WORKSPACE, "low-memory GVF workspace too small");
    const int64_t n = (int64_t)X * Y * Z;
    const size_t es = storage_bytes(st);
    unsigned char *base = static_cast<unsigned char *>(ws);
    TSF_DISPATCH_STORAGE(st, ST, {
        using T = typename Store<ST>::T;
        T *V = reinterpret_cast<T *>(base);              // 3 result planes
        T *A = reinterpret_cast<T *>(base + 3 * n * es);  // ping-pong plane
        T *F = reinterpret_cast<T *>(base + 4 * n * es);
        T *Q = reinterpret_cast<T *>(base + 5 * n * es);
        const unsigned init_blocks = (unsigned)((n + 255) / 256);
        for (int c = 0; c < 3; c++) {
            T *vc = V + c * n;
            gvf_one_init_kernel<ST><<<init_blocks, 256, 0, s>>>(d_field4_in, n, c, vc, F, Q);
            TSF_CHECK_LAUNCH("gvf_one_init_kernel");
            T *src = vc, *dst = A;
            for (int it = 0; it < iterations; it++) {
                launch_one_iteration<ST>(F, Q, src, dst, X, Y, Z, mu, s);
                TSF_CHECK_LAUNCH("gvf_one_kernel");
                T *t = src; src = dst; dst = t;
            }
            if (src != vc) TSF_TRY_CUDA(cudaMemcpyAsync(vc, src, n * es, cudaMemcpyDeviceToDevice, s));
        }
    });
    return launch_gvf_finish(base, d_field4_out, X, Y, Z, st, s);
}

}  // namespace tsf
