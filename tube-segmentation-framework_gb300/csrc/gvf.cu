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
// Two kernels compute the same iteration:
//  * gvf_plain_kernel: one iteration per launch, one thread per voxel, all
//    seven stencil reads through L1/L2.  HBM-bound at 9s B / voxel-iteration.
//  * gvf_tb_kernel: TB iterations per launch (temporal blocking).  A CTA owns
//    an x-y tile and streams through z; each time level keeps one z-plane of
//    the tile (with a halo that shrinks by one voxel per level) in shared
//    memory and its z-1 / z+1 neighbours in registers.  Intermediate levels
//    are rounded to the storage format exactly as a stored iteration would
//    be, so both kernels give bit-identical results.
#include "tsf_common.cuh"

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
template <int ST, int VX> struct VecIO;

template <int ST> struct VecIO<ST, 4> {
    using T = typename Store<ST>::T;
    static __device__ __forceinline__ void load(const T *p, float o[4]) {
        if constexpr (ST == TSF_STORE_F32) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
            o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
        } else {
            const uint2 raw = __ldg(reinterpret_cast<const uint2 *>(p));
            T c[4];
            memcpy(c, &raw, 8);
#pragma unroll
            for (int i = 0; i < 4; i++) o[i] = Store<ST>::load(c[i]);
        }
    }
    static __device__ __forceinline__ void store(T *p, const float o[4]) {
        if constexpr (ST == TSF_STORE_F32) {
            *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
            T c[4];
#pragma unroll
            for (int i = 0; i < 4; i++) c[i] = Store<ST>::store(o[i]);
            uint2 raw;
            memcpy(&raw, c, 8);
            *reinterpret_cast<uint2 *>(p) = raw;
        }
    }
};

template <int ST> struct VecIO<ST, 2> {
    using T = typename Store<ST>::T;
    static __device__ __forceinline__ void load(const T *p, float o[2]) {
        if constexpr (ST == TSF_STORE_F32) {
            const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
            o[0] = v.x; o[1] = v.y;
        } else {
            const unsigned raw = __ldg(reinterpret_cast<const unsigned *>(p));
            T c[2];
            memcpy(c, &raw, 4);
            o[0] = Store<ST>::load(c[0]);
            o[1] = Store<ST>::load(c[1]);
        }
    }
    static __device__ __forceinline__ void store(T *p, const float o[2]) {
        if constexpr (ST == TSF_STORE_F32) {
            *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
        } else {
            T c[2] = {Store<ST>::store(o[0]), Store<ST>::store(o[1])};
            unsigned raw;
            memcpy(&raw, c, 4);
            *reinterpret_cast<unsigned *>(p) = raw;
        }
    }
};

// Eight bytes of stored components: 4 voxels of a 16-bit format or 2 of FP32,
// unpacked / packed two at a time with the paired conversion intrinsics.
template <int ST> struct Packed8 {
    using T = typename Store<ST>::T;
    static constexpr int VX = 8 / (int)sizeof(T);
    static __device__ __forceinline__ uint2 load(const T *p) { return __ldg(reinterpret_cast<const uint2 *>(p)); }
    static __device__ __forceinline__ void unpack(uint2 raw, float o[VX]) {
        if constexpr (ST == TSF_STORE_F32) {
            o[0] = __uint_as_float(raw.x);
            o[1] = __uint_as_float(raw.y);
        } else if constexpr (ST == TSF_STORE_F16) {
            const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&raw.x));
            const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&raw.y));
            o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
        } else if constexpr (ST == TSF_STORE_BF16) {
            o[0] = __uint_as_float(raw.x << 16);
            o[1] = __uint_as_float(raw.x & 0xffff0000u);
            o[2] = __uint_as_float(raw.y << 16);
            o[3] = __uint_as_float(raw.y & 0xffff0000u);
        } else {
            o[0] = Store<ST>::load((int16_t)(raw.x & 0xffffu));
            o[1] = Store<ST>::load((int16_t)(raw.x >> 16));
            o[2] = Store<ST>::load((int16_t)(raw.y & 0xffffu));
            o[3] = Store<ST>::load((int16_t)(raw.y >> 16));
        }
    }
    // rounds to the storage format (the only rounding of an iteration's result)
    static __device__ __forceinline__ void store(T *p, const float o[VX]) {
        uint2 raw;
        if constexpr (ST == TSF_STORE_F32) {
            raw.x = __float_as_uint(o[0]);
            raw.y = __float_as_uint(o[1]);
        } else if constexpr (ST == TSF_STORE_F16) {
            const __half2 a = __floats2half2_rn(o[0], o[1]), b = __floats2half2_rn(o[2], o[3]);
            raw.x = *reinterpret_cast<const unsigned *>(&a);
            raw.y = *reinterpret_cast<const unsigned *>(&b);
        } else if constexpr (ST == TSF_STORE_BF16) {
            const __nv_bfloat162 a = __floats2bfloat162_rn(o[0], o[1]), b = __floats2bfloat162_rn(o[2], o[3]);
            raw.x = *reinterpret_cast<const unsigned *>(&a);
            raw.y = *reinterpret_cast<const unsigned *>(&b);
        } else {
            T c[VX];
#pragma unroll
            for (int i = 0; i < VX; i++) c[i] = Store<ST>::store(o[i]);
            memcpy(&raw, c, 8);
        }
        *reinterpret_cast<uint2 *>(p) = raw;
    }
};

// One thread = the VX voxels of one 8-byte vector of one row of one plane.
// All loads of a thread are independent and issued together -- per component
// the centre vector and its y+-1 and z+-1 neighbours, plus the f0 vectors --
// and stay packed in registers until used, so a warp keeps 18 eight-byte
// loads in flight at ~40 registers.  The neighbour vectors are other threads'
// centre vectors, served by L1/L2, so HBM still sees each stored component
// once.  x-neighbours come from the adjacent lanes by shuffles.  Mirror rule:
// rows and planes are computed at mirror(y), mirror(z); the vector holding
// x = 0 / X-1 copies the result of x = 2 / X-3 (needs VX >= 3, or the
// neighbouring vector, see below).  Per voxel the arithmetic is exactly
// gvf_plain_kernel's.
template <int ST>
__global__ void __launch_bounds__(256) gvf_vec_kernel(const typename Store<ST>::T *__restrict__ f,
                                                      const typename Store<ST>::T *__restrict__ src,
                                                      typename Store<ST>::T *__restrict__ dst, int X, int Y, int Z,
                                                      float mu) {
    using T = typename Store<ST>::T;
    using P = Packed8<ST>;
    constexpr int VX = P::VX;
    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (y >= Y) return;                              // whole warp
    const int x0 = (blockIdx.x * 32 + lane) * VX;
    const bool act = x0 < X;
    const int py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    const int64_t p = (int64_t)pz * plane + (int64_t)py * X + x0;
    const unsigned full = 0xffffffffu;

    uint2 rf[3], rc[3], ryp[3], rym[3], rzp[3], rzm[3];
    const uint2 zero = make_uint2(0u, 0u);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T *s = src + c * n + p;
        rf[c] = act ? P::load(f + c * n + p) : zero;
        rc[c] = act ? P::load(s) : zero;
        ryp[c] = act ? P::load(s + X) : zero;
        rym[c] = act ? P::load(s - X) : zero;
        rzp[c] = act ? P::load(s + plane) : zero;
        rzm[c] = act ? P::load(s - plane) : zero;
    }
    float fv[3][VX], sqr[VX];
#pragma unroll
    for (int c = 0; c < 3; c++) P::unpack(rf[c], fv[c]);
#pragma unroll
    for (int i = 0; i < VX; i++) sqr[i] = (fv[0][i] * fv[0][i] + fv[1][i] * fv[1][i]) + fv[2][i] * fv[2][i];
    const int64_t o = (int64_t)z * plane + (int64_t)y * X + x0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float cc[VX], yp[VX], ym[VX], zp[VX], zm[VX];
        P::unpack(rc[c], cc);
        P::unpack(ryp[c], yp);
        P::unpack(rym[c], ym);
        P::unpack(rzp[c], zp);
        P::unpack(rzm[c], zm);
        // x-neighbours: the last voxel of the lane to the left, the first of the lane to the right
        float xl = __shfl_up_sync(full, cc[VX - 1], 1);
        float xr = __shfl_down_sync(full, cc[0], 1);
        if (lane == 0) xl = (act && x0 > 0) ? Store<ST>::load(src[c * n + p - 1]) : 0.0f;
        if (lane == 31) xr = (act && x0 + VX < X) ? Store<ST>::load(src[c * n + p + VX]) : 0.0f;
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
            const float upd = mu * lap - (v - fv[c][i]) * sqr[i];
            res[i] = v + upd;                        // rounded to storage by the store
        }
        if constexpr (VX >= 3) {
            if (x0 == 0) res[0] = res[2];
            if (x0 + VX == X) res[VX - 1] = res[VX - 3];
        } else {
            // VX == 2: x = 0 takes x = 2 (first voxel of the next lane), x = X-1
            // takes x = X-3 (last voxel of the previous lane)
            const float r_next0 = __shfl_down_sync(full, res[0], 1);
            const float r_prev1 = __shfl_up_sync(full, res[1], 1);
            if (x0 == 0) res[0] = (lane == 31) ? 0.0f : r_next0;
            if (x0 + VX == X) res[1] = (lane == 0) ? 0.0f : r_prev1;
        }
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

// Temporal blocking is not enabled yet: every launch runs one iteration.
static int gvf_tb_levels(int) { return 1; }
static int launch_gvf_tb(int, const void *, const void *, void *, int, int, int, float, int, cudaStream_t) {
    return fail(TSF_ERR_INVALID_ARG, "temporal blocking unavailable");
}

size_t gvf_workspace_size(int X, int Y, int Z, int st) {
    return (size_t)3 * (size_t)X * (size_t)Y * (size_t)Z * storage_bytes(st);
}

constexpr int kVecBY = 8;

static int launch_gvf_plain(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z,
                            float mu, cudaStream_t s) {
    const int vx = st == TSF_STORE_F32 ? 2 : 4;     // voxels per 8-byte vector
    // the x-boundary copy needs the vector holding x = 2 / X-3 in the same warp
    if (X % vx == 0 && X >= 8 && !(vx == 2 && X % 64 == 2)) {
        dim3 b(32, kVecBY), g((X / vx + 31) / 32, (Y + kVecBY - 1) / kVecBY, Z);
        TSF_DISPATCH_STORAGE(st, ST, {
            using T = typename Store<ST>::T;
            gvf_vec_kernel<ST><<<g, b, 0, s>>>((const T *)d_f0, (const T *)src, (T *)dst, X, Y, Z, mu);
        });
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

// Runs `iterations` Jacobi iterations in place on d_v.  mode: 0 = choose,
// 1 = one iteration per launch only, 2 = temporal blocking where possible.
int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st,
            void *ws, size_t ws_bytes, int mode, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_v) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (iterations < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    if (iterations == 0) return TSF_OK;
    const size_t need = gvf_workspace_size(X, Y, Z, st);
    if (!ws || ws_bytes < need) return fail(TSF_ERR_WORKSPACE, "GVF workspace too small");
    void *a = d_v, *b = ws;
    int left = iterations;
    const int tb = (mode == 1) ? 1 : gvf_tb_levels(st);
    while (left > 0) {
        int k = left >= tb ? tb : left;
        if (k > 1) {
            r = launch_gvf_tb(st, d_f0, a, b, X, Y, Z, mu, k, s);
        } else {
            r = launch_gvf_plain(st, d_f0, a, b, X, Y, Z, mu, s);
        }
        if (r) return r;
        void *t = a; a = b; b = t;
        left -= k;
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
