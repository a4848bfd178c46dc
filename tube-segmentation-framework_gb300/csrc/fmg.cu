// fmg.cu -- full-multigrid GVF (reference runFMGGVF, fullMultigrid,
// multigridVcycle, gaussSeidelSmoothing, restrictVolume, prolongateVolume{,2},
// residual, computeNewResidual: gradientVectorFlow.cpp:5-441, 631-1005;
// kernels GVFgaussSeidel{,2}, restrictVolume, prolongate{,2}, residual,
// fmgResidual, createSqrMag, addTwoImages, MGGVFFinish: kernels.cl:1775-2061).
//
// Per component the reference solves mu*Lap(v) - |f|^2 v = -|f|^2 f with
// `iterations` FMG cycles (v0 = 1, v1 = 2, v2 = 2, three levels, spacing
// doubling per level).  Every intermediate image is rounded to the storage
// format, as the reference's CL_R images are.  Reproduced quirks: the
// Gauss-Seidel update divides by 12 mu + h^2 |f|^2 (not 12 mu + 2 h^2 |f|^2);
// the first half-sweep writes red points only and the second copies red
// points and computes black ones; coarse grids are the largest power-of-two
// cube below the largest extent; restriction reads 0 outside the fine image.
// Arithmetic uses IEEE division where the reference uses native_divide.
//
// All images of one run live in one workspace, laid out once; the restricted
// |f|^2 images are computed once per run (the reference recomputes identical
// ones in every cycle).
#include "packed.cuh"

namespace tsf {

struct Dim { int x, y, z; };
static inline int64_t nvox(Dim d) { return (int64_t)d.x * d.y * d.z; }

// calculateNewSize, gradientVectorFlow.cpp:371-395
static Dim fmg_new_size(Dim s) {
    bool ok = false;
    if (s.x == s.y && s.x == s.z) {
        int p = 1;
        while (p < s.x) p *= 2;
        ok = (p == s.x);
    }
    int ns;
    if (!ok) {
        int mx = s.x > s.y ? s.x : s.y;
        if (s.z > mx) mx = s.z;
        int i = 1;
        while ((1 << i) < mx) i++;
        ns = 1 << (i - 1);
    } else {
        ns = s.x / 2;
    }
    return Dim{ns, ns, ns};
}

template <int ST> using ST_T = typename Store<ST>::T;

template <int ST>
__device__ __forceinline__ float ld0(const ST_T<ST> *a, Dim d, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= d.x || y >= d.y || z >= d.z) return 0.0f;
    return Store<ST>::load(a[lin(x, y, z, d.x, d.y)]);
}
template <int ST>
__device__ __forceinline__ float ldc(const ST_T<ST> *a, Dim d, int x, int y, int z) {
    return Store<ST>::load(a[lin(clampi(x, d.x), clampi(y, d.y), clampi(z, d.z), d.x, d.y)]);
}

#define FMG_THREAD_XYZ(d)                                       \
    const int x = blockIdx.x * blockDim.x + threadIdx.x;        \
    const int y = blockIdx.y * blockDim.y + threadIdx.y;        \
    const int z = blockIdx.z * blockDim.z + threadIdx.z;        \
    if (x >= (d).x || y >= (d).y || z >= (d).z) return;

// createSqrMag (kernels.cl:1868-1878)
template <int ST>
__global__ void sqrmag_kernel(const void *F, Dim d, ST_T<ST> *sq) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(d);
    const int64_t i = lin(x, y, z, d.x, d.y);
    const float4 q = Vec4Load<ST>::load(F, i);
    sq[i] = Store<ST>::store((q.x * q.x + q.y * q.y) + q.z * q.z);
}

// fmgResidual (kernels.cl:2008-2053), spacing 1
template <int ST>
__global__ void fmg_residual_kernel(const void *F, const ST_T<ST> *f, Dim d, int comp, float mu, ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(d);
    const int px = mirror(x, d.x), py = mirror(y, d.y), pz = mirror(z, d.z);
    const float4 q = Vec4Load<ST>::load(F, lin(px, py, pz, d.x, d.y));
    const float v0 = comp == 0 ? q.x : (comp == 1 ? q.y : q.z);
    const float sqm = (q.x * q.x + q.y * q.y) + q.z * q.z;
    const float fc = ld0<ST>(f, d, px, py, pz);
    float s = ld0<ST>(f, d, px + 1, py, pz);
    s = s + ld0<ST>(f, d, px - 1, py, pz);
    s = s + ld0<ST>(f, d, px, py + 1, pz);
    s = s + ld0<ST>(f, d, px, py - 1, pz);
    s = s + ld0<ST>(f, d, px, py, pz + 1);
    s = s + ld0<ST>(f, d, px, py, pz - 1);
    s = s - 6.0f * fc;
    const float res = (mu * s) / (1.0f * 1.0f);
    const float value = (-sqm) * v0 - (res - sqm * fc);
    out[lin(x, y, z, d.x, d.y)] = Store<ST>::store(value);
}

// GVFgaussSeidel (RED = true) / GVFgaussSeidel2 (RED = false), kernels.cl:1775-1854
template <int ST, bool RED>
__global__ void gs_kernel(const ST_T<ST> *src, ST_T<ST> *dst, const ST_T<ST> *r, const ST_T<ST> *sq, Dim d,
                          float two_mu, float twelve_mu, float hh, float two_hh) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(d);
    const int px = mirror(x, d.x), py = mirror(y, d.y), pz = mirror(z, d.z);
    const bool red = ((px + py + pz) % 2) == 0;
    if (RED && !red) return;
    float value;
    if (!RED && red) {
        value = Store<ST>::load(src[lin(px, py, pz, d.x, d.y)]);
    } else {
        float s = ldc<ST>(src, d, px + 1, py, pz);
        s = s + ldc<ST>(src, d, px - 1, py, pz);
        s = s + ldc<ST>(src, d, px, py + 1, pz);
        s = s + ldc<ST>(src, d, px, py - 1, pz);
        s = s + ldc<ST>(src, d, px, py, pz + 1);
        s = s + ldc<ST>(src, d, px, py, pz - 1);
        const int64_t p = lin(px, py, pz, d.x, d.y);
        const float num = two_mu * s - two_hh * Store<ST>::load(r[p]);
        const float den = twelve_mu + hh * Store<ST>::load(sq[p]);
        value = num / den;
    }
    dst[lin(x, y, z, d.x, d.y)] = Store<ST>::store(value);
}

// residual (kernels.cl:1973-2006)
template <int ST>
__global__ void residual_kernel(const ST_T<ST> *r, const ST_T<ST> *v, const ST_T<ST> *sq, Dim d, float mu, float h,
                                ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(d);
    const int px = mirror(x, d.x), py = mirror(y, d.y), pz = mirror(z, d.z);
    const float vc = ld0<ST>(v, d, px, py, pz);
    float s = ld0<ST>(v, d, px + 1, py, pz);
    s = s + ld0<ST>(v, d, px - 1, py, pz);
    s = s + ld0<ST>(v, d, px, py + 1, pz);
    s = s + ld0<ST>(v, d, px, py - 1, pz);
    s = s + ld0<ST>(v, d, px, py, pz + 1);
    s = s + ld0<ST>(v, d, px, py, pz - 1);
    s = s - 6.0f * vc;
    const float lap = (mu * s) / (h * h);
    const float value = ld0<ST>(r, d, px, py, pz) - (lap - ld0<ST>(sq, d, px, py, pz) * vc);
    out[lin(x, y, z, d.x, d.y)] = Store<ST>::store(value);
}

// restrictVolume (kernels.cl:1923-1951)
template <int ST>
__global__ void restrict_kernel(const ST_T<ST> *fine, Dim fd, Dim cd, ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(cd);
    int px = 2 * x, py = 2 * y, pz = 2 * z;
    if (px >= 2 * cd.x - 1) px = 2 * cd.x - 3;
    if (py >= 2 * cd.y - 1) py = 2 * cd.y - 3;
    if (pz >= 2 * cd.z - 1) pz = 2 * cd.z - 3;
    float s = ld0<ST>(fine, fd, px, py, pz);
    s = s + ld0<ST>(fine, fd, px + 1, py, pz);
    s = s + ld0<ST>(fine, fd, px, py + 1, pz);
    s = s + ld0<ST>(fine, fd, px, py, pz + 1);
    s = s + ld0<ST>(fine, fd, px + 1, py + 1, pz);
    s = s + ld0<ST>(fine, fd, px, py + 1, pz + 1);
    s = s + ld0<ST>(fine, fd, px + 1, py + 1, pz + 1);
    s = s + ld0<ST>(fine, fd, px + 1, py, pz + 1);
    out[lin(x, y, z, cd.x, cd.y)] = Store<ST>::store(0.125f * s);
}

// prolongate (ADD) / prolongate2 (kernels.cl:1953-1970)
template <int ST, bool ADD>
__global__ void prolong_kernel(const ST_T<ST> *fine_in, const ST_T<ST> *coarse, Dim fd, Dim cd, ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_THREAD_XYZ(fd);
    const float c = ld0<ST>(coarse, cd, x / 2, y / 2, z / 2);
    const int64_t i = lin(x, y, z, fd.x, fd.y);
    const float value = ADD ? Store<ST>::load(fine_in[i]) + c : c;
    out[i] = Store<ST>::store(value);
}

// addTwoImages (kernels.cl:1857-1865), in place on a
template <int ST>
__global__ void add_kernel(ST_T<ST> *a, const ST_T<ST> *b, int64_t n) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = Store<ST>::store(Store<ST>::load(a[i]) + Store<ST>::load(b[i]));
}

// MGGVFFinish (kernels.cl:1907-1921): w = |v| (no special case for 0)
template <int ST>
__global__ void fmg_finish_kernel(const ST_T<ST> *fx, const ST_T<ST> *fy, const ST_T<ST> *fz, void *out, int64_t n) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = Store<ST>::load(fx[i]), y = Store<ST>::load(fy[i]), z = Store<ST>::load(fz[i]);
    store4<ST>(out, i, x, y, z, sqrtf((x * x + y * y) + z * z));
}

// ---------------------------------------------------------------------------
// vectorised level kernels: one thread per 4 voxels of a row (an 8-byte vector
// of a 16-bit format, 16 bytes of FP32; 8-byte vectors measured 5 % faster
// than 16-byte ones for 16-bit formats: half the registers per thread, twice
// the resident warps), loads issued together, x-neighbours by
// shuffles.  Rows evaluate at mirror(y), planes at mirror(z); the vector
// holding x = 0 / X-1 copies the result of x = 2 / X-3.  Per voxel the
// arithmetic is exactly the scalar kernels', so the results are identical.
// ---------------------------------------------------------------------------
template <int ST> struct FmgVec {
    using P = PackedV<ST, ST == TSF_STORE_F32 ? 16 : 8>;
    using Raw = typename P::Raw;
    static constexpr int VX = P::VX;
};

// x-neighbours of a row vector c: xl = value at x0-1, xr = value at x0+VX
template <int VX>
__device__ __forceinline__ void fmg_xnb(const float c[VX], float el, float er, int lane, float &xl, float &xr) {
    const unsigned full = 0xffffffffu;
    xl = __shfl_up_sync(full, c[VX - 1], 1);
    xr = __shfl_down_sync(full, c[0], 1);
    if (lane == 0) xl = el;
    if (lane == 31) xr = er;
}

#define FMG_VEC_PROLOGUE(d)                                                     \
    using P = typename FmgVec<ST>::P;                                           \
    constexpr int VX = FmgVec<ST>::VX;                                          \
    const int lane = threadIdx.x;                                               \
    const int y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;       \
    if (y >= (d).y) return;                                                     \
    const int x0 = (blockIdx.x * 32 + lane) * VX;                               \
    const bool act = x0 < (d).x;                                                \
    const int py = mirror(y, (d).y), pz = mirror(z, (d).z);                     \
    const int64_t sy = (d).x, sz = (int64_t)(d).x * (d).y;                      \
    const int64_t p = (int64_t)pz * sz + (int64_t)py * sy + (act ? x0 : 0);     \
    const int64_t o = (int64_t)z * sz + (int64_t)y * sy + x0;

template <int ST>
__device__ __forceinline__ void fmg_load(const ST_T<ST> *a, int64_t i, bool act, float out[FmgVec<ST>::VX]) {
    using P = typename FmgVec<ST>::P;
    P::unpack(act ? P::load(a + i) : P::zero(), out);
}

// GVFgaussSeidel (RED) / GVFgaussSeidel2, vectorised.  RED: lanes on black
// points write the source value, which no later pass reads (the reference
// leaves them unwritten).
template <int ST, bool RED>
__global__ void __launch_bounds__(256) gs_vec_kernel(const ST_T<ST> *src, ST_T<ST> *dst, const ST_T<ST> *r,
                                                     const ST_T<ST> *sq, Dim d, float two_mu, float twelve_mu,
                                                     float hh, float two_hh) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_VEC_PROLOGUE(d);
    // FP16 / BF16: the y and z neighbours enter the sum unconverted
    // (mixed-precision adds, the bits of convert-then-add)
    constexpr bool MIX = ST == TSF_STORE_F16 || ST == TSF_STORE_BF16;
    float c[VX], yp[VX], ym[VX], zp[VX], zm[VX], rr[VX], qq[VX];
    typename P::Raw ryp, rym, rzp, rzm;
    fmg_load<ST>(src, p, act, c);
    if constexpr (MIX) {
        ryp = act ? P::load(src + p + sy) : P::zero();
        rym = act ? P::load(src + p - sy) : P::zero();
        rzp = act ? P::load(src + p + sz) : P::zero();
        rzm = act ? P::load(src + p - sz) : P::zero();
    } else {
        fmg_load<ST>(src, p + sy, act, yp);
        fmg_load<ST>(src, p - sy, act, ym);
        fmg_load<ST>(src, p + sz, act, zp);
        fmg_load<ST>(src, p - sz, act, zm);
    }
    fmg_load<ST>(r, p, act, rr);
    fmg_load<ST>(sq, p, act, qq);
    const float el = (act && x0 > 0) ? Store<ST>::load(src[p - 1]) : 0.0f;
    const float er = (act && x0 + VX < d.x) ? Store<ST>::load(src[p + VX]) : 0.0f;
    float xl, xr;
    fmg_xnb<VX>(c, el, er, lane, xl, xr);
    if (x0 + VX >= d.x) xr = er;                  // last vector of a row: no lane to the right
    float res[VX];
#pragma unroll
    for (int i = 0; i < VX; i++) {
        const bool red = ((x0 + i + py + pz) & 1) == 0;
        if (RED != red) {
            res[i] = c[i];
        } else {
            float s = i == VX - 1 ? xr : c[i + 1 < VX ? i + 1 : i];
            s = s + (i == 0 ? xl : c[i > 0 ? i - 1 : 0]);
            if constexpr (MIX) {
                s = add16i<ST>(ryp.u, i, s);
                s = add16i<ST>(rym.u, i, s);
                s = add16i<ST>(rzp.u, i, s);
                s = add16i<ST>(rzm.u, i, s);
            } else {
                s = s + yp[i];
                s = s + ym[i];
                s = s + zp[i];
                s = s + zm[i];
            }
            const float num = two_mu * s - two_hh * rr[i];
            const float den = twelve_mu + hh * qq[i];
            res[i] = num / den;
        }
    }
    if (x0 == 0) res[0] = res[2];
    if (x0 + VX == d.x) res[VX - 1] = res[VX - 3];
    if (act) P::store(dst + o, res);
}

// residual (kernels.cl:1973-2006), vectorised
template <int ST>
__global__ void __launch_bounds__(256) residual_vec_kernel(const ST_T<ST> *r, const ST_T<ST> *v, const ST_T<ST> *sq,
                                                           Dim d, float mu, float h, ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_VEC_PROLOGUE(d);
    float c[VX], yp[VX], ym[VX], zp[VX], zm[VX], rr[VX], qq[VX];
    fmg_load<ST>(v, p, act, c);
    fmg_load<ST>(v, p + sy, act, yp);
    fmg_load<ST>(v, p - sy, act, ym);
    fmg_load<ST>(v, p + sz, act, zp);
    fmg_load<ST>(v, p - sz, act, zm);
    fmg_load<ST>(r, p, act, rr);
    fmg_load<ST>(sq, p, act, qq);
    const float el = (act && x0 > 0) ? Store<ST>::load(v[p - 1]) : 0.0f;
    const float er = (act && x0 + VX < d.x) ? Store<ST>::load(v[p + VX]) : 0.0f;
    float xl, xr;
    fmg_xnb<VX>(c, el, er, lane, xl, xr);
    if (x0 + VX >= d.x) xr = er;
    float res[VX];
#pragma unroll
    for (int i = 0; i < VX; i++) {
        float s = i == VX - 1 ? xr : c[i + 1 < VX ? i + 1 : i];
        s = s + (i == 0 ? xl : c[i > 0 ? i - 1 : 0]);
        s = s + yp[i];
        s = s + ym[i];
        s = s + zp[i];
        s = s + zm[i];
        s = s - 6.0f * c[i];
        const float lap = (mu * s) / (h * h);
        res[i] = rr[i] - (lap - qq[i] * c[i]);
    }
    if (x0 == 0) res[0] = res[2];
    if (x0 + VX == d.x) res[VX - 1] = res[VX - 3];
    if (act) P::store(out + o, res);
}

// fmgResidual (kernels.cl:2008-2053), spacing 1, vectorised
template <int ST>
__global__ void __launch_bounds__(256) fmg_residual_vec_kernel(const void *F, const ST_T<ST> *f, Dim d, int comp,
                                                               float mu, ST_T<ST> *out) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    FMG_VEC_PROLOGUE(d);
    float c[VX], yp[VX], ym[VX], zp[VX], zm[VX];
    fmg_load<ST>(f, p, act, c);
    fmg_load<ST>(f, p + sy, act, yp);
    fmg_load<ST>(f, p - sy, act, ym);
    fmg_load<ST>(f, p + sz, act, zp);
    fmg_load<ST>(f, p - sz, act, zm);
    const float el = (act && x0 > 0) ? Store<ST>::load(f[p - 1]) : 0.0f;
    const float er = (act && x0 + VX < d.x) ? Store<ST>::load(f[p + VX]) : 0.0f;
    float xl, xr;
    fmg_xnb<VX>(c, el, er, lane, xl, xr);
    if (x0 + VX >= d.x) xr = er;
    float res[VX];
#pragma unroll
    for (int i = 0; i < VX; i++) {
        const float4 q = act ? Vec4Load<ST>::load(F, p + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float v0 = comp == 0 ? q.x : (comp == 1 ? q.y : q.z);
        const float sqm = (q.x * q.x + q.y * q.y) + q.z * q.z;
        float s = i == VX - 1 ? xr : c[i + 1 < VX ? i + 1 : i];
        s = s + (i == 0 ? xl : c[i > 0 ? i - 1 : 0]);
        s = s + yp[i];
        s = s + ym[i];
        s = s + zp[i];
        s = s + zm[i];
        s = s - 6.0f * c[i];
        const float rs = (mu * s) / (1.0f * 1.0f);
        res[i] = (-sqm) * v0 - (rs - sqm * c[i]);
    }
    if (x0 == 0) res[0] = res[2];
    if (x0 + VX == d.x) res[VX - 1] = res[VX - 3];
    if (act) P::store(out + o, res);
}

// prolongate (ADD, in place on v) / prolongate2, vectorised: fine x0..x0+VX-1
// take coarse x0/2 .. (x0+VX-1)/2 (0 outside the coarse image)
template <int ST, bool ADD>
__global__ void __launch_bounds__(256) prolong_vec_kernel(const ST_T<ST> *coarse, Dim fd, Dim cd, ST_T<ST> *v) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    using P = typename FmgVec<ST>::P;
    constexpr int VX = FmgVec<ST>::VX;
    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (y >= fd.y) return;
    const int x0 = (blockIdx.x * 32 + lane) * VX;
    if (x0 >= fd.x) return;
    const int64_t o = ((int64_t)z * fd.y + y) * fd.x + x0;
    float res[VX];
    if (ADD) P::unpack(P::load(v + o), res);
#pragma unroll
    for (int i = 0; i < VX; i++) {
        const float c = ld0<ST>(coarse, cd, (x0 + i) / 2, y / 2, z / 2);
        res[i] = ADD ? res[i] + c : c;
    }
    P::store(v + o, res);
}

// addTwoImages, vectorised (n a multiple of VX)
template <int ST>
__global__ void __launch_bounds__(256) add_vec_kernel(ST_T<ST> *a, const ST_T<ST> *b, int64_t nvec) {
    pdl_trigger();
    pdl_wait();   // launched with pdl_config: the previous kernel's writes are visible
    using P = typename FmgVec<ST>::P;
    constexpr int VX = FmgVec<ST>::VX;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvec) return;
    float x[VX], y[VX];
    P::unpack(P::load(a + i * VX), x);
    P::unpack(P::load(b + i * VX), y);
#pragma unroll
    for (int k = 0; k < VX; k++) x[k] = x[k] + y[k];
    P::store(a + i * VX, x);
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
constexpr int kLevels = 3;  // l_max = 2 (gradientVectorFlow.cpp:750)

struct FmgLayout {
    Dim d[kLevels];
    // per level: r, sq, v, p, tmp (level 0's r is the fmgResidual output)
    size_t r[kLevels], sq[kLevels], v[kLevels], p[kLevels], tmp[kLevels];
    size_t comp[3];
    size_t bytes;
};

static size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

static FmgLayout fmg_layout(int X, int Y, int Z, int st) {
    FmgLayout L;
    L.d[0] = Dim{X, Y, Z};
    for (int l = 1; l < kLevels; l++) L.d[l] = fmg_new_size(L.d[l - 1]);
    const size_t es = storage_bytes(st);
    size_t off = 0;
    for (int c = 0; c < 3; c++) { L.comp[c] = off; off = a256(off + es * nvox(L.d[0])); }
    for (int l = 0; l < kLevels; l++) {
        const size_t b = es * (size_t)nvox(L.d[l]);
        L.r[l] = off; off = a256(off + b);
        L.sq[l] = off; off = a256(off + b);
        L.v[l] = off; off = a256(off + b);
        L.p[l] = off; off = a256(off + b);
        L.tmp[l] = off; off = a256(off + b);
    }
    L.bytes = off;
    return L;
}

size_t fmg_workspace_size(int X, int Y, int Z, int st) { return fmg_layout(X, Y, Z, st).bytes; }

// Every level kernel is launched with programmatic dependent launch (the
// V-cycles are hundreds of small launches); each kernel waits for its
// predecessor before touching memory.
template <typename K, typename... A>
static cudaError_t fmg_launch(K kernel, dim3 grid, dim3 block, cudaStream_t s, A... args) {
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = pdl_config(grid, block, 0, s, attr);
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int ST> struct FmgRun {
    using T = ST_T<ST>;
    const FmgLayout &L;
    char *ws;
    float mu;
    cudaStream_t s;

    T *buf(size_t off) const { return reinterpret_cast<T *>(ws + off); }
    static dim3 blk() { return dim3(32, 4, 2); }
    static dim3 grd(Dim d) { return dim3((d.x + 31) / 32, (d.y + 3) / 4, (d.z + 1) / 2); }
    // vectorised kernels: rows that split into at least two vectors
    static constexpr int VX = FmgVec<ST>::VX;
    static bool vec(Dim d) { return d.x % VX == 0 && d.x >= 2 * VX; }
    static dim3 vblk() { return dim3(32, 8, 1); }
    static dim3 vgrd(Dim d) { return dim3((d.x / VX + 31) / 32, (d.y + 7) / 8, d.z); }

    int gs(int l, T *v, const T *r, float h, int iterations) {
        if (iterations <= 0) return TSF_OK;
        const Dim d = L.d[l];
        T *v2 = buf(L.tmp[l]);
        const T *sq = buf(L.sq[l]);
        const float two_mu = 2.0f * mu, twelve_mu = 12.0f * mu, hh = h * h, two_hh = (2.0f * h) * h;
        for (int i = 0; i < iterations; i++) {
            if (vec(d)) {
                TSF_TRY_CUDA(fmg_launch(gs_vec_kernel<ST, true>, vgrd(d), vblk(), s, v, v2, r, sq, d, two_mu, twelve_mu, hh, two_hh));
                TSF_TRY_CUDA(fmg_launch(gs_vec_kernel<ST, false>, vgrd(d), vblk(), s, v2, v, r, sq, d, two_mu, twelve_mu, hh, two_hh));
            } else {
                TSF_TRY_CUDA(fmg_launch(gs_kernel<ST, true>, grd(d), blk(), s, v, v2, r, sq, d, two_mu, twelve_mu, hh, two_hh));
                TSF_TRY_CUDA(fmg_launch(gs_kernel<ST, false>, grd(d), blk(), s, v2, v, r, sq, d, two_mu, twelve_mu, hh, two_hh));
            }
        }
        TSF_CHECK_LAUNCHES("gs_kernel", 2 * iterations);
        return TSF_OK;
    }

    // multigridVcycle, gradientVectorFlow.cpp:397-441; v is updated in place
    int vcycle(int l, const T *r, T *v, float h) {
        int e = gs(l, v, r, h, 2);
        if (e) return e;
        if (l < kLevels - 1) {
            const Dim d = L.d[l], nd = L.d[l + 1];
            T *p = buf(L.p[l]);
            if (vec(d)) TSF_TRY_CUDA(fmg_launch(residual_vec_kernel<ST>, vgrd(d), vblk(), s, r, v, buf(L.sq[l]), d, mu, h, p));
            else TSF_TRY_CUDA(fmg_launch(residual_kernel<ST>, grd(d), blk(), s, r, v, buf(L.sq[l]), d, mu, h, p));
            T *r1 = buf(L.r[l + 1]);
            TSF_TRY_CUDA(fmg_launch(restrict_kernel<ST>, grd(nd), blk(), s, p, d, nd, r1));
            T *v1 = buf(L.v[l + 1]);
            TSF_TRY_CUDA(cudaMemsetAsync(v1, 0, sizeof(T) * (size_t)nvox(nd), s));
            TSF_CHECK_LAUNCHES("residual/restrict", 2);
            e = vcycle(l + 1, r1, v1, h * 2.0f);
            if (e) return e;
            if (vec(d)) {
                TSF_TRY_CUDA(fmg_launch(prolong_vec_kernel<ST, true>, vgrd(d), vblk(), s, v1, d, nd, v));   // in place
                TSF_CHECK_LAUNCH("prolong_vec_kernel");
            } else {
                TSF_TRY_CUDA(fmg_launch(prolong_kernel<ST, true>, grd(d), blk(), s, v, v1, d, nd, p));
                TSF_CHECK_LAUNCH("prolong_kernel");
                TSF_TRY_CUDA(cudaMemcpyAsync(v, p, sizeof(T) * (size_t)nvox(d), cudaMemcpyDeviceToDevice, s));
            }
        }
        return gs(l, v, r, h, 2);
    }

    // fullMultigrid, gradientVectorFlow.cpp:694-727; result in buf(L.v[l])
    int full(int l, float h) {
        const Dim d = L.d[l];
        T *v = buf(L.v[l]);
        if (l < kLevels - 1) {
            const Dim nd = L.d[l + 1];
            TSF_TRY_CUDA(fmg_launch(restrict_kernel<ST>, grd(nd), blk(), s, buf(L.r[l]), d, nd, buf(L.r[l + 1])));
            TSF_CHECK_LAUNCH("restrict_kernel");
            int e = full(l + 1, h * 2.0f);
            if (e) return e;
            if (vec(d)) TSF_TRY_CUDA(fmg_launch(prolong_vec_kernel<ST, false>, vgrd(d), vblk(), s, buf(L.v[l + 1]), d, nd, v));
            else TSF_TRY_CUDA(fmg_launch(prolong_kernel<ST, false>, grd(d), blk(), s, nullptr, buf(L.v[l + 1]), d, nd, v));
            TSF_CHECK_LAUNCH("prolong_kernel");
        } else {
            TSF_TRY_CUDA(cudaMemsetAsync(v, 0, sizeof(T) * (size_t)nvox(d), s));
        }
        return vcycle(l, buf(L.r[l]), v, h);   // v0 = 1 cycle
    }

    int run(const void *F, void *out, int iterations) {
        const Dim d0 = L.d[0];
        const int64_t n0 = nvox(d0);
        TSF_TRY_CUDA(fmg_launch(sqrmag_kernel<ST>, grd(d0), blk(), s, F, d0, buf(L.sq[0])));
        for (int l = 1; l < kLevels; l++)
            TSF_TRY_CUDA(fmg_launch(restrict_kernel<ST>, grd(L.d[l]), blk(), s, buf(L.sq[l - 1]), L.d[l - 1], L.d[l], buf(L.sq[l])));
        TSF_CHECK_LAUNCHES("sqrmag/restrict", kLevels);
        const unsigned nb = (unsigned)((n0 + 255) / 256);
        for (int c = 0; c < 3; c++) {
            T *f = buf(L.comp[c]);
            TSF_TRY_CUDA(cudaMemsetAsync(f, 0, sizeof(T) * (size_t)n0, s));
            for (int it = 0; it < iterations; it++) {
                if (vec(d0)) TSF_TRY_CUDA(fmg_launch(fmg_residual_vec_kernel<ST>, vgrd(d0), vblk(), s, F, f, d0, c, mu, buf(L.r[0])));
                else TSF_TRY_CUDA(fmg_launch(fmg_residual_kernel<ST>, grd(d0), blk(), s, F, f, d0, c, mu, buf(L.r[0])));
                TSF_CHECK_LAUNCH("fmg_residual_kernel");
                int e = full(0, 1.0f);
                if (e) return e;
                if (vec(d0)) {
                    const int64_t nvec = n0 / VX;
                    TSF_TRY_CUDA(fmg_launch(add_vec_kernel<ST>, (unsigned)((nvec + 255) / 256), 256, s, f, buf(L.v[0]), nvec));
                } else {
                    TSF_TRY_CUDA(fmg_launch(add_kernel<ST>, nb, 256, s, f, buf(L.v[0]), n0));
                }
                TSF_CHECK_LAUNCH("add_kernel");
            }
        }
        TSF_TRY_CUDA(fmg_launch(fmg_finish_kernel<ST>, nb, 256, s, buf(L.comp[0]), buf(L.comp[1]), buf(L.comp[2]), out, n0));
        TSF_CHECK_LAUNCH("fmg_finish_kernel");
        return TSF_OK;
    }
};

int run_fmg(const void *f4_in, void *f4_out, int X, int Y, int Z, float mu, int iterations, int st, void *ws,
            size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!f4_in || !f4_out) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (iterations < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    const FmgLayout L = fmg_layout(X, Y, Z, st);
    for (int l = 1; l < kLevels; l++)
        if (L.d[l].x < 4) return fail(TSF_ERR_INVALID_ARG, "volume too small for three multigrid levels");
    if (!ws || ws_bytes < L.bytes) return fail(TSF_ERR_WORKSPACE, "FMG workspace too small");
    TSF_DISPATCH_STORAGE(st, ST, {
        FmgRun<ST> run{L, (char *)ws, mu, s};
        return run.run(f4_in, f4_out, iterations);
    });
    return TSF_OK;
}

}  // namespace tsf
