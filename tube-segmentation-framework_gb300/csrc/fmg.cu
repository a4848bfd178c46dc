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
#include "tsf_common.cuh"

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
    FMG_THREAD_XYZ(d);
    const int64_t i = lin(x, y, z, d.x, d.y);
    const float4 q = Vec4Load<ST>::load(F, i);
    sq[i] = Store<ST>::store((q.x * q.x + q.y * q.y) + q.z * q.z);
}

// fmgResidual (kernels.cl:2008-2053), spacing 1
template <int ST>
__global__ void fmg_residual_kernel(const void *F, const ST_T<ST> *f, Dim d, int comp, float mu, ST_T<ST> *out) {
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
    FMG_THREAD_XYZ(fd);
    const float c = ld0<ST>(coarse, cd, x / 2, y / 2, z / 2);
    const int64_t i = lin(x, y, z, fd.x, fd.y);
    const float value = ADD ? Store<ST>::load(fine_in[i]) + c : c;
    out[i] = Store<ST>::store(value);
}

// addTwoImages (kernels.cl:1857-1865), in place on a
template <int ST>
__global__ void add_kernel(ST_T<ST> *a, const ST_T<ST> *b, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = Store<ST>::store(Store<ST>::load(a[i]) + Store<ST>::load(b[i]));
}

// MGGVFFinish (kernels.cl:1907-1921): w = |v| (no special case for 0)
template <int ST>
__global__ void fmg_finish_kernel(const ST_T<ST> *fx, const ST_T<ST> *fy, const ST_T<ST> *fz, void *out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = Store<ST>::load(fx[i]), y = Store<ST>::load(fy[i]), z = Store<ST>::load(fz[i]);
    store4<ST>(out, i, x, y, z, sqrtf((x * x + y * y) + z * z));
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

template <int ST> struct FmgRun {
    using T = ST_T<ST>;
    const FmgLayout &L;
    char *ws;
    float mu;
    cudaStream_t s;

    T *buf(size_t off) const { return reinterpret_cast<T *>(ws + off); }
    static dim3 blk() { return dim3(32, 4, 2); }
    static dim3 grd(Dim d) { return dim3((d.x + 31) / 32, (d.y + 3) / 4, (d.z + 1) / 2); }

    int gs(int l, T *v, const T *r, float h, int iterations) {
        if (iterations <= 0) return TSF_OK;
        const Dim d = L.d[l];
        T *v2 = buf(L.tmp[l]);
        const T *sq = buf(L.sq[l]);
        const float two_mu = 2.0f * mu, twelve_mu = 12.0f * mu, hh = h * h, two_hh = (2.0f * h) * h;
        for (int i = 0; i < iterations; i++) {
            gs_kernel<ST, true><<<grd(d), blk(), 0, s>>>(v, v2, r, sq, d, two_mu, twelve_mu, hh, two_hh);
            gs_kernel<ST, false><<<grd(d), blk(), 0, s>>>(v2, v, r, sq, d, two_mu, twelve_mu, hh, two_hh);
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
            residual_kernel<ST><<<grd(d), blk(), 0, s>>>(r, v, buf(L.sq[l]), d, mu, h, p);
            T *r1 = buf(L.r[l + 1]);
            restrict_kernel<ST><<<grd(nd), blk(), 0, s>>>(p, d, nd, r1);
            T *v1 = buf(L.v[l + 1]);
            TSF_TRY_CUDA(cudaMemsetAsync(v1, 0, sizeof(T) * (size_t)nvox(nd), s));
            TSF_CHECK_LAUNCHES("residual/restrict", 2);
            e = vcycle(l + 1, r1, v1, h * 2.0f);
            if (e) return e;
            prolong_kernel<ST, true><<<grd(d), blk(), 0, s>>>(v, v1, d, nd, p);
            TSF_CHECK_LAUNCH("prolong_kernel");
            TSF_TRY_CUDA(cudaMemcpyAsync(v, p, sizeof(T) * (size_t)nvox(d), cudaMemcpyDeviceToDevice, s));
        }
        return gs(l, v, r, h, 2);
    }

    // fullMultigrid, gradientVectorFlow.cpp:694-727; result in buf(L.v[l])
    int full(int l, float h) {
        const Dim d = L.d[l];
        T *v = buf(L.v[l]);
        if (l < kLevels - 1) {
            const Dim nd = L.d[l + 1];
            restrict_kernel<ST><<<grd(nd), blk(), 0, s>>>(buf(L.r[l]), d, nd, buf(L.r[l + 1]));
            TSF_CHECK_LAUNCH("restrict_kernel");
            int e = full(l + 1, h * 2.0f);
            if (e) return e;
            prolong_kernel<ST, false><<<grd(d), blk(), 0, s>>>(nullptr, buf(L.v[l + 1]), d, nd, v);
            TSF_CHECK_LAUNCH("prolong_kernel");
        } else {
            TSF_TRY_CUDA(cudaMemsetAsync(v, 0, sizeof(T) * (size_t)nvox(d), s));
        }
        return vcycle(l, buf(L.r[l]), v, h);   // v0 = 1 cycle
    }

    int run(const void *F, void *out, int iterations) {
        const Dim d0 = L.d[0];
        const int64_t n0 = nvox(d0);
        sqrmag_kernel<ST><<<grd(d0), blk(), 0, s>>>(F, d0, buf(L.sq[0]));
        for (int l = 1; l < kLevels; l++)
            restrict_kernel<ST><<<grd(L.d[l]), blk(), 0, s>>>(buf(L.sq[l - 1]), L.d[l - 1], L.d[l], buf(L.sq[l]));
        TSF_CHECK_LAUNCHES("sqrmag/restrict", kLevels);
        const unsigned nb = (unsigned)((n0 + 255) / 256);
        for (int c = 0; c < 3; c++) {
            T *f = buf(L.comp[c]);
            TSF_TRY_CUDA(cudaMemsetAsync(f, 0, sizeof(T) * (size_t)n0, s));
            for (int it = 0; it < iterations; it++) {
                fmg_residual_kernel<ST><<<grd(d0), blk(), 0, s>>>(F, f, d0, c, mu, buf(L.r[0]));
                TSF_CHECK_LAUNCH("fmg_residual_kernel");
                int e = full(0, 1.0f);
                if (e) return e;
                add_kernel<ST><<<nb, 256, 0, s>>>(f, buf(L.v[0]), n0);
                TSF_CHECK_LAUNCH("add_kernel");
            }
        }
        fmg_finish_kernel<ST><<<nb, 256, 0, s>>>(buf(L.comp[0]), buf(L.comp[1]), buf(L.comp[2]), out, n0);
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
