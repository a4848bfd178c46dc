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
#include "eigen3.cuh"
#include "tsf_common.cuh"

namespace tsf {

struct CircleTable {
    float c[32];
    float s[32];
};

// cos(j), sin(j), j = 0..31 radians, rounded to 6 significant digits: the
// sample directions of the reference (kernels.cl:1068-1069).
CircleTable host_circle_table() {
    CircleTable t;
    char buf[64];
    for (int j = 0; j < 32; j++) {
        snprintf(buf, sizeof buf, "%.6g", cos((double)j));
        t.c[j] = strtof(buf, nullptr);
        snprintf(buf, sizeof buf, "%.6g", sin((double)j));
        t.s[j] = strtof(buf, nullptr);
    }
    return t;
}

// Hessian of the field at (x,y,z): central differences of the x, y, z
// channels (reference gradient / gradientNormalized, kernels.cl:700-810),
// optionally divided by each neighbour's w.  Symmetric from the lower
// triangle (kernels.cl:1094-1098).
template <int ST, bool NORM>
__device__ __forceinline__ void hessian(const void *F, int X, int Y, int Z, int x, int y, int z, float H[3][3]) {
    const float4 xp = Vec4Load<ST>::load(F, lin(clampi(x + 1, X), y, z, X, Y));
    const float4 xm = Vec4Load<ST>::load(F, lin(clampi(x - 1, X), y, z, X, Y));
    const float4 yp = Vec4Load<ST>::load(F, lin(x, clampi(y + 1, Y), z, X, Y));
    const float4 ym = Vec4Load<ST>::load(F, lin(x, clampi(y - 1, Y), z, X, Y));
    const float4 zp = Vec4Load<ST>::load(F, lin(x, y, clampi(z + 1, Z), X, Y));
    const float4 zm = Vec4Load<ST>::load(F, lin(x, y, clampi(z - 1, Z), X, Y));
    float Fxx, Fyx, Fyy, Fzx, Fzy, Fzz;
    if (NORM) {
        Fxx = 0.5f * (xp.x / xp.w - xm.x / xm.w);
        Fyx = 0.5f * (xp.y / xp.w - xm.y / xm.w);
        Fyy = 0.5f * (yp.y / yp.w - ym.y / ym.w);
        Fzx = 0.5f * (xp.z / xp.w - xm.z / xm.w);
        Fzy = 0.5f * (yp.z / yp.w - ym.z / ym.w);
        Fzz = 0.5f * (zp.z / zp.w - zm.z / zm.w);
    } else {
        Fxx = 0.5f * (xp.x - xm.x);
        Fyx = 0.5f * (xp.y - xm.y);
        Fyy = 0.5f * (yp.y - ym.y);
        Fzx = 0.5f * (xp.z - xm.z);
        Fzy = 0.5f * (yp.z - ym.z);
        Fzz = 0.5f * (zp.z - zm.z);
    }
    H[0][0] = Fxx; H[0][1] = Fyx; H[0][2] = Fzx;
    H[1][0] = Fyx; H[1][1] = Fyy; H[1][2] = Fzy;
    H[2][0] = Fzx; H[2][1] = Fzy; H[2][2] = Fzz;
}

// OpenCL linear filter, unnormalised coordinates, clamp to edge (OpenCL 1.1
// section 8.2); weights summed in the specification's order.
template <int ST>
__device__ __forceinline__ float3 sample_linear(const void *F, int X, int Y, int Z, float u, float v, float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const int i1 = clampi(i0 + 1, X), j1 = clampi(j0 + 1, Y), k1 = clampi(k0 + 1, Z);
    i0 = clampi(i0, X); j0 = clampi(j0, Y); k0 = clampi(k0, Z);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float w000 = (ia * ib) * ic, w100 = (a * ib) * ic, w010 = (ia * b) * ic, w110 = (a * b) * ic;
    const float w001 = (ia * ib) * c, w101 = (a * ib) * c, w011 = (ia * b) * c, w111 = (a * b) * c;
    const int64_t r00 = lin(0, j0, k0, X, Y), r10 = lin(0, j1, k0, X, Y);
    const int64_t r01 = lin(0, j0, k1, X, Y), r11 = lin(0, j1, k1, X, Y);
    const float4 t000 = Vec4Load<ST>::load(F, r00 + i0), t100 = Vec4Load<ST>::load(F, r00 + i1);
    const float4 t010 = Vec4Load<ST>::load(F, r10 + i0), t110 = Vec4Load<ST>::load(F, r10 + i1);
    const float4 t001 = Vec4Load<ST>::load(F, r01 + i0), t101 = Vec4Load<ST>::load(F, r01 + i1);
    const float4 t011 = Vec4Load<ST>::load(F, r11 + i0), t111 = Vec4Load<ST>::load(F, r11 + i1);
    float3 o;
    o.x = w000 * t000.x; o.x = o.x + w100 * t100.x; o.x = o.x + w010 * t010.x; o.x = o.x + w110 * t110.x;
    o.x = o.x + w001 * t001.x; o.x = o.x + w101 * t101.x; o.x = o.x + w011 * t011.x; o.x = o.x + w111 * t111.x;
    o.y = w000 * t000.y; o.y = o.y + w100 * t100.y; o.y = o.y + w010 * t010.y; o.y = o.y + w110 * t110.y;
    o.y = o.y + w001 * t001.y; o.y = o.y + w101 * t101.y; o.y = o.y + w011 * t011.y; o.y = o.y + w111 * t111.y;
    o.z = w000 * t000.z; o.z = o.z + w100 * t100.z; o.z = o.z + w010 * t010.z; o.z = o.z + w110 * t110.z;
    o.z = o.z + w001 * t001.z; o.z = o.z + w101 * t101.z; o.z = o.z + w011 * t011.z; o.z = o.z + w111 * t111.z;
    return o;
}

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

int launch_tdf_circle(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                      void *d_T, int unorm, float *d_R, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_field4 || !d_T || !d_R) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!(rstep >= 0.0f) || !(rmin >= 0.0f)) return fail(TSF_ERR_INVALID_ARG, "invalid radius range");
    const CircleTable tab = host_circle_table();
    const dim3 b(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    const bool norm = !(rmax < 4.0f);   // kernels.cl:1083-1091
#define TSF_TDF_LAUNCH(ST, NORM, UN) \
    tdf_circle_kernel<ST, NORM, UN><<<g, b, 0, s>>>(d_field4, X, Y, Z, rmin, rmax, rstep, tab, d_T, d_R)
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
