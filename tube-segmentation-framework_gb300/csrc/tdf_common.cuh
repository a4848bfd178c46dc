// tdf_common.cuh -- device pieces of the circle-fitting TDF shared by the
// forward kernel (tdf.cu) and its reverse-mode derivative (tdf_adjoint.cu):
// the sample-direction table, the Hessian of the field and the OpenCL linear
// sampler (reference kernels.cl:700-810, 1065-1157).
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "eigen3.cuh"
#include "tsf_common.cuh"

namespace tsf {

struct CircleTable {
    float c[32];
    float s[32];
    int n;      // samples per radius
};

// cos(j), sin(j), j = 0..31 radians, rounded to 6 significant digits: the
// sample directions of the reference (kernels.cl:1068-1069).  With fewer
// samples, entry j holds table entry j * stride (the reference's disabled
// sample-count switch, kernels.cl:1120-1131, takes its samples that way).
inline CircleTable host_circle_table(int samples = 32, int stride = 1) {
    CircleTable t;
    char buf[64];
    for (int j = 0; j < 32; j++) {
        const int q = j < samples ? j * stride : 0;
        snprintf(buf, sizeof buf, "%.6g", cos((double)q));
        t.c[j] = strtof(buf, nullptr);
        snprintf(buf, sizeof buf, "%.6g", sin((double)q));
        t.s[j] = strtof(buf, nullptr);
    }
    t.n = samples;
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

// sample_linear for a point whose 8 corners are all inside the volume (the
// caller guarantees it): the clamps are no-ops there and are skipped, and the
// corners are addressed from one 32-bit base (X*Y*Z < 2^31).  Same weights
// and the same sums in the same order, so the same bits as sample_linear.
template <int ST>
__device__ __forceinline__ float3 sample_linear_in(const void *F, int X, int XY, float u, float v, float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    const int base = (int)fu + X * (int)fv + XY * (int)fw;
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float w000 = (ia * ib) * ic, w100 = (a * ib) * ic, w010 = (ia * b) * ic, w110 = (a * b) * ic;
    const float w001 = (ia * ib) * c, w101 = (a * ib) * c, w011 = (ia * b) * c, w111 = (a * b) * c;
    const float4 t000 = Vec4Load<ST>::load(F, base), t100 = Vec4Load<ST>::load(F, base + 1);
    const float4 t010 = Vec4Load<ST>::load(F, base + X), t110 = Vec4Load<ST>::load(F, base + X + 1);
    const float4 t001 = Vec4Load<ST>::load(F, base + XY), t101 = Vec4Load<ST>::load(F, base + XY + 1);
    const float4 t011 = Vec4Load<ST>::load(F, base + XY + X), t111 = Vec4Load<ST>::load(F, base + XY + X + 1);
    float3 o;
    o.x = w000 * t000.x; o.x = o.x + w100 * t100.x; o.x = o.x + w010 * t010.x; o.x = o.x + w110 * t110.x;
    o.x = o.x + w001 * t001.x; o.x = o.x + w101 * t101.x; o.x = o.x + w011 * t011.x; o.x = o.x + w111 * t111.x;
    o.y = w000 * t000.y; o.y = o.y + w100 * t100.y; o.y = o.y + w010 * t010.y; o.y = o.y + w110 * t110.y;
    o.y = o.y + w001 * t001.y; o.y = o.y + w101 * t101.y; o.y = o.y + w011 * t011.y; o.y = o.y + w111 * t111.y;
    o.z = w000 * t000.z; o.z = o.z + w100 * t100.z; o.z = o.z + w010 * t010.z; o.z = o.z + w110 * t110.z;
    o.z = o.z + w001 * t001.z; o.z = o.z + w101 * t101.z; o.z = o.z + w011 * t011.z; o.z = o.z + w111 * t111.z;
    return o;
}

// One stored 16-bit field4 texel (8 bytes) to floats, as Vec4Load does
// (snorm16: x and y read together, snorm16_pair2, the same bits).
template <int ST> __device__ __forceinline__ float4 unpack_texel(uint32_t lo, uint32_t hi) {
    using T = typename Store<ST>::T;
    if constexpr (ST == TSF_STORE_SNORM16) {
        const float2 xy = snorm16_pair2(lo);
        return make_float4(xy.x, xy.y, snorm16_from_bits(hi), snorm16_from_bits(hi >> 16));
    } else {
        const uint2 raw = make_uint2(lo, hi);
        T c[4];
        memcpy(c, &raw, 8);
        return make_float4(Store<ST>::load(c[0]), Store<ST>::load(c[1]), Store<ST>::load(c[2]), Store<ST>::load(c[3]));
    }
}

// sample_linear_in on the x-paired copy of a 16-bit field: entry i holds
// texel i and texel i + 1 (16 bytes), so each of the four (y, z) corner rows
// is one 16-byte load instead of two 8-byte loads.  Same texels, weights and
// sums in the same order, so the same bits as sample_linear_in.
template <int ST>
__device__ __forceinline__ float3 sample_linear_pair_in(const uint4 *P, int X, int XY, float u, float v, float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    const int base = (int)fu + X * (int)fv + XY * (int)fw;
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float w000 = (ia * ib) * ic, w100 = (a * ib) * ic, w010 = (ia * b) * ic, w110 = (a * b) * ic;
    const float w001 = (ia * ib) * c, w101 = (a * ib) * c, w011 = (ia * b) * c, w111 = (a * b) * c;
    const uint4 p00 = __ldg(P + base), p10 = __ldg(P + base + X);
    const uint4 p01 = __ldg(P + base + XY), p11 = __ldg(P + base + XY + X);
    const float4 t000 = unpack_texel<ST>(p00.x, p00.y), t100 = unpack_texel<ST>(p00.z, p00.w);
    const float4 t010 = unpack_texel<ST>(p10.x, p10.y), t110 = unpack_texel<ST>(p10.z, p10.w);
    const float4 t001 = unpack_texel<ST>(p01.x, p01.y), t101 = unpack_texel<ST>(p01.z, p01.w);
    const float4 t011 = unpack_texel<ST>(p11.x, p11.y), t111 = unpack_texel<ST>(p11.z, p11.w);
    float3 o;
    o.x = w000 * t000.x; o.x = o.x + w100 * t100.x; o.x = o.x + w010 * t010.x; o.x = o.x + w110 * t110.x;
    o.x = o.x + w001 * t001.x; o.x = o.x + w101 * t101.x; o.x = o.x + w011 * t011.x; o.x = o.x + w111 * t111.x;
    o.y = w000 * t000.y; o.y = o.y + w100 * t100.y; o.y = o.y + w010 * t010.y; o.y = o.y + w110 * t110.y;
    o.y = o.y + w001 * t001.y; o.y = o.y + w101 * t101.y; o.y = o.y + w011 * t011.y; o.y = o.y + w111 * t111.y;
    o.z = w000 * t000.z; o.z = o.z + w100 * t100.z; o.z = o.z + w010 * t010.z; o.z = o.z + w110 * t110.z;
    o.z = o.z + w001 * t001.z; o.z = o.z + w101 * t101.z; o.z = o.z + w011 * t011.z; o.z = o.z + w111 * t111.z;
    return o;
}

// Margin m such that every trilinear corner of a sample at distance <= r
// from a voxel lies within m - 1 voxels of it, for sample directions
// a = cos e3 + sin e2 with |e2|, |e3| <= 1.00005 and |e2 . e3| <= 1e-3
// (then |a| <= 1.0012; corners lie within ceil(|a| r + 0.5) of the voxel).
__host__ __device__ __forceinline__ int sample_margin(float rmax) { return (int)ceilf(rmax * 1.002f + 0.5f) + 2; }

// Whether a voxel's samples can take sample_linear_in: the margin box lies in
// the volume and the eigenvectors are finite, unit and orthogonal up to
// rounding (false for NaN / inf, which then take the clamped sampler).
__device__ __forceinline__ bool samples_inside(int x, int y, int z, int X, int Y, int Z, int m, const float e2[3],
                                               const float e3[3]) {
    if (x < m || y < m || z < m || x + m >= X || y + m >= Y || z + m >= Z) return false;
    const float n2 = (e2[0] * e2[0] + e2[1] * e2[1]) + e2[2] * e2[2];
    const float n3 = (e3[0] * e3[0] + e3[1] * e3[1]) + e3[2] * e3[2];
    const float d = (e2[0] * e3[0] + e2[1] * e3[1]) + e2[2] * e3[2];
    return n2 <= 1.0001f && n3 <= 1.0001f && d >= -1e-3f && d <= 1e-3f;
}

}  // namespace tsf
