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

// The sample direction a = c e3 + s e2 (per component two products and a
// sum, kernels.cl:1136), the x and y products paired.
__device__ __forceinline__ float3 circle_dir(float c, float s, float e2x, float e2y, float e2z, float e3x, float e3y,
                                             float e3z) {
    const float2 p = mul2(make_float2(c, c), make_float2(e3x, e3y));
    const float2 q = mul2(make_float2(s, s), make_float2(e2x, e2y));
    return make_float3(p.x + q.x, p.y + q.y, c * e3z + s * e2z);
}

// The sample position x + r a (kernels.cl:1137), the x and y products
// paired.
__device__ __forceinline__ float3 circle_point(float fx, float fy, float fz, float r, float3 a) {
    const float2 p = mul2(make_float2(r, r), make_float2(a.x, a.y));
    return make_float3(fx + p.x, fy + p.y, fz + r * a.z);
}

// The sample's radial term ((-g.x) a.x + (-g.y) a.y) + (-g.z) a.z
// (kernels.cl:1138-1139), the first two products paired.
__device__ __forceinline__ float radial_term(float3 g, float3 a) {
    const float2 p = mul2(make_float2(-g.x, -g.y), make_float2(a.x, a.y));
    return (p.x + p.y) + (-g.z) * a.z;
}

// The eight trilinear weights w000, w100, w010, w110, w001, w101, w011, w111
// with the specification's products ((1-a)(1-b))(1-c) ..., the products of
// the two x-neighbour weights paired (.f32x2: each rounded as alone).
__device__ __forceinline__ void tri_weights(float a, float b, float c, float w[8]) {
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float2 p0 = mul2(make_float2(ia, a), make_float2(ib, ib));
    const float2 p1 = mul2(make_float2(ia, a), make_float2(b, b));
    const float2 q0 = mul2(p0, make_float2(ic, ic)), q1 = mul2(p1, make_float2(ic, ic));
    const float2 q2 = mul2(p0, make_float2(c, c)), q3 = mul2(p1, make_float2(c, c));
    w[0] = q0.x; w[1] = q0.y; w[2] = q1.x; w[3] = q1.y;
    w[4] = q2.x; w[5] = q2.y; w[6] = q3.x; w[7] = q3.y;
}

// Sum over the eight corners of w_i * t_i for the x, y and z channels, in
// corner order: the x and y products of a corner paired, every sum one at a
// time (the assembler contracts a paired product feeding a paired sum).
__device__ __forceinline__ float3 tri_sum(const float w[8], const float4 t[8]) {
    float2 pxy[8];
    float pz[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        pxy[i] = mul2(make_float2(w[i], w[i]), make_float2(t[i].x, t[i].y));
        pz[i] = w[i] * t[i].z;
    }
    float3 o;
    o.x = pxy[0].x;
    o.y = pxy[0].y;
    o.z = pz[0];
#pragma unroll
    for (int i = 1; i < 8; i++) {
        o.x = o.x + pxy[i].x;
        o.y = o.y + pxy[i].y;
        o.z = o.z + pz[i];
    }
    return o;
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
    float wt[8];
    tri_weights(a, b, c, wt);
    const int64_t r00 = lin(0, j0, k0, X, Y), r10 = lin(0, j1, k0, X, Y);
    const int64_t r01 = lin(0, j0, k1, X, Y), r11 = lin(0, j1, k1, X, Y);
    const float4 t000 = Vec4Load<ST>::load(F, r00 + i0), t100 = Vec4Load<ST>::load(F, r00 + i1);
    const float4 t010 = Vec4Load<ST>::load(F, r10 + i0), t110 = Vec4Load<ST>::load(F, r10 + i1);
    const float4 t001 = Vec4Load<ST>::load(F, r01 + i0), t101 = Vec4Load<ST>::load(F, r01 + i1);
    const float4 t011 = Vec4Load<ST>::load(F, r11 + i0), t111 = Vec4Load<ST>::load(F, r11 + i1);
    const float4 tt[8] = {t000, t100, t010, t110, t001, t101, t011, t111};
    return tri_sum(wt, tt);
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
    float wt[8];
    tri_weights(a, b, c, wt);
    const float4 t000 = Vec4Load<ST>::load(F, base), t100 = Vec4Load<ST>::load(F, base + 1);
    const float4 t010 = Vec4Load<ST>::load(F, base + X), t110 = Vec4Load<ST>::load(F, base + X + 1);
    const float4 t001 = Vec4Load<ST>::load(F, base + XY), t101 = Vec4Load<ST>::load(F, base + XY + 1);
    const float4 t011 = Vec4Load<ST>::load(F, base + XY + X), t111 = Vec4Load<ST>::load(F, base + XY + X + 1);
    const float4 tt[8] = {t000, t100, t010, t110, t001, t101, t011, t111};
    return tri_sum(wt, tt);
}

// One field4 texel (8 bytes) of the x-paired copy to floats, the values
// Vec4Load gives for the stored texel.  snorm16: the copy holds the offset
// form (snorm16_offset2, written by the pair kernel), x and y read together.
template <int ST> __device__ __forceinline__ float4 unpack_texel(uint32_t lo, uint32_t hi) {
    using T = typename Store<ST>::T;
    if constexpr (ST == TSF_STORE_SNORM16) {
        const float2 xy = snorm16_offset_pair2(lo);
        return make_float4(xy.x, xy.y, snorm16_offset_lo(hi), snorm16_offset_lo(hi >> 16));
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
    float wt[8];
    tri_weights(a, b, c, wt);
    const uint4 p00 = __ldg(P + base), p10 = __ldg(P + base + X);
    const uint4 p01 = __ldg(P + base + XY), p11 = __ldg(P + base + XY + X);
    const float4 t000 = unpack_texel<ST>(p00.x, p00.y), t100 = unpack_texel<ST>(p00.z, p00.w);
    const float4 t010 = unpack_texel<ST>(p10.x, p10.y), t110 = unpack_texel<ST>(p10.z, p10.w);
    const float4 t001 = unpack_texel<ST>(p01.x, p01.y), t101 = unpack_texel<ST>(p01.z, p01.w);
    const float4 t011 = unpack_texel<ST>(p11.x, p11.y), t111 = unpack_texel<ST>(p11.z, p11.w);
    const float4 tt[8] = {t000, t100, t010, t110, t001, t101, t011, t111};
    return tri_sum(wt, tt);
}

// sample_linear (clamp to edge) on the x-paired copy: entry (i, j, k) holds
// texels i and min(i + 1, X - 1) of row (j, k), so with i = clamp(i0) one
// 16-byte load gives both x corners of a corner row -- except for i0 < 0, where
// both corners clamp to column 0 and the entry's first texel serves twice.
// The same texels, weights and sums, so the same bits as sample_linear
// (X * Y * Z < 2^31 for the 32-bit offsets, as for the paired copy itself).
template <int ST>
__device__ __forceinline__ float3 sample_linear_pair_clamped(const uint4 *P, int X, int Y, int Z, float u, float v,
                                                             float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    const int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const int ic = clampi(i0, X);
    const int j1 = clampi(j0 + 1, Y), k1 = clampi(k0 + 1, Z), jc = clampi(j0, Y), kc = clampi(k0, Z);
    const bool xlo = i0 < 0;
    float wt[8];
    tri_weights(a, b, c, wt);
    const uint4 p00 = __ldg(P + ic + X * (jc + Y * kc)), p10 = __ldg(P + ic + X * (j1 + Y * kc));
    const uint4 p01 = __ldg(P + ic + X * (jc + Y * k1)), p11 = __ldg(P + ic + X * (j1 + Y * k1));
    const float4 t000 = unpack_texel<ST>(p00.x, p00.y), t010 = unpack_texel<ST>(p10.x, p10.y);
    const float4 t001 = unpack_texel<ST>(p01.x, p01.y), t011 = unpack_texel<ST>(p11.x, p11.y);
    const float4 t100 = xlo ? t000 : unpack_texel<ST>(p00.z, p00.w), t110 = xlo ? t010 : unpack_texel<ST>(p10.z, p10.w);
    const float4 t101 = xlo ? t001 : unpack_texel<ST>(p01.z, p01.w), t111 = xlo ? t011 : unpack_texel<ST>(p11.z, p11.w);
    const float4 tt[8] = {t000, t100, t010, t110, t001, t101, t011, t111};
    return tri_sum(wt, tt);
}

// Margin m such that every trilinear corner of a sample at distance <= r
// from a voxel lies within m - 1 voxels of it, for sample directions
// a = cos e3 + sin e2 with |e2|, |e3| <= 1.00005 and |e2 . e3| <= 1e-3
// (then |a| <= 1.0012; corners lie within ceil(|a| r + 0.5) of the voxel).
__host__ __device__ __forceinline__ int sample_margin(float rmax) { return (int)ceilf(rmax * 1.002f + 0.5f) + 2; }

// Room for the unclamped sampler around a voxel: its distance to the nearest
// face (capped at 255), or 0 when the eigenvectors are not finite, unit and
// orthogonal up to rounding.  The samples at radius r may take
// sample_linear_in when sample_margin(r) <= this value (the margin box of
// samples_inside, checked per radius instead of for rmax).
__device__ __forceinline__ unsigned char sample_room(int x, int y, int z, int X, int Y, int Z, const float e2[3],
                                                     const float e3[3]) {
    const float n2 = (e2[0] * e2[0] + e2[1] * e2[1]) + e2[2] * e2[2];
    const float n3 = (e3[0] * e3[0] + e3[1] * e3[1]) + e3[2] * e3[2];
    const float d = (e2[0] * e3[0] + e2[1] * e3[1]) + e2[2] * e3[2];
    if (!(n2 <= 1.0001f && n3 <= 1.0001f && d >= -1e-3f && d <= 1e-3f)) return 0;
    const int m = min(min(min(x, y), z), min(min(X - 1 - x, Y - 1 - y), Z - 1 - z));
    return (unsigned char)max(0, min(m, 255));
}

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
