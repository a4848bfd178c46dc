// clshim.cpp -- test infrastructure: image access of the OpenCL C shim
// (clshim.hpp), restated from the OpenCL 1.1 specification (section 8.2,
// image addressing and filtering; section 8.3, conversion rules for
// normalised integer channel types).
#include "clshim.hpp"

namespace clshim {
thread_local size_t g_id[3];
thread_local size_t g_size[3];

size_t Image::elem() const {
    switch (fmt) {
    case F32: case S32: case U32: return 4;
    case SNORM16: case UNORM16: case S16: case U16: return 2;
    default: return 1;
    }
}

float Image::readf(int64_t t, int c) const {
    const int64_t i = t * channels + c;
    switch (fmt) {
    case F32: return static_cast<const float *>(data)[i];
    case SNORM16: {
        const float v = (float)static_cast<const int16_t *>(data)[i] / 32767.0f;
        return v < -1.0f ? -1.0f : v;
    }
    case UNORM16: return (float)static_cast<const uint16_t *>(data)[i] / 65535.0f;
    default: return (float)readi(t, c);
    }
}

int64_t Image::readi(int64_t t, int c) const {
    const int64_t i = t * channels + c;
    switch (fmt) {
    case S8: return static_cast<const int8_t *>(data)[i];
    case U8: return static_cast<const uint8_t *>(data)[i];
    case S16: return static_cast<const int16_t *>(data)[i];
    case U16: return static_cast<const uint16_t *>(data)[i];
    case S32: return static_cast<const int32_t *>(data)[i];
    case U32: return static_cast<const uint32_t *>(data)[i];
    default: return (int64_t)readf(t, c);
    }
}

template <class T> static T sat(int64_t v, int64_t lo, int64_t hi) { return (T)(v < lo ? lo : (v > hi ? hi : v)); }

void Image::writef(int64_t t, int c, float v) const {
    const int64_t i = t * channels + c;
    switch (fmt) {
    case F32: static_cast<float *>(data)[i] = v; break;
    case SNORM16: static_cast<int16_t *>(data)[i] = convert_short_sat_rte(v * 32767.0f); break;
    case UNORM16: static_cast<uint16_t *>(data)[i] = convert_ushort_sat_rte(v * 65535.0f); break;
    default: writei(t, c, (int64_t)v);
    }
}

void Image::writei(int64_t t, int c, int64_t v) const {
    const int64_t i = t * channels + c;
    switch (fmt) {
    case S8: static_cast<int8_t *>(data)[i] = sat<int8_t>(v, -128, 127); break;
    case U8: static_cast<uint8_t *>(data)[i] = sat<uint8_t>(v, 0, 255); break;
    case S16: static_cast<int16_t *>(data)[i] = sat<int16_t>(v, -32768, 32767); break;
    case U16: static_cast<uint16_t *>(data)[i] = sat<uint16_t>(v, 0, 65535); break;
    case S32: static_cast<int32_t *>(data)[i] = (int32_t)v; break;
    case U32: static_cast<uint32_t *>(data)[i] = (uint32_t)v; break;
    default: writef(t, c, (float)v);
    }
}

float4 fetchf(const Image *im, int64_t t) {
    float4 r = make_vec<float4>(0.0f, 0.0f, 0.0f, 1.0f);
    for (int c = 0; c < im->channels; c++) r.v[c] = im->readf(t, c);
    return r;
}

int4 fetchi(const Image *im, int64_t t) {
    int4 r = make_vec<int4>(0, 0, 0, 1);
    for (int c = 0; c < im->channels; c++) r.v[c] = (int)im->readi(t, c);
    return r;
}

// CLK_FILTER_LINEAR, unnormalised coordinates: i0 = floor(u - 0.5),
// i1 = i0 + 1 (each through the addressing mode), a = frac(u - 0.5);
// T = (1-a)(1-b)(1-c) T000 + a(1-b)(1-c) T100 + (1-a)b(1-c) T010 + ab(1-c) T110
//   + (1-a)(1-b)c T001 + a(1-b)c T101 + (1-a)bc T011 + abc T111.
float4 linearf(const Image *im, float u, float v, float w, int s) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floor(uu), fv = floor(vv), fw = floor(ww);
    const int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float wt[8] = {(ia * ib) * ic, (a * ib) * ic, (ia * b) * ic, (a * b) * ic,
                         (ia * ib) * c,  (a * ib) * c,  (ia * b) * c,  (a * b) * c};
    float4 r = make_vec<float4>(0.0f, 0.0f, 0.0f, 0.0f);
    for (int q = 0; q < 8; q++) {
        const int64_t t = texel_at(im, i0 + (q & 1), j0 + ((q >> 1) & 1), k0 + (q >> 2), s);
        const float4 tv = t < 0 ? make_vec<float4>(0.0f, 0.0f, 0.0f, im->channels == 4 ? 0.0f : 1.0f) : fetchf(im, t);
        for (int ch = 0; ch < 4; ch++) r.v[ch] = q == 0 ? wt[q] * tv.v[ch] : r.v[ch] + wt[q] * tv.v[ch];
    }
    return r;
}
}  // namespace clshim
