// clshim.hpp -- test infrastructure, not part of the product.
//
// The subset of OpenCL C 1.1 that the reference's kernel source (kernels.cl)
// uses, as a C++17 header, so that the reference's own kernel text compiles
// unmodified on the CPU (after one mechanical rewrite of vector literals, see
// make_ref.py) and can be run against the oracle:
//   * vector types charN/intN/floatN (N = 2, 3, 4, 8) with the component
//     names and swizzles the source uses, component-wise arithmetic with
//     scalar widening, comparisons that yield -1 / 0 masks, select();
//   * the geometric, math and conversion built-ins the source calls;
//   * images and samplers: read_image{f,i,ui} with nearest / linear filtering
//     and clamp-to-edge / clamp (border 0) addressing on unnormalised
//     coordinates, write_image{f,i,ui} with the channel-format conversions
//     (FLOAT, SNORM_INT16, UNORM_INT16, integer formats) -- restated from the
//     OpenCL 1.1 specification, sections 6.11.13 and 8.2-8.3;
//   * work-item functions backed by per-thread state, set by the launcher.
// Arithmetic follows the source's expression order; build with
// -ffp-contract=off so that no product is fused into an add.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

#define __kernel
#define __global
#define __local
#define __private
#define __constant const
#define __read_only
#define __write_only
#define restrict __restrict__

// ---------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------
template <class T, int N> struct vec;

// A swizzle view: the parent's storage, read as the components I...
template <class T, int N, int... I> struct swz {
    T d[N];
    static constexpr int M = sizeof...(I);
    operator vec<T, M>() const;
    template <class O> swz &operator=(const O &o);
    template <class O> swz &operator+=(const O &o);
    template <class O> swz &operator-=(const O &o);
    template <class O> swz &operator*=(const O &o);
    template <class O> swz &operator/=(const O &o);
};

// component k of a vector-like value, or the scalar itself, as type E
template <class E, class X> inline E comp(const X &x, int k);

#define CLSHIM_VEC_OPS(N_)                                                                   \
    T &operator[](int i) { return v[i]; }                                                    \
    const T &operator[](int i) const { return v[i]; }                                        \
    template <class O> vec &operator+=(const O &o) {                                         \
        for (int k = 0; k < N_; k++) v[k] = v[k] + comp<T>(o, k);                            \
        return *this;                                                                        \
    }                                                                                        \
    template <class O> vec &operator-=(const O &o) {                                         \
        for (int k = 0; k < N_; k++) v[k] = v[k] - comp<T>(o, k);                            \
        return *this;                                                                        \
    }                                                                                        \
    template <class O> vec &operator*=(const O &o) {                                         \
        for (int k = 0; k < N_; k++) v[k] = v[k] * comp<T>(o, k);                            \
        return *this;                                                                        \
    }                                                                                        \
    template <class O> vec &operator/=(const O &o) {                                         \
        for (int k = 0; k < N_; k++) v[k] = v[k] / comp<T>(o, k);                            \
        return *this;                                                                        \
    }

template <class T> struct vec<T, 2> {
    union {
        T v[2];
        struct { T x, y; };
        struct { T s0, s1; };
    };
    CLSHIM_VEC_OPS(2)
};

template <class T> struct vec<T, 3> {
    union {
        T v[3];
        struct { T x, y, z; };
        struct { T s0, s1, s2; };
        swz<T, 3, 0, 1> xy;
        swz<T, 3, 0, 1, 2> xyz;
        swz<T, 3, 0, 1, 2, 2> xyzz;
    };
    CLSHIM_VEC_OPS(3)
};

template <class T> struct vec<T, 4> {
    union {
        T v[4];
        struct { T x, y, z, w; };
        struct { T s0, s1, s2, s3; };
        swz<T, 4, 0, 1> xy;
        swz<T, 4, 0, 1, 2> xyz;
        swz<T, 4, 0, 1, 2, 2> xyzz;
    };
    CLSHIM_VEC_OPS(4)
};

template <class T> struct vec<T, 8> {
    union {
        T v[8];
        struct { T s0, s1, s2, s3, s4, s5, s6, s7; };
    };
    CLSHIM_VEC_OPS(8)
};

typedef vec<char, 2> char2;
typedef vec<char, 4> char4;
typedef vec<int, 2> int2;
typedef vec<int, 3> int3;
typedef vec<int, 4> int4;
typedef vec<int, 8> int8;
typedef vec<uint, 4> uint4;
typedef vec<float, 2> float2;
typedef vec<float, 3> float3;
typedef vec<float, 4> float4;

template <class X> struct vtraits {
    static constexpr bool is = false;
    using elem = X;
    static constexpr int n = 1;
};
template <class T, int N> struct vtraits<vec<T, N>> {
    static constexpr bool is = true;
    using elem = T;
    static constexpr int n = N;
    static vec<T, N> get(const vec<T, N> &a) { return a; }
};
template <class T, int N, int... I> struct vtraits<swz<T, N, I...>> {
    static constexpr bool is = true;
    using elem = T;
    static constexpr int n = sizeof...(I);
    static vec<T, sizeof...(I)> get(const swz<T, N, I...> &a) { return a; }
};

template <class T, int N, int... I> swz<T, N, I...>::operator vec<T, M>() const {
    vec<T, M> r;
    int k = 0;
    ((r.v[k++] = d[I]), ...);
    return r;
}

template <class E, class X> inline E comp(const X &x, int k) {
    if constexpr (vtraits<X>::is) return (E)vtraits<X>::get(x).v[k];
    else return (E)x;
}

template <class A, class B> struct binres {
    static constexpr bool va = vtraits<A>::is, vb = vtraits<B>::is;
    using E = typename std::conditional<va, vtraits<A>, vtraits<B>>::type::elem;
    static constexpr int n = va ? vtraits<A>::n : vtraits<B>::n;
    using type = vec<E, n>;
};

#define CLSHIM_BINOP(OP)                                                                           \
    template <class A, class B, class = typename std::enable_if<vtraits<A>::is || vtraits<B>::is>::type> \
    inline typename binres<A, B>::type operator OP(const A &a, const B &b) {                      \
        using R = binres<A, B>;                                                                    \
        typename R::type r;                                                                        \
        for (int k = 0; k < R::n; k++) r.v[k] = comp<typename R::E>(a, k) OP comp<typename R::E>(b, k); \
        return r;                                                                                  \
    }
CLSHIM_BINOP(+)
CLSHIM_BINOP(-)
CLSHIM_BINOP(*)
CLSHIM_BINOP(/)
#undef CLSHIM_BINOP

// comparisons: -1 where true, 0 where false (OpenCL 1.1 section 6.3.d)
#define CLSHIM_CMPOP(OP)                                                                           \
    template <class A, class B, class = typename std::enable_if<vtraits<A>::is || vtraits<B>::is>::type> \
    inline vec<int, binres<A, B>::n> operator OP(const A &a, const B &b) {                        \
        using R = binres<A, B>;                                                                    \
        vec<int, R::n> r;                                                                          \
        for (int k = 0; k < R::n; k++)                                                             \
            r.v[k] = (comp<typename R::E>(a, k) OP comp<typename R::E>(b, k)) ? -1 : 0;            \
        return r;                                                                                  \
    }
CLSHIM_CMPOP(==)
CLSHIM_CMPOP(!=)
CLSHIM_CMPOP(<)
CLSHIM_CMPOP(<=)
CLSHIM_CMPOP(>)
CLSHIM_CMPOP(>=)
#undef CLSHIM_CMPOP

template <class T, int N> inline vec<T, N> operator-(const vec<T, N> &a) {
    vec<T, N> r;
    for (int k = 0; k < N; k++) r.v[k] = -a.v[k];
    return r;
}
template <class T, int N, int... I> inline vec<T, sizeof...(I)> operator-(const swz<T, N, I...> &a) {
    return -vec<T, sizeof...(I)>(a);
}

#define CLSHIM_ASSIGNOP(OP)                                                              \
    template <class T, int N, int... I> template <class O>                               \
    swz<T, N, I...> &swz<T, N, I...>::operator OP##=(const O &o) {                       \
        int k = 0;                                                                       \
        ((d[I] = d[I] OP comp<T>(o, k++)), ...);                                         \
        return *this;                                                                    \
    }
CLSHIM_ASSIGNOP(+)
CLSHIM_ASSIGNOP(-)
CLSHIM_ASSIGNOP(*)
CLSHIM_ASSIGNOP(/)
#undef CLSHIM_ASSIGNOP

template <class T, int N, int... I> template <class O> swz<T, N, I...> &swz<T, N, I...>::operator=(const O &o) {
    const vec<T, M> t = [&] {
        vec<T, M> r;
        for (int k = 0; k < M; k++) r.v[k] = comp<T>(o, k);
        return r;
    }();
    int k = 0;
    ((d[I] = t.v[k++]), ...);
    return *this;
}

// Vector literals (T)(a, b, ...): the arguments' components in order; one
// scalar argument is replicated (OpenCL 1.1 section 6.1.6).
template <class V, class... A> inline V make_vec(const A &...a) {
    using E = typename vtraits<V>::elem;
    constexpr int N = vtraits<V>::n;
    V r;
    int k = 0;
    auto put = [&](const auto &x) {
        using X = typename std::decay<decltype(x)>::type;
        if constexpr (vtraits<X>::is) {
            const auto t = vtraits<X>::get(x);
            for (int i = 0; i < vtraits<X>::n; i++) r.v[k++] = (E)t.v[i];
        } else {
            r.v[k++] = (E)x;
        }
    };
    (put(a), ...);
    if (sizeof...(A) == 1 && k == 1)
        for (int i = 1; i < N; i++) r.v[i] = r.v[0];
    return r;
}

// select(a, b, c): b where the most significant bit of c is set, else a
template <class A, class B, class Cm> inline auto select(const A &a, const B &b, const Cm &c) {
    auto va = vtraits<A>::get(a);
    using V = decltype(va);
    V r;
    for (int k = 0; k < vtraits<V>::n; k++) r.v[k] = comp<int>(c, k) < 0 ? comp<typename vtraits<V>::elem>(b, k) : va.v[k];
    return r;
}

// ---------------------------------------------------------------------------
// math and geometric built-ins (single precision)
// ---------------------------------------------------------------------------
#define M_PI_F 3.14159265358979323846f
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float fabs(float x) { return __builtin_fabsf(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float ceil(float x) { return __builtin_ceilf(x); }
inline float round(float x) { return __builtin_roundf(x); }   // halfway cases away from zero
inline float acos(float x) { return __builtin_acosf(x); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float sin(float x) { return __builtin_sinf(x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float native_divide(float a, float b) { return a / b; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }

template <class A, class B> inline float dot(const A &a, const B &b) {
    constexpr int N = vtraits<A>::n;
    float s = comp<float>(a, 0) * comp<float>(b, 0);
    for (int k = 1; k < N; k++) s = s + comp<float>(a, k) * comp<float>(b, k);
    return s;
}
template <class A> inline float length(const A &a) { return sqrt(dot(a, a)); }
template <class A, class B> inline float distance(const A &a, const B &b) { return length(a - b); }
template <class A> inline auto normalize(const A &a) { return vtraits<A>::get(a) / length(a); }
template <class T, int N> inline vec<T, N> floor(const vec<T, N> &a) {
    vec<T, N> r;
    for (int k = 0; k < N; k++) r.v[k] = floor(a.v[k]);
    return r;
}
template <class T, int N> inline vec<T, N> round(const vec<T, N> &a) {
    vec<T, N> r;
    for (int k = 0; k < N; k++) r.v[k] = round(a.v[k]);
    return r;
}
template <class T, int N> inline vec<T, N> fabs(const vec<T, N> &a) {
    vec<T, N> r;
    for (int k = 0; k < N; k++) r.v[k] = fabs(a.v[k]);
    return r;
}

// conversions: convert_T (round toward zero for float -> int, as C casts)
#define CLSHIM_CONVERT(NAME, E, N)                                         \
    template <class A> inline vec<E, N> NAME(const A &a) {                 \
        vec<E, N> r;                                                       \
        for (int k = 0; k < N; k++) r.v[k] = (E)comp<double>(a, k);        \
        return r;                                                          \
    }
CLSHIM_CONVERT(convert_float3, float, 3)
CLSHIM_CONVERT(convert_float4, float, 4)
CLSHIM_CONVERT(convert_int3, int, 3)
CLSHIM_CONVERT(convert_int4, int, 4)
#undef CLSHIM_CONVERT

// convert_ushort_sat_rte: round to nearest even, saturate to [0, 65535]
inline ushort convert_ushort_sat_rte(float v) {
    if (!(v > 0.0f)) return 0;           // negative and NaN -> 0
    if (v >= 65535.0f) return 65535;
    return (ushort)__builtin_rintf(v);   // default rounding mode: to nearest even
}
inline short convert_short_sat_rte(float v) {
    if (v != v) return 0;
    if (v <= -32768.0f) return -32768;
    if (v >= 32767.0f) return 32767;
    return (short)__builtin_rintf(v);
}

// vloadN / vstoreN: element offset i * N
template <class P> inline auto vload2(size_t i, const P *p) { return make_vec<vec<P, 2>>(p[2 * i], p[2 * i + 1]); }
template <class P> inline auto vload3(size_t i, const P *p) {
    return make_vec<vec<P, 3>>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
template <class A, class P> inline void vstore2(const A &a, size_t i, P *p) {
    for (int k = 0; k < 2; k++) p[2 * i + k] = comp<P>(a, k);
}
template <class A, class P> inline void vstore3(const A &a, size_t i, P *p) {
    for (int k = 0; k < 3; k++) p[3 * i + k] = comp<P>(a, k);
}
template <class A, class P> inline void vstore4(const A &a, size_t i, P *p) {
    for (int k = 0; k < 4; k++) p[4 * i + k] = comp<P>(a, k);
}

// atomics (the launcher runs work-items of one launch on several threads)
inline int atomic_inc(volatile int *p) { return __atomic_fetch_add(p, 1, __ATOMIC_SEQ_CST); }
inline int atomic_min(volatile int *p, int v) {
    int old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
    while (v < old && !__atomic_compare_exchange_n(p, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
    }
    return old;
}

// ---------------------------------------------------------------------------
// work-items
// ---------------------------------------------------------------------------
namespace clshim {
extern thread_local size_t g_id[3];
extern thread_local size_t g_size[3];
}  // namespace clshim
inline size_t get_global_id(int d) { return clshim::g_id[d]; }
inline size_t get_global_size(int d) { return clshim::g_size[d]; }

// ---------------------------------------------------------------------------
// images and samplers
// ---------------------------------------------------------------------------
enum {
    CLK_NORMALIZED_COORDS_FALSE = 0,
    CLK_ADDRESS_CLAMP_TO_EDGE = 2,
    CLK_ADDRESS_CLAMP = 4,
    CLK_FILTER_NEAREST = 0x10,
    CLK_FILTER_LINEAR = 0x20
};
typedef int sampler_t;

namespace clshim {
// channel data types of the images the reference creates
enum Format { F32, SNORM16, UNORM16, S8, U8, S16, U16, S32, U32 };

struct Image {
    int w = 1, h = 1, d = 1;
    int channels = 1;   // 1 (R), 2 (RG) or 4 (RGBA)
    Format fmt = F32;
    void *data = nullptr;
    size_t elem() const;
    float readf(int64_t texel, int c) const;          // normalised / float formats
    int64_t readi(int64_t texel, int c) const;        // integer formats
    void writef(int64_t texel, int c, float v) const;
    void writei(int64_t texel, int c, int64_t v) const;
};
}  // namespace clshim

typedef clshim::Image *image3d_t;
typedef clshim::Image *image2d_t;

namespace clshim {
// texel index of integer coordinates under the sampler's addressing; -1 = border
inline int64_t texel_at(const Image *im, int x, int y, int z, int s) {
    if (s & CLK_ADDRESS_CLAMP) {
        if (x < 0 || y < 0 || z < 0 || x >= im->w || y >= im->h || z >= im->d) return -1;
    } else {
        x = x < 0 ? 0 : (x >= im->w ? im->w - 1 : x);
        y = y < 0 ? 0 : (y >= im->h ? im->h - 1 : y);
        z = z < 0 ? 0 : (z >= im->d ? im->d - 1 : z);
    }
    return (int64_t)x + (int64_t)im->w * ((int64_t)y + (int64_t)im->h * z);
}
float4 fetchf(const Image *im, int64_t t);   // (r, g, b, a) with missing channels (0, 0, 1)
int4 fetchi(const Image *im, int64_t t);
// linear filter, unnormalised coordinates (OpenCL 1.1 section 8.2)
float4 linearf(const Image *im, float u, float v, float w, int s);
}  // namespace clshim

template <class C> inline float4 read_imagef(image3d_t im, sampler_t s, const C &c) {
    using namespace clshim;
    const bool fl = std::is_same<typename vtraits<C>::elem, float>::value;
    if (fl && (s & CLK_FILTER_LINEAR)) return linearf(im, comp<float>(c, 0), comp<float>(c, 1), comp<float>(c, 2), s);
    int x, y, z;
    if (fl) {
        x = (int)floor(comp<float>(c, 0));
        y = (int)floor(comp<float>(c, 1));
        z = vtraits<C>::n > 2 ? (int)floor(comp<float>(c, 2)) : 0;
    } else {
        x = comp<int>(c, 0);
        y = comp<int>(c, 1);
        z = vtraits<C>::n > 2 ? comp<int>(c, 2) : 0;
    }
    const int64_t t = texel_at(im, x, y, z, s);
    if (t < 0) return make_vec<float4>(0.0f, 0.0f, 0.0f, im->channels == 4 ? 0.0f : 1.0f);
    return fetchf(im, t);
}
template <class C> inline int4 read_imagei(image3d_t im, sampler_t s, const C &c) {
    using namespace clshim;
    const int z = vtraits<C>::n > 2 ? comp<int>(c, 2) : 0;
    const int64_t t = texel_at(im, comp<int>(c, 0), comp<int>(c, 1), z, s);
    if (t < 0) return make_vec<int4>(0, 0, 0, im->channels == 4 ? 0 : 1);
    return fetchi(im, t);
}
template <class C> inline uint4 read_imageui(image3d_t im, sampler_t s, const C &c) {
    const int4 r = read_imagei(im, s, c);
    return make_vec<uint4>(r);
}
// write: coordinates outside the image are ignored
template <class C> inline int64_t clshim_write_texel(image3d_t im, const C &c) {
    const int x = comp<int>(c, 0), y = comp<int>(c, 1), z = vtraits<C>::n > 2 ? comp<int>(c, 2) : 0;
    if (x < 0 || y < 0 || z < 0 || x >= im->w || y >= im->h || z >= im->d) return -1;
    return (int64_t)x + (int64_t)im->w * ((int64_t)y + (int64_t)im->h * z);
}
template <class C, class V> inline void write_imagef(image3d_t im, const C &c, const V &v) {
    const int64_t t = clshim_write_texel(im, c);
    if (t < 0) return;
    for (int k = 0; k < im->channels; k++) im->writef(t, k, comp<float>(v, vtraits<V>::is ? k : 0));
}
template <class C, class V> inline void write_imagei(image3d_t im, const C &c, const V &v) {
    const int64_t t = clshim_write_texel(im, c);
    if (t < 0) return;
    for (int k = 0; k < im->channels; k++) im->writei(t, k, comp<int64_t>(v, vtraits<V>::is ? k : 0));
}
template <class C, class V> inline void write_imageui(image3d_t im, const C &c, const V &v) { write_imagei(im, c, v); }
inline int get_image_width(image3d_t im) { return im->w; }
inline int get_image_height(image3d_t im) { return im->h; }
inline int get_image_depth(image3d_t im) { return im->d; }
