// tsf_common.cuh -- shared device helpers for libtsf_gb300 (sm_103a).
//
// Storage formats, their conversions, clamped index helpers and the error
// plumbing of the C ABI.  All kernels are compiled with -fmad=false: every
// product and sum is rounded separately, so a kernel and the float oracle that
// evaluates the same expression in the same order agree bit for bit.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/tsf/tsf_c.h"

namespace tsf {

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int check_cuda(cudaError_t e, const char *what);
void count_launches(int n);   // process-wide kernel launch counter

#define TSF_TRY_CUDA(expr)                                   \
    do {                                                     \
        cudaError_t e__ = (expr);                            \
        if (e__ != cudaSuccess) return ::tsf::check_cuda(e__, #expr); \
    } while (0)

// Checks the launch(es) just issued and adds `n` to the launch counter.
#define TSF_CHECK_LAUNCHES(name, n)                                         \
    do {                                                                    \
        cudaError_t e__ = cudaGetLastError();                               \
        if (e__ != cudaSuccess) return ::tsf::check_cuda(e__, name);       \
        ::tsf::count_launches(n);                                           \
    } while (0)
#define TSF_CHECK_LAUNCH(name) TSF_CHECK_LAUNCHES(name, 1)

inline int check_dims(int X, int Y, int Z) {
    if (X < 4 || Y < 4 || Z < 4) return fail(TSF_ERR_INVALID_ARG, "volume extents must be >= 4 per axis");
    if ((int64_t)X * Y * Z > (int64_t)1 << 34) return fail(TSF_ERR_INVALID_ARG, "volume too large");
    return TSF_OK;
}

// Device ordinals the per-device caches of this library cover.
constexpr int kMaxDevices = 64;

inline bool valid_storage(int s) { return s >= TSF_STORE_F32 && s <= TSF_STORE_SNORM16; }

// ---------------------------------------------------------------------------
// storage formats
// ---------------------------------------------------------------------------
template <int ST> struct Store;

template <> struct Store<TSF_STORE_F32> {
    using T = float;
    static __device__ __forceinline__ float load(T v) { return v; }
    static __device__ __forceinline__ T store(float v) { return v; }
};

template <> struct Store<TSF_STORE_F16> {
    using T = __half;
    static __device__ __forceinline__ float load(T v) { return __half2float(v); }
    static __device__ __forceinline__ T store(float v) { return __float2half_rn(v); }
};

template <> struct Store<TSF_STORE_BF16> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float load(T v) { return __bfloat162float(v); }
    static __device__ __forceinline__ T store(float v) { return __float2bfloat16_rn(v); }
};

// OpenCL CL_SNORM_INT16: write convert_short_sat_rte(v * 32767), read
// max(-1, s / 32767) (kernels_no_3d_write.cl:9-21, OpenCL 1.1 section 8.3).
//
// The read uses neither a division nor an integer -> float conversion (the
// conversion unit runs at a fraction of the FMA rate and bounded the 16-bit
// GVF iteration).  With t = s * 2^-15,
//   s / 32767 = t / (1 - 2^-15) = t (1 + 2^-15 + 2^-30 + 2^-45 + ...),
// and one fma gives RN(t + t * c) with c = 2^-15 + 2^-30 (an FP32 value, the
// same bits as RN(1 / 32767)).  The exact fma operand s (2^30 + 2^15 + 1)
// 2^-45 lies below s / 32767 by |s| / (2^45 (2^15 - 1)) <= 2^-45: less than
// one unit of 2^-45, while every rounding boundary of the result is a
// multiple of that unit and the operand, whose low bits repeat s, is never
// one -- so both round to the same FP32 value.  t itself comes from the bit
// pattern: flipping bit 15 of the stored 16 bits gives s + 2^15 (0..65535),
// and placed as the low mantissa bits of 384.0f (0x43C00000, where one unit
// of the mantissa is 2^-15) it makes the FP32 value 384 + (s + 2^15) 2^-15
// = 385 + t; one subtraction (exact: same exponent) leaves t.  Checked
// against exact rational arithmetic for all 65,536 inputs
// (tests/test_snorm16_read.py).
__device__ __forceinline__ float snorm16_from_bits(unsigned u16) {
    const float t = __fsub_rn(__uint_as_float((u16 & 0xffffu) ^ 0x43C08000u), 385.0f);
    return fmaxf(-1.0f, __fmaf_rn(t, __uint_as_float(0x38000100u), t));
}

// convert_short_sat_rte: PTX float -> integer conversions round as asked
// (.rni: to nearest even), clamp to the destination range and turn NaN into
// 0 -- the OpenCL rule, in one conversion.
__device__ __forceinline__ unsigned short snorm16_bits(float v) {
    const float f = __fmul_rn(v, 32767.0f);
    unsigned short i;
    asm("cvt.rni.s16.f32 %0, %1;" : "=h"(i) : "f"(f));
    return i;
}

// Two FP32 operations in one instruction (PTX .f32x2, sm_100 and later),
// each rounded like its scalar counterpart.  The explicit .rn keeps the
// assembler from contracting a product and a following sum into an fma.
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// Both values of a 32-bit word of two stored snorm16 values (low half
// first), read as snorm16_from_bits does with the two subtractions and the
// two fmas paired.  The clamp moves to the integers: s = -32768 and
// s = -32767 both read as -1, so one paired 16-bit max replaces the two FP32
// max operations; two byte permutations place each half under 384.0f's
// exponent.
__device__ __forceinline__ float2 snorm16_pair2(unsigned w) {
    const unsigned x = __vmaxs2(w, 0x80018001u) ^ 0x80008000u;   // s + 2^15 in each half
    const float2 b = make_float2(__uint_as_float(__byte_perm(x, 0x43C00000u, 0x7610)),
                                 __uint_as_float(__byte_perm(x, 0x43C00000u, 0x7632)));
    const float2 t = sub2(b, make_float2(385.0f, 385.0f));
    const float c = __uint_as_float(0x38000100u);
    return fma2(t, make_float2(c, c), t);
}

// The offset form of a word of two snorm16 values: each half clamped to
// -32767 and moved to s + 2^15 (1..65535) -- the first step of
// snorm16_pair2, done once where a copy of the field is written so that the
// readers of the copy skip it.  Same values on reading: -32768 and -32767
// both read as -1.
__device__ __forceinline__ unsigned snorm16_offset2(unsigned w) { return __vmaxs2(w, 0x80018001u) ^ 0x80008000u; }

// Reads of the offset form (snorm16_offset2): the two values of a word, and
// the low half alone; the same bits as snorm16_pair2 / snorm16_from_bits of
// the original values (t >= -32767 2^-15, whose fma read is exactly -1, so
// no clamp is left to do).
__device__ __forceinline__ float2 snorm16_offset_pair2(unsigned x) {
    const float2 b = make_float2(__uint_as_float(__byte_perm(x, 0x43C00000u, 0x7610)),
                                 __uint_as_float(__byte_perm(x, 0x43C00000u, 0x7632)));
    const float2 t = sub2(b, make_float2(385.0f, 385.0f));
    const float c = __uint_as_float(0x38000100u);
    return fma2(t, make_float2(c, c), t);
}
__device__ __forceinline__ float snorm16_offset_lo(unsigned x) {
    const float t = __fsub_rn(__uint_as_float(__byte_perm(x, 0x43C00000u, 0x7610)), 385.0f);
    return __fmaf_rn(t, __uint_as_float(0x38000100u), t);
}

// Two snorm16 values of a pair stored as one 32-bit word (low half first).
__device__ __forceinline__ unsigned snorm16_store2(float2 v) {
    const float2 f = mul2(v, make_float2(32767.0f, 32767.0f));
    unsigned short lo, hi;
    asm("cvt.rni.s16.f32 %0, %1;" : "=h"(lo) : "f"(f.x));
    asm("cvt.rni.s16.f32 %0, %1;" : "=h"(hi) : "f"(f.y));
    unsigned u;
    asm("mov.b32 %0, {%1, %2};" : "=r"(u) : "h"(lo), "h"(hi));
    return u;
}

template <> struct Store<TSF_STORE_SNORM16> {
    using T = int16_t;
    static __device__ __forceinline__ float load(T v) { return snorm16_from_bits((unsigned)(uint16_t)v); }
    static __device__ __forceinline__ T store(float v) { return (T)snorm16_bits(v); }
};

// Value after a store and a load (what the next reader sees).
template <int ST> __device__ __forceinline__ float quantize(float v) {
    return Store<ST>::load(Store<ST>::store(v));
}

// OpenCL CL_UNORM_INT16 TDF (kernels.cl:11-13): convert_ushort_sat_rte(v*65535).
__device__ __forceinline__ uint16_t to_unorm16(float v) {
    float f = __fmul_rn(v, 65535.0f);
    int i = __float2int_rn(f);
    i = max(0, min(65535, i));
    return (uint16_t)i;
}
__device__ __forceinline__ float from_unorm16(uint16_t u) { return __fdiv_rn((float)u, 65535.0f); }

// Four stored components of a field4 voxel, loaded with one vector access.
template <int ST> struct Vec4Load;

template <> struct Vec4Load<TSF_STORE_F32> {
    static __device__ __forceinline__ float4 load(const void *base, int64_t i) {
        return __ldg(reinterpret_cast<const float4 *>(base) + i);
    }
};

template <int ST> struct Vec4Load {
    static __device__ __forceinline__ float4 load(const void *base, int64_t i) {
        uint2 raw = __ldg(reinterpret_cast<const uint2 *>(base) + i);
        if constexpr (ST == TSF_STORE_SNORM16) {
            const float2 xy = snorm16_pair2(raw.x);
            return make_float4(xy.x, xy.y, snorm16_from_bits(raw.y), snorm16_from_bits(raw.y >> 16));
        } else {
            using T = typename Store<ST>::T;
            T c[4];
            memcpy(c, &raw, 8);
            return make_float4(Store<ST>::load(c[0]), Store<ST>::load(c[1]), Store<ST>::load(c[2]),
                               Store<ST>::load(c[3]));
        }
    }
};

template <int ST> __device__ __forceinline__ void store4(void *base, int64_t i, float a, float b,
                                                         float c, float d) {
    using T = typename Store<ST>::T;
    if constexpr (ST == TSF_STORE_F32) {
        reinterpret_cast<float4 *>(base)[i] = make_float4(a, b, c, d);
    } else {
        T v[4] = {Store<ST>::store(a), Store<ST>::store(b), Store<ST>::store(c), Store<ST>::store(d)};
        uint2 raw;
        memcpy(&raw, v, 8);
        reinterpret_cast<uint2 *>(base)[i] = raw;
    }
}

__host__ __device__ __forceinline__ int clampi(int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

// Mirror boundary rule of GVF3DIteration (kernels.cl:1472-1475).
__host__ __device__ __forceinline__ int mirror(int w, int n) {
    int p = (w == 0) ? 2 : w;
    return (p >= n - 1) ? n - 3 : p;
}

__host__ __device__ __forceinline__ int64_t lin(int x, int y, int z, int X, int Y) {
    return (int64_t)x + (int64_t)X * ((int64_t)y + (int64_t)Y * (int64_t)z);
}

// Dispatch a runtime storage format to a template.
#define TSF_DISPATCH_STORAGE(st, ST, ...)                                     \
    switch (st) {                                                             \
    case TSF_STORE_F32: { constexpr int ST = TSF_STORE_F32; __VA_ARGS__; } break;      \
    case TSF_STORE_F16: { constexpr int ST = TSF_STORE_F16; __VA_ARGS__; } break;      \
    case TSF_STORE_BF16: { constexpr int ST = TSF_STORE_BF16; __VA_ARGS__; } break;    \
    case TSF_STORE_SNORM16: { constexpr int ST = TSF_STORE_SNORM16; __VA_ARGS__; } break; \
    default: return fail(TSF_ERR_INVALID_ARG, "unknown storage format");      \
    }

inline size_t storage_bytes(int st) { return st == TSF_STORE_F32 ? 4 : (valid_storage(st) ? 2 : 0); }

// ---------------------------------------------------------------------------
// programmatic dependent launch
// ---------------------------------------------------------------------------
// A kernel launched with pdl_config may be scheduled while the kernel before
// it in the stream is still finishing.  It must call pdl_wait() before its
// first access to global memory that the previous kernel writes or reads
// (the wait returns once that grid has completed and its writes are
// visible); pdl_trigger() lets the next such kernel be scheduled as this
// grid's CTAs exit.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, size_t smem, cudaStream_t s, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

}  // namespace tsf
