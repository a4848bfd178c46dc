// packed.cuh -- 8- or 16-byte vectors of stored field components and their
// conversion to / from FP32, shared by the GVF kernels.
#pragma once

#include "tsf_common.cuh"

namespace tsf {

// BYTES (8 or 16) bytes of stored components -- 4 or 8 voxels of a 16-bit
// format, 2 or 4 of FP32 -- unpacked / packed two at a time with the paired
// conversion intrinsics.
template <int ST, int BYTES> struct PackedV {
    using T = typename Store<ST>::T;
    static constexpr int VX = BYTES / (int)sizeof(T);
    static constexpr int W = BYTES / 4;              // 32-bit words
    struct Raw { unsigned u[W]; };
    static __device__ __forceinline__ Raw load(const T *p) {
        Raw r;
        if constexpr (BYTES == 16) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
            r.u[0] = v.x; r.u[1] = v.y; r.u[2] = v.z; r.u[3] = v.w;
        } else {
            const uint2 v = __ldg(reinterpret_cast<const uint2 *>(p));
            r.u[0] = v.x; r.u[1] = v.y;
        }
        return r;
    }
    // plain load (any address space, e.g. shared memory)
    static __device__ __forceinline__ Raw load_plain(const T *p) {
        Raw r;
        if constexpr (BYTES == 16) {
            const uint4 v = *reinterpret_cast<const uint4 *>(p);
            r.u[0] = v.x; r.u[1] = v.y; r.u[2] = v.z; r.u[3] = v.w;
        } else {
            const uint2 v = *reinterpret_cast<const uint2 *>(p);
            r.u[0] = v.x; r.u[1] = v.y;
        }
        return r;
    }
    static __device__ __forceinline__ Raw zero() {
        Raw r;
#pragma unroll
        for (int i = 0; i < W; i++) r.u[i] = 0u;
        return r;
    }
    static __device__ __forceinline__ void unpack(const Raw &raw, float o[VX]) {
#pragma unroll
        for (int k = 0; k < W; k++) {
            const unsigned u = raw.u[k];
            if constexpr (ST == TSF_STORE_F32) {
                o[k] = __uint_as_float(u);
            } else if constexpr (ST == TSF_STORE_F16) {
                const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u));
                o[2 * k] = a.x; o[2 * k + 1] = a.y;
            } else if constexpr (ST == TSF_STORE_BF16) {
                o[2 * k] = __uint_as_float(u << 16);
                o[2 * k + 1] = __uint_as_float(u & 0xffff0000u);
            } else {
                const float2 a = snorm16_pair2(u);
                o[2 * k] = a.x; o[2 * k + 1] = a.y;
            }
        }
    }
    // rounds to the storage format (the only rounding of an iteration's result)
    static __device__ __forceinline__ void store(T *p, const float o[VX]) {
        unsigned u[W];
#pragma unroll
        for (int k = 0; k < W; k++) {
            if constexpr (ST == TSF_STORE_F32) {
                u[k] = __float_as_uint(o[k]);
            } else if constexpr (ST == TSF_STORE_F16) {
                const __half2 h = __floats2half2_rn(o[2 * k], o[2 * k + 1]);
                u[k] = *reinterpret_cast<const unsigned *>(&h);
            } else if constexpr (ST == TSF_STORE_BF16) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(o[2 * k], o[2 * k + 1]);
                u[k] = *reinterpret_cast<const unsigned *>(&h);
            } else {
                u[k] = snorm16_store2(make_float2(o[2 * k], o[2 * k + 1]));
            }
        }
        if constexpr (BYTES == 16) *reinterpret_cast<uint4 *>(p) = make_uint4(u[0], u[1], u[2], u[3]);
        else *reinterpret_cast<uint2 *>(p) = make_uint2(u[0], u[1]);
    }
};

// Mixed-precision arithmetic on one 16-bit half of a 32-bit word (K = 0: the
// low half, element 2k of a packed vector; K = 1: the high half), with a
// single rounding to FP32 (PTX add / sub / fma with .f16 / .bf16 sources and
// an .f32 destination, sm_100 and later).  A 16-bit value converts to FP32
// exactly, so
//   add16(u, c)    == RN(float(h) + c)      == convert, then add
//   sub16(u, c)    == RN(float(h) - c)      == convert, then subtract
// and, for FP16 only, the square of an FP16 value is exact in FP32 (11-bit
// significands, product within FP32's normal range), so
//   sqadd16(u, c)  == RN(float(h)^2 + c)    == convert, square, then add.
// (BF16 squares can leave FP32's normal range, so BF16 uses no sqadd16.)
template <int ST, int K> __device__ __forceinline__ float add16(unsigned u, float c) {
    static_assert(ST == TSF_STORE_F16 || ST == TSF_STORE_BF16, "16-bit float storage only");
    float d;
    if constexpr (ST == TSF_STORE_F16) {
        if constexpr (K == 0)
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tadd.rn.f32.f16 %0, l, %2;}" : "=f"(d) : "r"(u), "f"(c));
        else
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tadd.rn.f32.f16 %0, h, %2;}" : "=f"(d) : "r"(u), "f"(c));
    } else {
        if constexpr (K == 0)
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tadd.rn.f32.bf16 %0, l, %2;}" : "=f"(d) : "r"(u), "f"(c));
        else
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tadd.rn.f32.bf16 %0, h, %2;}" : "=f"(d) : "r"(u), "f"(c));
    }
    return d;
}

template <int ST, int K> __device__ __forceinline__ float sub16(unsigned u, float c) {
    static_assert(ST == TSF_STORE_F16 || ST == TSF_STORE_BF16, "16-bit float storage only");
    float d;
    if constexpr (ST == TSF_STORE_F16) {
        if constexpr (K == 0)
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tsub.rn.f32.f16 %0, l, %2;}" : "=f"(d) : "r"(u), "f"(c));
        else
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tsub.rn.f32.f16 %0, h, %2;}" : "=f"(d) : "r"(u), "f"(c));
    } else {
        if constexpr (K == 0)
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tsub.rn.f32.bf16 %0, l, %2;}" : "=f"(d) : "r"(u), "f"(c));
        else
            asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tsub.rn.f32.bf16 %0, h, %2;}" : "=f"(d) : "r"(u), "f"(c));
    }
    return d;
}

template <int K> __device__ __forceinline__ float sqadd16(unsigned u, float c) {
    float d;
    if constexpr (K == 0)
        asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tfma.rn.f32.f16 %0, l, l, %2;}" : "=f"(d) : "r"(u), "f"(c));
    else
        asm("{.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tfma.rn.f32.f16 %0, h, h, %2;}" : "=f"(d) : "r"(u), "f"(c));
    return d;
}

// Element i of a packed 16-bit vector, i a run-time index that unrolling
// turns into a constant (the branch folds away).
template <int ST> __device__ __forceinline__ float add16i(const unsigned *u, int i, float c) {
    return (i & 1) ? add16<ST, 1>(u[i >> 1], c) : add16<ST, 0>(u[i >> 1], c);
}

// Element i (0..3) of a packed 4-element 16-bit vector.
template <int ST, int I> __device__ __forceinline__ float add16v(const unsigned *u, float c) {
    return add16<ST, I & 1>(u[I >> 1], c);
}
template <int ST, int I> __device__ __forceinline__ float sub16v(const unsigned *u, float c) {
    return sub16<ST, I & 1>(u[I >> 1], c);
}
template <int I> __device__ __forceinline__ float sqadd16v(const unsigned *u, float c) {
    return sqadd16<I & 1>(u[I >> 1], c);
}

}  // namespace tsf
