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
                o[2 * k] = Store<ST>::load((int16_t)(u & 0xffffu));
                o[2 * k + 1] = Store<ST>::load((int16_t)(u >> 16));
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
                const int16_t lo = Store<ST>::store(o[2 * k]), hi = Store<ST>::store(o[2 * k + 1]);
                u[k] = (unsigned)(uint16_t)lo | ((unsigned)(uint16_t)hi << 16);
            }
        }
        if constexpr (BYTES == 16) *reinterpret_cast<uint4 *>(p) = make_uint4(u[0], u[1], u[2], u[3]);
        else *reinterpret_cast<uint2 *>(p) = make_uint2(u[0], u[1]);
    }
};


}  // namespace tsf
