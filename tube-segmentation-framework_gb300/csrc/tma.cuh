// tma.cuh -- inline-PTX wrappers for the Blackwell asynchronous copy path:
// mbarriers (init, arrive with an expected transaction count, bounded
// parity wait) and tiled tensor loads (cp.async.bulk.tensor) from a
// CUtensorMap, plus the host-side tensor-map encoder obtained from the driver
// at run time (no link against libcuda).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

namespace tsf {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes barrier initialisation visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one arrival that also announces `bytes` of incoming transactions
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// one plain arrival (release at CTA scope)
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Upper bound of a barrier wait, in SM clock cycles (about 2 s at 2 GHz).  A
// copy that has not landed by then is treated as lost: the caller records an
// error instead of spinning forever.
constexpr long long kWaitCycles = 4000000000LL;

// Waits until the phase with the given parity has completed; false when
// `limit` cycles pass first.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = kWaitCycles) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}

// Tiled 4-D tensor load of one box into shared memory; completion is signalled
// on `bar` as transaction bytes.  c0 is the innermost coordinate: c0 times the
// element size must be a multiple of 16 bytes (other coordinates are free and
// may lie outside the tensor, which reads as zero).
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                            int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Host: cuTensorMapEncodeTiled from the driver (NULL if unavailable).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// Host: 4-D map (x, y, z, component) over a planar field of three X*Y*Z
// planes with es-byte elements, box (bx, by, 1, 3).  False if the driver
// rejects it (strides must be multiples of 16 bytes).
bool encode_planar(CUtensorMap *m, const void *base, int X, int Y, int Z, int es, int bx, int by);

}  // namespace tsf
