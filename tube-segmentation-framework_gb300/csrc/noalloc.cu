// noalloc.cu -- tsf_gvf_static: GVF iterations for callers that cannot
// allocate device memory.
//
// tsf_gvf needs a caller-provided workspace (one ping-pong copy of the planar
// field).  Some callers can neither call cudaMalloc nor hand over a
// workspace: plug-in hosts that own the device allocator and expose only the
// input and output buffers, or real-time imaging pipelines that forbid any
// device allocation once they are running.  This entry point serves them: its
// scratch is a fixed array in the library's own device memory, reserved when
// the library's device code is loaded on a GPU and kept until the process
// exits.
//
// Limits and rules:
//  * At most kStaticScratchBytes (96 MiB) of scratch: 3 * X*Y*Z stored
//    components, i.e. up to 256^3 voxels in a 16-bit format or 8,388,608
//    voxels in FP32.  Larger volumes are rejected with TSF_ERR_CAPACITY.
//  * The first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.  The address is kept for the life of the
//    process, so cudaDeviceReset between calls is not supported (the module
//    may be loaded again at another address).
//  * All calls share the one array: calls that overlap on the GPU (other
//    streams, other host threads) race on it.  The scratch needs no clearing:
//    the first iteration overwrites all of it.
//  * Nothing is allocated: no cudaMalloc, cudaFree or allocating library call.
#include <mutex>

#include "tsf_common.cuh"

namespace tsf {

int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st, void *ws,
            size_t ws_bytes, int mode, cudaStream_t s);
size_t gvf_workspace_size(int X, int Y, int Z, int st);

constexpr size_t kStaticScratchBytes = (size_t)96 << 20;

static __device__ __align__(256) unsigned char g_gvf_static_scratch[kStaticScratchBytes];

static std::mutex g_static_mutex;
static void *g_static_ptr[kMaxDevices];

// Device address of the scratch array on the current device (set up once per
// device).  Returns TSF_OK and the pointer, or an error.
static int static_scratch(void **out) {
    int dev = 0;
    TSF_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(TSF_ERR_INVALID_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_gvf_static_scratch);
        if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(g_gvf_static_scratch)");
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return TSF_OK;
}

}  // namespace tsf

extern "C" int tsf_gvf_static(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
                              int storage, void *stream) {
    using namespace tsf;
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(storage)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    const size_t need = gvf_workspace_size(X, Y, Z, storage);
    if (need > kStaticScratchBytes)
        return fail(TSF_ERR_CAPACITY, "volume too large for tsf_gvf_static: it needs " + std::to_string(need) +
                                          " bytes of scratch, the static array holds " +
                                          std::to_string(kStaticScratchBytes) + " (use tsf_gvf with a workspace)");
    void *ws = nullptr;
    r = static_scratch(&ws);
    if (r) return r;
    return run_gvf(d_f0, d_v, X, Y, Z, mu, iterations, storage, ws, kStaticScratchBytes, 0,
                   reinterpret_cast<cudaStream_t>(stream));
}
