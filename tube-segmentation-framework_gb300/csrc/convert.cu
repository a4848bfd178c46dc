// convert.cu -- a field from one storage format to another (no counterpart in
// the reference, whose fields keep one format for the whole run): the value
// each stored component reads as (Store<SRC>::load) rounded to the target
// format (Store<DST>::store).  Used to continue a 16-bit GVF in FP32, or to
// store an FP32 field in 16 bits for the TDF.
#include "tsf_common.cuh"

namespace tsf {

template <int SRC, int DST>
__global__ void __launch_bounds__(256) convert_kernel(const typename Store<SRC>::T *__restrict__ in,
                                                      typename Store<DST>::T *__restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = Store<DST>::store(Store<SRC>::load(in[i]));
}

}  // namespace tsf

extern "C" int tsf_convert_field(const void *d_in, int in_storage, void *d_out, int out_storage, int64_t n,
                                 void *stream) {
    using namespace tsf;
    if (!valid_storage(in_storage) || !valid_storage(out_storage)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_in || !d_out || n < 0) return fail(TSF_ERR_INVALID_ARG, "invalid buffers");
    if (n == 0) return TSF_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t blocks64 = (n + 255) / 256;
    const unsigned blocks = (unsigned)(blocks64 < 65536 ? blocks64 : 65536);
    TSF_DISPATCH_STORAGE(in_storage, SI, {
        TSF_DISPATCH_STORAGE(out_storage, SO, {
            convert_kernel<SI, SO><<<blocks, 256, 0, s>>>(static_cast<const typename Store<SI>::T *>(d_in),
                                                          static_cast<typename Store<SO>::T *>(d_out), n);
        });
    });
    TSF_CHECK_LAUNCH("convert_kernel");
    return TSF_OK;
}
