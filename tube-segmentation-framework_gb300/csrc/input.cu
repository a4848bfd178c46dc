// input.cu -- conversion of the raw input volume to [0,1] floats (reference
// toFloat kernel, kernels.cl:989-1015; limits from getLimits,
// tube-segmentation.cpp:1380-1396): v = clamp(v, min, max);
// out = (v - min) / (max - min).  One thread per voxel; 1-4 B read and 4 B
// written per voxel.
#include "tsf_common.cuh"

namespace tsf {

template <typename In>
__global__ void to_float_kernel(const In *__restrict__ in, int64_t n, float lo, float hi, float *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = (float)in[i];
    v = v > hi ? hi : v;
    v = v < lo ? lo : v;
    out[i] = (v - lo) / (hi - lo);
}

int launch_to_float(const void *d_in, int type, int64_t n, float lo, float hi, float *d_out, cudaStream_t s) {
    if (!d_in || !d_out || n <= 0) return fail(TSF_ERR_INVALID_ARG, "invalid to_float arguments");
    if (!(hi > lo)) return fail(TSF_ERR_INVALID_ARG, "maximum must be greater than minimum");
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    switch (type) {
    case TSF_TYPE_UINT8: to_float_kernel<uint8_t><<<blocks, threads, 0, s>>>((const uint8_t *)d_in, n, lo, hi, d_out); break;
    case TSF_TYPE_INT8: to_float_kernel<int8_t><<<blocks, threads, 0, s>>>((const int8_t *)d_in, n, lo, hi, d_out); break;
    case TSF_TYPE_UINT16: to_float_kernel<uint16_t><<<blocks, threads, 0, s>>>((const uint16_t *)d_in, n, lo, hi, d_out); break;
    case TSF_TYPE_INT16: to_float_kernel<int16_t><<<blocks, threads, 0, s>>>((const int16_t *)d_in, n, lo, hi, d_out); break;
    case TSF_TYPE_FLOAT32: to_float_kernel<float><<<blocks, threads, 0, s>>>((const float *)d_in, n, lo, hi, d_out); break;
    default: return fail(TSF_ERR_INVALID_ARG, "unknown voxel type");
    }
    TSF_CHECK_LAUNCH("to_float_kernel");
    return TSF_OK;
}

}  // namespace tsf

extern "C" int tsf_to_float(const void *d_in, int type, int64_t n, float minimum, float maximum, float *d_out,
                            void *stream) {
    return tsf::launch_to_float(d_in, type, n, minimum, maximum, d_out, reinterpret_cast<cudaStream_t>(stream));
}
