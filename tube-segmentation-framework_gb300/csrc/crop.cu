// crop.cu -- the cropping stage of readDatasetAndTransfer
// (tube-segmentation.cpp:1556-1799; kernels cropDatasetThreshold and
// cropDatasetLung, kernels.cl:813-946) on the raw, typed volume.
//
// Both kernels count, per slice, the scan lines that are "inside": for
// cropDatasetThreshold a scan line with some voxel above the threshold, for
// cropDatasetLung one whose run-length state machine (white above the HU limit,
// black below, areas detected when a run count reaches 30) sees two white areas
// and one black, or more than one of each.  The reference runs one work-item
// per slice for each of the three slice directions.  Slices along x and along y
// scan the same lines -- the z-columns at (x, y) -- so one pass decides every
// z-column once and adds its verdict to both the x and the y count
// (crop_zlines_kernel); slices along z scan the x-rows at (y, z)
// (crop_xrows_kernel, rows staged through shared memory so that the loads are
// coalesced while each thread walks its own row).  Counts are integers, so
// the order of the atomic additions changes nothing.
#include <algorithm>

#include "tsf_common.cuh"

namespace tsf {

// Value reading of the reference's three image types (kernel argument `type`):
// 1 signed integer (read_imagei), 2 unsigned integer (read_imageui), 3 float.
template <typename T> struct CropRead;
template <> struct CropRead<int8_t> {
    static constexpr int kind = 1;
    static __device__ __forceinline__ float as_float(int8_t v) { return (float)(int)v; }
    static __device__ __forceinline__ int hu(int8_t v) { return (int)(int16_t)v; }
};
template <> struct CropRead<int16_t> {
    static constexpr int kind = 1;
    static __device__ __forceinline__ float as_float(int16_t v) { return (float)(int)v; }
    static __device__ __forceinline__ int hu(int16_t v) { return (int)v; }
};
template <> struct CropRead<uint8_t> {
    static constexpr int kind = 2;
    static __device__ __forceinline__ float as_float(uint8_t v) { return (float)(unsigned)v; }
    static __device__ __forceinline__ int hu(uint8_t v) { return (int)(int16_t)(uint16_t)v; }
};
template <> struct CropRead<uint16_t> {
    static constexpr int kind = 2;
    static __device__ __forceinline__ float as_float(uint16_t v) { return (float)(unsigned)v; }
    // read_imageui(...).x stored into a short: the 16 bits reinterpreted
    static __device__ __forceinline__ int hu(uint16_t v) { return (int)(int16_t)v; }
};
template <> struct CropRead<float> {
    static constexpr int kind = 3;
    static __device__ __forceinline__ float as_float(float v) { return v; }
    static __device__ __forceinline__ int hu(float) { return 0; }   // lung cropping rejects float data
};

// One scan line's state (cropDatasetLung's counters, or "found" for the threshold).
template <bool LUNG> struct LineState {
    int w = 0, b = 0, dw = 0, db = 0;
    bool found = false;
    template <typename T> __device__ __forceinline__ void step(T v, float thr, int hu_limit) {
        if constexpr (LUNG) {
            if (CropRead<T>::hu(v) > hu_limit) {
                if (w == 30) {
                    dw++;
                    b = 0;
                }
                w++;
            } else {
                if (b == 30) {
                    db++;
                    w = 0;
                }
                b++;
            }
        } else {
            found = found || CropRead<T>::as_float(v) > thr;
        }
    }
    __device__ __forceinline__ bool inside() const {
        if constexpr (LUNG) return (dw == 2 && db == 1) || (db > 1 && dw > 1);
        else return found;
    }
};

constexpr int kZlTX = 32, kZlTY = 8;

// z-columns: thread (x, y) walks z; counts_x[x] and counts_y[y] gain its verdict
template <typename T, bool LUNG>
__global__ void __launch_bounds__(kZlTX *kZlTY) crop_zlines_kernel(const T *__restrict__ vol, int X, int Y, int Z,
                                                                     float thr, int hu_limit, int *__restrict__ cx,
                                                                     int *__restrict__ cy) {
    __shared__ int sx[kZlTX], sy[kZlTY];
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (ty == 0) sx[tx] = 0;
    if (tx < kZlTY && ty == 0) sy[tx] = 0;
    __syncthreads();
    const int x = blockIdx.x * kZlTX + tx, y = blockIdx.y * kZlTY + ty;
    if (x < X && y < Y) {
        LineState<LUNG> s;
        const size_t plane = (size_t)X * Y;
        const T *p = vol + (size_t)x + (size_t)X * y;
        int z = 0;
        for (; z + 4 <= Z; z += 4) {
            const T v0 = __ldg(p + plane * z), v1 = __ldg(p + plane * (z + 1)), v2 = __ldg(p + plane * (z + 2)),
                    v3 = __ldg(p + plane * (z + 3));
            s.step(v0, thr, hu_limit);
            s.step(v1, thr, hu_limit);
            s.step(v2, thr, hu_limit);
            s.step(v3, thr, hu_limit);
        }
        for (; z < Z; z++) s.step(__ldg(p + plane * z), thr, hu_limit);
        if (s.inside()) {
            atomicAdd(&sx[tx], 1);
            atomicAdd(&sy[ty], 1);
        }
    }
    __syncthreads();
    if (ty == 0 && x < X && sx[tx]) atomicAdd(&cx[x], sx[tx]);
    if (ty == 0 && tx < kZlTY) {
        const int yy = blockIdx.y * kZlTY + tx;
        if (yy < Y && sy[tx]) atomicAdd(&cy[yy], sy[tx]);
    }
}

constexpr int kXrRows = 128, kXrChunk = 32;

// x-rows: 128 consecutive rows (index y + Y z) per block, one thread per row;
// chunks of 32 elements of all 128 rows are staged through shared memory
template <typename T, bool LUNG>
__global__ void __launch_bounds__(kXrRows) crop_xrows_kernel(const T *__restrict__ vol, int X, int Y, int Z,
                                                               float thr, int hu_limit, int *__restrict__ cz) {
    __shared__ T tile[kXrRows][kXrChunk + 1];
    const int64_t rows = (int64_t)Y * Z;
    const int64_t r0 = (int64_t)blockIdx.x * kXrRows;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LineState<LUNG> s;
    for (int c0 = 0; c0 < X; c0 += kXrChunk) {
        const int cn = min(kXrChunk, X - c0);
        // each warp loads rows warp, warp + 4, ... ; lane = element of the chunk
        for (int r = warp; r < kXrRows; r += kXrRows / 32) {
            const int64_t row = r0 + r;
            if (row < rows && lane < cn) tile[r][lane] = __ldg(vol + (size_t)row * X + c0 + lane);
        }
        __syncthreads();
        if (r0 + threadIdx.x < rows)
            for (int k = 0; k < cn; k++) s.step(tile[threadIdx.x][k], thr, hu_limit);
        __syncthreads();
    }
    const int64_t row = r0 + threadIdx.x;
    const bool in = row < rows && s.inside();
    // rows of one z are consecutive: add per z, one atomic per distinct z in the warp
    const int z = row < rows ? (int)(row / Y) : -1;
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if (!m) return;
    const unsigned same = __match_any_sync(0xffffffffu, z);
    const int leader = __ffs(same) - 1;
    const int cnt = __popc(m & same);
    if (lane == leader && z >= 0 && cnt) atomicAdd(&cz[z], cnt);
}

__global__ void crop_finish_kernel(const int *__restrict__ c, int16_t *__restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int16_t)c[i];   // the reference counts in a short
}

template <typename T>
__global__ void crop_copy_kernel(const T *__restrict__ src, int X, int Y, int x1, int y1, int z1, int SX, int SY, int SZ,
                                 T *__restrict__ dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= SX || y >= SY || z >= SZ) return;
    dst[(size_t)x + (size_t)SX * ((size_t)y + (size_t)SY * z)] =
        src[(size_t)(x + x1) + (size_t)X * ((size_t)(y + y1) + (size_t)Y * (z + z1))];
}

static size_t crop_elem(int type) {
    switch (type) {
    case TSF_TYPE_UINT8:
    case TSF_TYPE_INT8: return 1;
    case TSF_TYPE_UINT16:
    case TSF_TYPE_INT16: return 2;
    case TSF_TYPE_FLOAT32: return 4;
    default: return 0;
    }
}

#define TSF_DISPATCH_TYPE(type, T, ...)                                    \
    switch (type) {                                                        \
    case TSF_TYPE_UINT8: { using T = uint8_t; __VA_ARGS__; } break;        \
    case TSF_TYPE_INT8: { using T = int8_t; __VA_ARGS__; } break;          \
    case TSF_TYPE_UINT16: { using T = uint16_t; __VA_ARGS__; } break;      \
    case TSF_TYPE_INT16: { using T = int16_t; __VA_ARGS__; } break;        \
    case TSF_TYPE_FLOAT32: { using T = float; __VA_ARGS__; } break;        \
    default: return fail(TSF_ERR_INVALID_ARG, "unknown data type");       \
    }

size_t crop_workspace_size(int X, int Y, int Z) { return ((size_t)X + Y + Z) * sizeof(int); }

template <typename T, bool LUNG>
static int crop_launch(const T *vol, int X, int Y, int Z, float thr, int *c, cudaStream_t s) {
    const int hu_limit = CropRead<T>::kind == 2 ? -150 + 1024 : -150;
    const dim3 g1((X + kZlTX - 1) / kZlTX, (Y + kZlTY - 1) / kZlTY);
    crop_zlines_kernel<T, LUNG><<<g1, dim3(kZlTX, kZlTY), 0, s>>>(vol, X, Y, Z, thr, hu_limit, c, c + X);
    const int64_t rows = (int64_t)Y * Z;
    crop_xrows_kernel<T, LUNG><<<(unsigned)((rows + kXrRows - 1) / kXrRows), kXrRows, 0, s>>>(vol, X, Y, Z, thr,
                                                                                               hu_limit, c + X + Y);
    TSF_CHECK_LAUNCHES("crop scan lines", 2);
    return TSF_OK;
}

int run_crop_scan_lines(const void *vol, int type, int X, int Y, int Z, int method, float thr, int16_t *counts,
                        void *ws, size_t ws_bytes, cudaStream_t s) {
    if (X <= 0 || Y <= 0 || Z <= 0 || (int64_t)X * Y * Z > (int64_t)1 << 34)
        return fail(TSF_ERR_INVALID_ARG, "bad volume extents");
    if (!vol || !counts) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (crop_elem(type) == 0) return fail(TSF_ERR_INVALID_ARG, "unknown data type");
    if (method != 0 && method != 1) return fail(TSF_ERR_INVALID_ARG, "cropping method must be 0 (threshold) or 1 (lung)");
    if (method == 1 && type == TSF_TYPE_FLOAT32)
        return fail(TSF_ERR_INVALID_ARG, "lung cropping reads integer HU values; float data is not supported");
    if (Y > 65535 * kZlTY) return fail(TSF_ERR_INVALID_ARG, "volume too tall");
    if (!ws || ws_bytes < crop_workspace_size(X, Y, Z)) return fail(TSF_ERR_WORKSPACE, "cropping workspace too small");
    int *c = static_cast<int *>(ws);
    const int n = X + Y + Z;
    TSF_TRY_CUDA(cudaMemsetAsync(c, 0, (size_t)n * sizeof(int), s));
    int r = TSF_OK;
    TSF_DISPATCH_TYPE(type, T, {
        r = method ? crop_launch<T, true>(static_cast<const T *>(vol), X, Y, Z, thr, c, s)
                   : crop_launch<T, false>(static_cast<const T *>(vol), X, Y, Z, thr, c, s);
    });
    if (r) return r;
    crop_finish_kernel<<<(n + 255) / 256, 256, 0, s>>>(c, counts, n);
    TSF_CHECK_LAUNCH("crop_finish_kernel");
    return TSF_OK;
}

int run_crop_copy(const void *src, int type, int X, int Y, int Z, const int *box, void *dst, cudaStream_t s) {
    if (!src || !dst || !box) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (crop_elem(type) == 0) return fail(TSF_ERR_INVALID_ARG, "unknown data type");
    const int x1 = box[0], y1 = box[1], z1 = box[2], SX = box[3], SY = box[4], SZ = box[5];
    if (x1 < 0 || y1 < 0 || z1 < 0 || SX <= 0 || SY <= 0 || SZ <= 0 || x1 + SX > X || y1 + SY > Y || z1 + SZ > Z)
        return fail(TSF_ERR_INVALID_ARG, "crop box outside the volume");
    if (SZ > 65535) return fail(TSF_ERR_INVALID_ARG, "crop box too deep");
    const dim3 blk(64, 4), grd((SX + 63) / 64, (SY + 3) / 4, SZ);
    TSF_DISPATCH_TYPE(type, T, {
        crop_copy_kernel<T><<<grd, blk, 0, s>>>(static_cast<const T *>(src), X, Y, x1, y1, z1, SX, SY, SZ,
                                                static_cast<T *>(dst));
    });
    TSF_CHECK_LAUNCH("crop_copy_kernel");
    return TSF_OK;
}

}  // namespace tsf

extern "C" size_t tsf_crop_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return tsf::crop_workspace_size(X, Y, Z);
}

extern "C" int tsf_crop_scan_lines(const void *d_volume, int type, int X, int Y, int Z, int method, float threshold,
                                   int16_t *d_counts, void *d_workspace, size_t workspace_bytes, void *stream) {
    return tsf::run_crop_scan_lines(d_volume, type, X, Y, Z, method, threshold, d_counts, d_workspace,
                                    workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_crop_copy(const void *d_volume, int type, int X, int Y, int Z, const int *box, void *d_out,
                             void *stream) {
    return tsf::run_crop_copy(d_volume, type, X, Y, Z, box, d_out, reinterpret_cast<cudaStream_t>(stream));
}
