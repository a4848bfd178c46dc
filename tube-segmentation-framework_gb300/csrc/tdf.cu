// tdf.cu -- the circle-fitting TDF's host side and its small kernels: the
// launch of the sweep kernels (tdf_kernels.cuh) with the reference's tred2 +
// tql2 (eigen mode 0; mode 1, the closed form, is instantiated in
// tdf_closed.cu), the x-paired 16-bit copy of the field and combine
// (kernels.cl:561-572).
#include "tdf_kernels.cuh"

namespace tsf {

int launch_tdf_kernels_closed(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                              const CircleTable &tab, void *d_T, int unorm, float *d_R, cudaStream_t s, int kernel,
                              const uint4 *P, int fast_ok);

// The x-paired copy of a 16-bit field4 image: P[i] = (texel i, texel of the
// next x, clamped at the last column), 16 bytes per voxel.  OFFSET (snorm16):
// the texels in the offset form (snorm16_offset2), which the samplers of the
// copy read with one step less per value.
template <bool OFFSET>
__global__ void tdf_pair_kernel(const uint2 *__restrict__ F, uint4 *__restrict__ P, int X, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % X);
    const uint2 a = __ldg(F + i), b = __ldg(F + i + (x + 1 < X ? 1 : 0));
    if (OFFSET)
        P[i] = make_uint4(snorm16_offset2(a.x), snorm16_offset2(a.y), snorm16_offset2(b.x), snorm16_offset2(b.y));
    else
        P[i] = make_uint4(a.x, a.y, b.x, b.y);
}

size_t tdf_workspace_size(int X, int Y, int Z, int st) {
    if (X <= 0 || Y <= 0 || Z <= 0 || !valid_storage(st) || st == TSF_STORE_F32) return 0;
    return (size_t)X * Y * Z * sizeof(uint4);
}

template <bool UNORM>
__global__ void combine_kernel(const void *__restrict__ Ts, const float *__restrict__ Rs, void *Tl, float *Rl, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (UNORM) {
        const uint16_t s = reinterpret_cast<const uint16_t *>(Ts)[i];
        uint16_t *L = reinterpret_cast<uint16_t *>(Tl);
        if (L[i] < s) { L[i] = s; Rl[i] = Rs[i]; }
    } else {
        const float s = reinterpret_cast<const float *>(Ts)[i];
        float *L = reinterpret_cast<float *>(Tl);
        if (L[i] < s) { L[i] = s; Rl[i] = Rs[i]; }
    }
}

// tdf_mode: 0 = default (per storage format, see launch_tdf_kernels), 1 = one
// voxel per lane, 2 = one sample per lane, 3 = load-balanced sweeps.
// ws / ws_bytes: room for the x-paired copy of a 16-bit field (tdf_workspace_size);
// without it, or for FP32 storage, the samples read the field itself.
// samples / stride: circle samples per radius and the table stride (32 / 1 in
// the reference); eigen: 0 = tred2 + tql2, 1 = the closed form.
int launch_tdf_circle(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                      void *d_T, int unorm, float *d_R, cudaStream_t s, int tdf_mode, void *ws, size_t ws_bytes,
                      int samples, int stride, int eigen) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_field4 || !d_T || !d_R) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!(rstep >= 0.0f) || !(rmin >= 0.0f)) return fail(TSF_ERR_INVALID_ARG, "invalid radius range");
    if (samples < 4 || samples > 32 || samples % 4 != 0 || stride < 1 || (samples - 1) * stride >= 32)
        return fail(TSF_ERR_INVALID_ARG, "samples must be a multiple of 4 in [4, 32] and (samples - 1) * stride < 32");
    if (eigen != 0 && eigen != 1) return fail(TSF_ERR_INVALID_ARG, "eigen mode must be 0 (tql2) or 1 (closed form)");
    const CircleTable tab = host_circle_table(samples, stride);
    if (tdf_mode < 0 || tdf_mode > 3) return fail(TSF_ERR_INVALID_ARG, "unknown TDF kernel");
    const bool queue = tdf_mode != 1;   // the brick kernels (0, 2, 3) may sample the paired copy
    const int fast_ok = (int64_t)X * Y * Z < ((int64_t)1 << 31) - 1;   // 32-bit texel offsets
    const int64_t n = (int64_t)X * Y * Z;
    const size_t need = tdf_workspace_size(X, Y, Z, st);
    const bool pair = queue && fast_ok && need > 0 && ws && ws_bytes >= need &&
                      (reinterpret_cast<uintptr_t>(ws) & 15) == 0 && (reinterpret_cast<uintptr_t>(d_field4) & 7) == 0;
    uint4 *P = pair ? static_cast<uint4 *>(ws) : nullptr;
    if (pair) {
        if (st == TSF_STORE_SNORM16)
            tdf_pair_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const uint2 *>(d_field4), P,
                                                                               X, n);
        else
            tdf_pair_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<const uint2 *>(d_field4),
                                                                                P, X, n);
        TSF_CHECK_LAUNCH("tdf_pair_kernel");
    }
    if (eigen == 1)
        return launch_tdf_kernels_closed(d_field4, X, Y, Z, st, rmin, rmax, rstep, tab, d_T, unorm, d_R, s, tdf_mode,
                                         P, fast_ok);
    return launch_tdf_kernels<0>(d_field4, X, Y, Z, st, rmin, rmax, rstep, tab, d_T, unorm, d_R, s, tdf_mode, P,
                                 fast_ok);
}

int launch_tdf_combine(const void *Ts, const float *Rs, void *Tl, float *Rl, int64_t n, int unorm, cudaStream_t s) {
    if (!Ts || !Rs || !Tl || !Rl || n <= 0) return fail(TSF_ERR_INVALID_ARG, "invalid combine arguments");
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if (unorm) combine_kernel<true><<<blocks, threads, 0, s>>>(Ts, Rs, Tl, Rl, n);
    else combine_kernel<false><<<blocks, threads, 0, s>>>(Ts, Rs, Tl, Rl, n);
    TSF_CHECK_LAUNCH("combine_kernel");
    return TSF_OK;
}

}  // namespace tsf
