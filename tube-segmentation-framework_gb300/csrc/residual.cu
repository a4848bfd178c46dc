// residual.cu -- FP64 norms of the GVF residual, and a Jacobi GVF that stops
// on them.
//
// The reference runs a fixed number of GVF iterations (Jacobi,
// gradientVectorFlow.cpp:1137-1151) or FMG cycles (:803) and never measures
// how far from the solution it is; its multigrid computes residual images
// (residual / fmgResidual, kernels.cl:1973-2053) only to restrict them to the
// coarse grid.  Here the residual is reduced to norms, per component c:
//   kind 0, the Jacobi update of GVF3DIteration (kernels.cl:1486-1490):
//       r_c = mu * L(v_c) - (v_c - f0_c) |f0|^2      (= v_{k+1} - v_k before rounding)
//   kind 1, fmgResidual on the finest level (kernels.cl:2008-2053, spacing 1):
//       r_c = -|f0|^2 f0_c - (mu * (sum of 6 neighbours - 6 v_c) - |f0|^2 v_c)
// each evaluated at the mirrored position of every voxel, in FP32 in the
// reference's operation order, exactly like the kernels that produce these
// values.  The squares are accumulated in FP64: a product of two floats is
// exact in double, each block sums its threads' terms in a fixed tree order
// and one thread sums the blocks in block order, so the norms do not depend
// on scheduling and repeat bit for bit.  The grid has a fixed size for a given
// volume (not derived from the device), so they also agree between devices.
#include "tsf_common.cuh"

namespace tsf {

constexpr int kResThreads = 256;
constexpr int kResMaxBlocks = 1024;

// Component c of voxel p of a planar (3 planes of n) or field4 field.
template <int ST, bool F4> __device__ __forceinline__ float res_load(const void *base, int64_t n, int64_t p, int c) {
    using T = typename Store<ST>::T;
    const T *b = static_cast<const T *>(base);
    return Store<ST>::load(__ldg(F4 ? b + 4 * p + c : b + c * n + p));
}

template <int ST, bool F4, int KIND>
__global__ void __launch_bounds__(kResThreads) residual_kernel(const void *__restrict__ f0, const void *__restrict__ v,
                                                               int X, int Y, int Z, float mu,
                                                               double *__restrict__ part) {
    const int64_t n = (int64_t)X * Y * Z;
    const int64_t sx = 1, sy = X, sz = (int64_t)X * Y;
    double acc[3] = {0.0, 0.0, 0.0};
    float amax = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % X);
        const int64_t yz = i / X;
        const int y = (int)(yz % Y), z = (int)(yz / Y);
        const int64_t p = lin(mirror(x, X), mirror(y, Y), mirror(z, Z), X, Y);
        const float fx = res_load<ST, F4>(f0, n, p, 0), fy = res_load<ST, F4>(f0, n, p, 1),
                    fz = res_load<ST, F4>(f0, n, p, 2);
        const float sqr = (fx * fx + fy * fy) + fz * fz;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float vc = res_load<ST, F4>(v, n, p, c);
            const float xp = res_load<ST, F4>(v, n, p + sx, c), xm = res_load<ST, F4>(v, n, p - sx, c);
            const float yp = res_load<ST, F4>(v, n, p + sy, c), ym = res_load<ST, F4>(v, n, p - sy, c);
            const float zp = res_load<ST, F4>(v, n, p + sz, c), zm = res_load<ST, F4>(v, n, p - sz, c);
            const float fc = c == 0 ? fx : (c == 1 ? fy : fz);
            float r;
            if (KIND == 0) {
                float lap = -6.0f * vc;
                lap = lap + xp;
                lap = lap + xm;
                lap = lap + yp;
                lap = lap + ym;
                lap = lap + zp;
                lap = lap + zm;
                r = mu * lap - (vc - fc) * sqr;
            } else {
                float s6 = xp + xm;
                s6 = s6 + yp;
                s6 = s6 + ym;
                s6 = s6 + zp;
                s6 = s6 + zm;
                const float residue = (mu * (s6 - 6.0f * vc)) / 1.0f;
                r = -sqr * fc - (residue - sqr * vc);
            }
            acc[c] += (double)r * (double)r;
            amax = fmaxf(amax, fabsf(r));
        }
    }
    // block reduction in a fixed order: warps by shuffles, then warp 0
    __shared__ double sacc[3][kResThreads / 32];
    __shared__ float smax[kResThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 3; c++)
        for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_down_sync(0xffffffffu, acc[c], o);
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_down_sync(0xffffffffu, amax, o));
    if (lane == 0) {
        for (int c = 0; c < 3; c++) sacc[c][w] = acc[c];
        smax[w] = amax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[3] = {0.0, 0.0, 0.0};
        float m = 0.0f;
        for (int k = 0; k < kResThreads / 32; k++) {
            for (int c = 0; c < 3; c++) s[c] += sacc[c][k];
            m = fmaxf(m, smax[k]);
        }
        for (int c = 0; c < 3; c++) part[4 * blockIdx.x + c] = s[c];
        part[4 * blockIdx.x + 3] = (double)m;
    }
}

// out: sqrt of the per-component sums, of their total, and the max |r|.
__global__ void residual_final_kernel(const double *__restrict__ part, int nblocks, double *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[3] = {0.0, 0.0, 0.0}, m = 0.0;
    for (int b = 0; b < nblocks; b++) {
        for (int c = 0; c < 3; c++) s[c] += part[4 * b + c];
        m = fmax(m, part[4 * b + 3]);
    }
    out[0] = sqrt(s[0]);
    out[1] = sqrt(s[1]);
    out[2] = sqrt(s[2]);
    out[3] = sqrt((s[0] + s[1]) + s[2]);
    out[4] = m;
}

size_t residual_workspace_size() { return (size_t)(4 * kResMaxBlocks + 8) * sizeof(double); }

static int residual_blocks(int64_t n) {
    const int64_t b = (n + kResThreads - 1) / kResThreads;
    return (int)(b < kResMaxBlocks ? b : kResMaxBlocks);
}

// Launches the reduction; the five norms land in device memory at
// ws + 4 * kResMaxBlocks doubles (read by the caller after the stream).
int launch_residual(const void *d_f0, const void *d_v, int X, int Y, int Z, float mu, int st, int kind, int layout,
                    void *ws, size_t ws_bytes, cudaStream_t s, double **d_out) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_v) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (kind != 0 && kind != 1) return fail(TSF_ERR_INVALID_ARG, "residual kind must be 0 (Jacobi) or 1 (FMG)");
    if (layout != 0 && layout != 1) return fail(TSF_ERR_INVALID_ARG, "layout must be 0 (planar) or 1 (field4)");
    if (!ws || ws_bytes < residual_workspace_size() || (reinterpret_cast<uintptr_t>(ws) & 7))
        return fail(TSF_ERR_WORKSPACE, "residual workspace too small or misaligned");
    const int64_t n = (int64_t)X * Y * Z;
    const int nb = residual_blocks(n);
    double *part = static_cast<double *>(ws);
    double *out = part + 4 * kResMaxBlocks;
#define TSF_RES_LAUNCH(F4, K) residual_kernel<ST, F4, K><<<nb, kResThreads, 0, s>>>(d_f0, d_v, X, Y, Z, mu, part)
    TSF_DISPATCH_STORAGE(st, ST, {
        if (layout) {
            if (kind) TSF_RES_LAUNCH(true, 1); else TSF_RES_LAUNCH(true, 0);
        } else {
            if (kind) TSF_RES_LAUNCH(false, 1); else TSF_RES_LAUNCH(false, 0);
        }
    });
#undef TSF_RES_LAUNCH
    residual_final_kernel<<<1, 32, 0, s>>>(part, nb, out);
    TSF_CHECK_LAUNCHES("residual kernels", 2);
    *d_out = out;
    return TSF_OK;
}

int run_residual_norm(const void *d_f0, const void *d_v, int X, int Y, int Z, float mu, int st, int kind, int layout,
                      double *norms, void *ws, size_t ws_bytes, cudaStream_t s) {
    if (!norms) return fail(TSF_ERR_INVALID_ARG, "null norms");
    double *d_out = nullptr;
    int r = launch_residual(d_f0, d_v, X, Y, Z, mu, st, kind, layout, ws, ws_bytes, s, &d_out);
    if (r) return r;
    TSF_TRY_CUDA(cudaMemcpyAsync(norms, d_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
    TSF_TRY_CUDA(cudaStreamSynchronize(s));
    return TSF_OK;
}

size_t gvf_workspace_size(int X, int Y, int Z, int st);
int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st, void *ws,
            size_t ws_bytes, int mode, cudaStream_t s);

size_t gvf_converge_workspace_size(int X, int Y, int Z, int st) {
    return (gvf_workspace_size(X, Y, Z, st) + 255) / 256 * 256 + residual_workspace_size();
}

// Jacobi GVF in chunks of check_every iterations; after each chunk the RMS of
// the next update, sqrt(sum_c |r_c|^2 / (3N)) (kind 0), is compared with the
// tolerance.  Stops at the first chunk end where it is <= tolerance, or after
// max_iterations.
int run_gvf_converge(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int max_iterations, int check_every,
                     double tolerance, int st, int *iterations_done, double *rms, void *ws, size_t ws_bytes,
                     cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (max_iterations < 0 || check_every < 1) return fail(TSF_ERR_INVALID_ARG, "need max_iterations >= 0, check_every >= 1");
    if (!(tolerance >= 0.0)) return fail(TSF_ERR_INVALID_ARG, "tolerance must be >= 0");
    const size_t gws = (gvf_workspace_size(X, Y, Z, st) + 255) / 256 * 256;
    if (!ws || ws_bytes < gvf_converge_workspace_size(X, Y, Z, st))
        return fail(TSF_ERR_WORKSPACE, "GVF convergence workspace too small");
    void *rws = static_cast<char *>(ws) + gws;
    const double n3 = 3.0 * (double)X * Y * Z;
    int done = 0;
    double norms[5] = {0, 0, 0, 0, 0};
    for (;;) {
        r = run_residual_norm(d_f0, d_v, X, Y, Z, mu, st, 0, 0, norms, rws, residual_workspace_size(), s);
        if (r) return r;
        const double cur = norms[3] / sqrt(n3);
        if (rms) *rms = cur;
        if (iterations_done) *iterations_done = done;
        if (cur <= tolerance || done >= max_iterations) break;
        const int k = check_every < max_iterations - done ? check_every : max_iterations - done;
        r = run_gvf(d_f0, d_v, X, Y, Z, mu, k, st, ws, gws, 0, s);
        if (r) return r;
        done += k;
    }
    return (done >= max_iterations && norms[3] / sqrt(n3) > tolerance) ? TSF_ERR_NOT_CONVERGED : TSF_OK;
}

}  // namespace tsf

extern "C" size_t tsf_gvf_residual_workspace_size(void) { return tsf::residual_workspace_size(); }

extern "C" int tsf_gvf_residual_norm(const void *d_f0, const void *d_v, int X, int Y, int Z, float mu, int storage,
                                     int kind, int layout, double *norms, void *d_workspace, size_t workspace_bytes,
                                     void *stream) {
    return tsf::run_residual_norm(d_f0, d_v, X, Y, Z, mu, storage, kind, layout, norms, d_workspace, workspace_bytes,
                                  reinterpret_cast<cudaStream_t>(stream));
}

extern "C" size_t tsf_gvf_converge_workspace_size(int X, int Y, int Z, int storage) {
    return tsf::gvf_converge_workspace_size(X, Y, Z, storage);
}

extern "C" int tsf_gvf_converge(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int max_iterations,
                                int check_every, double tolerance, int storage, int *iterations_done,
                                double *residual_rms, void *d_workspace, size_t workspace_bytes, void *stream) {
    return tsf::run_gvf_converge(d_f0, d_v, X, Y, Z, mu, max_iterations, check_every, tolerance, storage,
                                 iterations_done, residual_rms, d_workspace, workspace_bytes,
                                 reinterpret_cast<cudaStream_t>(stream));
}
