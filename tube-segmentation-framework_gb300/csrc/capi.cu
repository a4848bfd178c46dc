// capi.cu -- the extern "C" entry points of libtsf_gb300 (declared in
// include/tsf/tsf_c.h) and the error plumbing they share.
#include <atomic>
#include <cstring>
#include <string>

#include "tsf_common.cuh"

namespace tsf {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int check_cuda(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return TSF_ERR_CUDA;
}

// implemented in the kernel translation units
int host_blur_mask(float sigma, float *mask, int *half_width);
int launch_blur(const float *d_in, float *d_out, int X, int Y, int Z, float sigma, cudaStream_t s);
int launch_vector_field(const float *d_in, int X, int Y, int Z, float fmax, int vsign, int st, void *d_planar,
                        void *d_field4, cudaStream_t s);
size_t gvf_workspace_size(int X, int Y, int Z, int st);
int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st, void *ws,
            size_t ws_bytes, int mode, cudaStream_t s);
int launch_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int st, cudaStream_t s);
size_t gvf_one_workspace_size(int X, int Y, int Z, int st);
int run_gvf_one_component(const void *d_field4_in, int X, int Y, int Z, float mu, int iterations, int st,
                          void *d_field4_out, void *ws, size_t ws_bytes, cudaStream_t s);
int launch_tdf_circle(const void *d_field4, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                      void *d_T, int unorm, float *d_R, cudaStream_t s, int tdf_mode, void *ws = nullptr,
                      size_t ws_bytes = 0, int samples = 32, int stride = 1, int eigen = 0);
size_t tdf_workspace_size(int X, int Y, int Z, int st);
int launch_tdf_combine(const void *Ts, const float *Rs, void *Tl, float *Rl, int64_t n, int unorm, cudaStream_t s);
size_t candidates_workspace_size(int X, int Y, int Z);
size_t compact_workspace_size(int X, int Y, int Z);
int run_compact_mask(const int8_t *mask, int X, int Y, int Z, int32_t *pos, int64_t cap, int64_t *count, void *ws,
                     size_t ws_bytes, cudaStream_t s);
int run_candidates(const void *T, int unorm, const float *R, const void *F, int st, int X, int Y, int Z,
                   float tdf_high, int cube_size, int32_t *vertices, int64_t max_vertices, int8_t *centerpoints,
                   int32_t *cand_out, int64_t max_cand, int64_t *n_cand, int64_t *n_vert, void *ws, size_t ws_bytes,
                   cudaStream_t s);
size_t fmg_workspace_size(int X, int Y, int Z, int st);
int run_fmg(const void *f4_in, void *f4_out, int X, int Y, int Z, float mu, int iterations, int st, void *ws,
            size_t ws_bytes, cudaStream_t s);

}  // namespace tsf

using namespace tsf;

static inline cudaStream_t S(void *p) { return reinterpret_cast<cudaStream_t>(p); }

extern "C" {

int tsf_abi_version(void) { return TSF_ABI_VERSION; }

const char *tsf_last_error_string(void) { return g_last_error.c_str(); }

size_t tsf_storage_bytes(int storage) { return storage_bytes(storage); }

unsigned long long tsf_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int tsf_blur_mask(float sigma, float *mask_out, int *half_width) {
    if (!mask_out || !half_width) return fail(TSF_ERR_INVALID_ARG, "null pointer");
    return host_blur_mask(sigma, mask_out, half_width);
}

int tsf_blur(const float *d_in, float *d_out, int X, int Y, int Z, float sigma, void *stream) {
    return launch_blur(d_in, d_out, X, Y, Z, sigma, S(stream));
}

int tsf_vector_field(const float *d_in, int X, int Y, int Z, float fmax, int vsign, int storage, void *d_planar,
                     void *d_field4, void *stream) {
    return launch_vector_field(d_in, X, Y, Z, fmax, vsign, storage, d_planar, d_field4, S(stream));
}

size_t tsf_gvf_workspace_size(int X, int Y, int Z, int storage) {
    if (!valid_storage(storage) || X <= 0 || Y <= 0 || Z <= 0) return 0;
    return gvf_workspace_size(X, Y, Z, storage);
}

int tsf_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int storage,
            void *d_workspace, size_t workspace_bytes, void *stream) {
    return run_gvf(d_f0, d_v, X, Y, Z, mu, iterations, storage, d_workspace, workspace_bytes, 0, S(stream));
}

// Same as tsf_gvf with a forced kernel choice (0 = default, 1 = the
// register-vector / per-voxel kernels, 2 = same as 0).  Used by the tests to
// show every kernel gives one result.
int tsf_gvf_mode(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int storage,
                 void *d_workspace, size_t workspace_bytes, int mode, void *stream) {
    return run_gvf(d_f0, d_v, X, Y, Z, mu, iterations, storage, d_workspace, workspace_bytes, mode, S(stream));
}

int tsf_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int storage, void *stream) {
    return launch_gvf_finish(d_v, d_field4, X, Y, Z, storage, S(stream));
}

size_t tsf_gvf_one_component_workspace_size(int X, int Y, int Z, int storage) {
    if (!valid_storage(storage) || X <= 0 || Y <= 0 || Z <= 0) return 0;
    return gvf_one_workspace_size(X, Y, Z, storage);
}

int tsf_gvf_one_component(const void *d_field4_in, int X, int Y, int Z, float mu, int iterations, int storage,
                          void *d_field4_out, void *d_workspace, size_t workspace_bytes, void *stream) {
    return run_gvf_one_component(d_field4_in, X, Y, Z, mu, iterations, storage, d_field4_out, d_workspace,
                                 workspace_bytes, S(stream));
}

int tsf_tdf_circle(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax, float rstep,
                   void *d_T, int tdf_unorm16, float *d_R, void *stream) {
    return launch_tdf_circle(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_T, tdf_unorm16, d_R, S(stream), 0);
}

size_t tsf_tdf_workspace_size(int X, int Y, int Z, int storage) { return tdf_workspace_size(X, Y, Z, storage); }

int tsf_tdf_circle_ws(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax, float rstep,
                      void *d_T, int tdf_unorm16, float *d_R, void *d_workspace, size_t workspace_bytes,
                      void *stream) {
    return launch_tdf_circle(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_T, tdf_unorm16, d_R, S(stream), 0,
                             d_workspace, workspace_bytes);
}

int tsf_tdf_circle_ex(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax, float rstep,
                      const tsf_tdf_options *options, void *d_T, int tdf_unorm16, float *d_R, void *d_workspace,
                      size_t workspace_bytes, void *stream) {
    const tsf_tdf_options def = {32, 1, 0, 0};
    const tsf_tdf_options &o = options ? *options : def;
    if (o.kernel < 0 || o.kernel > 3) return fail(TSF_ERR_INVALID_ARG, "kernel must be 0, 1, 2 or 3");
    return launch_tdf_circle(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_T, tdf_unorm16, d_R, S(stream),
                             o.kernel, d_workspace, workspace_bytes, o.samples, o.stride, o.eigen);
}

// tsf_tdf_circle with the kernel forced (0 = default, 1 = one voxel per lane).
int tsf_tdf_circle_mode(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax, float rstep,
                        void *d_T, int tdf_unorm16, float *d_R, int mode, void *stream) {
    return launch_tdf_circle(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_T, tdf_unorm16, d_R, S(stream), mode);
}

int tsf_tdf_combine(const void *d_T_small, const float *d_R_small, void *d_T_large, float *d_R_large, int64_t n,
                    int tdf_unorm16, void *stream) {
    return launch_tdf_combine(d_T_small, d_R_small, d_T_large, d_R_large, n, tdf_unorm16, S(stream));
}

size_t tsf_candidates_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return candidates_workspace_size(X, Y, Z);
}

int tsf_candidates(const void *d_T, int tdf_unorm16, const float *d_R, const void *d_field4, int storage, int X,
                   int Y, int Z, float tdf_high, int cube_size, int32_t *d_vertices, int64_t max_vertices,
                   int8_t *d_centerpoints, int32_t *d_candidates, int64_t max_candidates, int64_t *n_candidates,
                   int64_t *n_vertices, void *d_workspace, size_t workspace_bytes, void *stream) {
    return run_candidates(d_T, tdf_unorm16, d_R, d_field4, storage, X, Y, Z, tdf_high, cube_size, d_vertices,
                          max_vertices, d_centerpoints, d_candidates, max_candidates, n_candidates, n_vertices,
                          d_workspace, workspace_bytes, S(stream));
}

size_t tsf_compact_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return compact_workspace_size(X, Y, Z);
}

int tsf_compact_mask(const int8_t *d_mask, int X, int Y, int Z, int32_t *d_positions, int64_t max_positions,
                     int64_t *count, void *d_workspace, size_t workspace_bytes, void *stream) {
    return run_compact_mask(d_mask, X, Y, Z, d_positions, max_positions, count, d_workspace, workspace_bytes,
                            S(stream));
}

size_t tsf_gvf_fmg_workspace_size(int X, int Y, int Z, int storage) {
    if (!valid_storage(storage) || X <= 0 || Y <= 0 || Z <= 0) return 0;
    return fmg_workspace_size(X, Y, Z, storage);
}

int tsf_gvf_fmg(const void *d_field4_in, void *d_field4_out, int X, int Y, int Z, float mu, int iterations,
                int storage, void *d_workspace, size_t workspace_bytes, void *stream) {
    return run_fmg(d_field4_in, d_field4_out, X, Y, Z, mu, iterations, storage, d_workspace, workspace_bytes,
                   S(stream));
}

}  // extern "C"
