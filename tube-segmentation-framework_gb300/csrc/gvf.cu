// gvf.cu -- gradient vector flow, Jacobi form (reference GVF3DIteration /
// GVF3DFinish, kernels.cl:1464-1515; host loop gradientVectorFlow.cpp:1007-1172).
//
// Layout in HBM: the field v and the data term f0 are planar (three planes of
// N stored components each), so every access is a unit-stride run and a
// voxel-iteration moves exactly 9 stored components: v (3) and f0 (3) read,
// v (3) written -- 36 B in FP32, 18 B in the 16-bit formats.  |f0|^2 is
// recomputed from the stored f0 each time, exactly like the reference (which
// keeps f0z in v.w and f0x,f0y in an RG image).
//
// Two kernels compute the same iteration:
//  * gvf_plain_kernel: one iteration per launch, one thread per voxel, all
//    seven stencil reads through L1/L2.  HBM-bound at 9s B / voxel-iteration.
//  * gvf_tb_kernel: TB iterations per launch (temporal blocking).  A CTA owns
//    an x-y tile and streams through z; each time level keeps one z-plane of
//    the tile (with a halo that shrinks by one voxel per level) in shared
//    memory and its z-1 / z+1 neighbours in registers.  Intermediate levels
//    are rounded to the storage format exactly as a stored iteration would
//    be, so both kernels give bit-identical results.
#include "tsf_common.cuh"

namespace tsf {

// ---------------------------------------------------------------------------
// one iteration per launch
// ---------------------------------------------------------------------------
template <int ST>
__global__ void __launch_bounds__(256) gvf_plain_kernel(const typename Store<ST>::T *__restrict__ f,
                                                        const typename Store<ST>::T *__restrict__ src,
                                                        typename Store<ST>::T *__restrict__ dst,
                                                        int X, int Y, int Z, float mu) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    const int64_t n = (int64_t)X * Y * Z;
    const int px = mirror(x, X), py = mirror(y, Y), pz = mirror(z, Z);
    const int64_t p = lin(px, py, pz, X, Y);
    const int64_t sx = 1, sy = X, sz = (int64_t)X * Y;
    const float fx = Store<ST>::load(__ldg(f + p));
    const float fy = Store<ST>::load(__ldg(f + n + p));
    const float fz = Store<ST>::load(__ldg(f + 2 * n + p));
    const float sqr = (fx * fx + fy * fy) + fz * fz;
    const int64_t o = lin(x, y, z, X, Y);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const typename Store<ST>::T *s = src + c * n;
        const float v = Store<ST>::load(__ldg(s + p));
        float lap = -6.0f * v;
        lap = lap + Store<ST>::load(__ldg(s + p + sx));
        lap = lap + Store<ST>::load(__ldg(s + p - sx));
        lap = lap + Store<ST>::load(__ldg(s + p + sy));
        lap = lap + Store<ST>::load(__ldg(s + p - sy));
        lap = lap + Store<ST>::load(__ldg(s + p + sz));
        lap = lap + Store<ST>::load(__ldg(s + p - sz));
        const float fc = c == 0 ? fx : (c == 1 ? fy : fz);
        const float upd = mu * lap - (v - fc) * sqr;
        dst[c * n + o] = Store<ST>::store(v + upd);
    }
}

// ---------------------------------------------------------------------------
// GVF3DFinish: planar -> field4 with w = |v| (1 if 0)
// ---------------------------------------------------------------------------
template <int ST>
__global__ void gvf_finish_kernel(const typename Store<ST>::T *__restrict__ v, void *field4, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = Store<ST>::load(v[i]), y = Store<ST>::load(v[n + i]), z = Store<ST>::load(v[2 * n + i]);
    const float l = sqrtf((x * x + y * y) + z * z);
    store4<ST>(field4, i, x, y, z, l > 0.0f ? l : 1.0f);
}

// Temporal blocking is not enabled yet: every launch runs one iteration.
static int gvf_tb_levels(int) { return 1; }
static int launch_gvf_tb(int, const void *, const void *, void *, int, int, int, float, int, cudaStream_t) {
    return fail(TSF_ERR_INVALID_ARG, "temporal blocking unavailable");
}

size_t gvf_workspace_size(int X, int Y, int Z, int st) {
    return (size_t)3 * (size_t)X * (size_t)Y * (size_t)Z * storage_bytes(st);
}

static int launch_gvf_plain(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z,
                            float mu, cudaStream_t s) {
    dim3 b(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    TSF_DISPATCH_STORAGE(st, ST, {
        using T = typename Store<ST>::T;
        gvf_plain_kernel<ST><<<g, b, 0, s>>>((const T *)d_f0, (const T *)src, (T *)dst, X, Y, Z, mu);
    });
    TSF_CHECK_LAUNCH("gvf_plain_kernel");
    return TSF_OK;
}

// Runs `iterations` Jacobi iterations in place on d_v.  mode: 0 = choose,
// 1 = one iteration per launch only, 2 = temporal blocking where possible.
int run_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations, int st,
            void *ws, size_t ws_bytes, int mode, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_v) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (iterations < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    if (iterations == 0) return TSF_OK;
    const size_t need = gvf_workspace_size(X, Y, Z, st);
    if (!ws || ws_bytes < need) return fail(TSF_ERR_WORKSPACE, "GVF workspace too small");
    void *a = d_v, *b = ws;
    int left = iterations;
    const int tb = (mode == 1) ? 1 : gvf_tb_levels(st);
    while (left > 0) {
        int k = left >= tb ? tb : left;
        if (k > 1) {
            r = launch_gvf_tb(st, d_f0, a, b, X, Y, Z, mu, k, s);
        } else {
            r = launch_gvf_plain(st, d_f0, a, b, X, Y, Z, mu, s);
        }
        if (r) return r;
        void *t = a; a = b; b = t;
        left -= k;
    }
    if (a != d_v) {
        TSF_TRY_CUDA(cudaMemcpyAsync(d_v, a, need, cudaMemcpyDeviceToDevice, s));
    }
    return TSF_OK;
}

int launch_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int st, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_v || !d_field4) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    const int64_t n = (int64_t)X * Y * Z;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    TSF_DISPATCH_STORAGE(st, ST, {
        using T = typename Store<ST>::T;
        gvf_finish_kernel<ST><<<blocks, threads, 0, s>>>((const T *)d_v, d_field4, n);
    });
    TSF_CHECK_LAUNCH("gvf_finish_kernel");
    return TSF_OK;
}

}  // namespace tsf
