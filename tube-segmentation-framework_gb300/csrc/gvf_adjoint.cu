// gvf_adjoint.cu -- reverse-mode derivative of K GVF Jacobi iterations with
// respect to the data term f0 and to mu (no counterpart in the reference,
// which has no derivatives).
//
// Forward map of one iteration, per component c, at output w with p = m(w)
// (the mirror rule, applied per axis: 0 -> 2, size-1 -> size-3):
//     v'_c[w] = v_c[p] + mu * L(v_c)[p] - (v_c[p] - f_c[p]) * s[p],
//     L(u)[p] = sum_{6 neighbours q} u[q] - 6 u[p],   s = |f|^2.
// Given lambda' = dL/dv', with g = fold(lambda'), g[p] = sum_{w : m(w) = p} lambda'[w]
// (zero outside the interior [1, size-2]^3, the image of m):
//     lambda_c[q] = g_c[q] (1 - 6 mu - s[q]) + mu * sum_{6 neighbours r of q} g_c[r]
//     dL/df_c[q] += g_c[q] s[q] - 2 f_c[q] sum_d g_d[q] (v_d[q] - f_d[q])
//     dL/dmu    += sum_c sum_q g_c[q] L(v_c)[q]
// and, since v_0 = f0 (GVF3DInit), dL/df0 += lambda_0 at the end.
// Storage rounding of the forward states is treated as the identity.
//
// Checkpointing: the forward states v_C, v_2C, ... are kept (v_0 is f0; C =
// checkpoint interval, ceil(sqrt(K)) by default); each segment is recomputed
// from its checkpoint into a (C-1)-state buffer and then reversed, so the
// memory is about K/C + C states and the extra work at most one forward pass.
// The last segment's states are left in the buffer by the forward pass, and
// C = 1 (every state kept, K-1 states: 100 GB for 500 FP32 iterations at
// 256^3, which fits GB300's HBM) recomputes nothing.  Cotangents are FP32;
// the mu derivative is accumulated in FP64, per block in a fixed order, so the
// result does not depend on scheduling.
#include "tsf_common.cuh"

namespace tsf {

int gvf_step(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu, cudaStream_t s);
bool gvf_adjoint_zs_eligible(int st, const void *g, const void *v, const void *f, const void *gf, const void *lam,
                             int X);
int gvf_adjoint_zs_max_grid();
int launch_gvf_adjoint_zs(int st, const float *g, const void *v, const void *f, float *lam_out, float *gf,
                          double *dmu_block, int X, int Y, int Z, float mu, cudaStream_t s);

// folded cotangent at (x, y, z): sum of lambda' over the voxels that mirror to it
__device__ __forceinline__ float fold_at(const float *__restrict__ lp, int x, int y, int z, int X, int Y, int Z) {
    if (x < 1 || y < 1 || z < 1 || x > X - 2 || y > Y - 2 || z > Z - 2) return 0.0f;
    int xs[2] = {x, 0}, ys[2] = {y, 0}, zs[2] = {z, 0};
    int nx = 1, ny = 1, nz = 1;
    if (x == 2) xs[nx++] = 0;
    else if (x == X - 3) xs[nx++] = X - 1;
    if (y == 2) ys[ny++] = 0;
    else if (y == Y - 3) ys[ny++] = Y - 1;
    if (z == 2) zs[nz++] = 0;
    else if (z == Z - 3) zs[nz++] = Z - 1;
    // X == 5: index 2 is both 2 and X-3 -> sources 0, 2, 4
    int xs3 = -1, ys3 = -1, zs3 = -1;
    if (x == 2 && X - 3 == 2) xs3 = X - 1;
    if (y == 2 && Y - 3 == 2) ys3 = Y - 1;
    if (z == 2 && Z - 3 == 2) zs3 = Z - 1;
    float g = 0.0f;
    for (int c = 0; c < nz + (zs3 >= 0); c++) {
        const int zz = c < nz ? zs[c] : zs3;
        for (int b = 0; b < ny + (ys3 >= 0); b++) {
            const int yy = b < ny ? ys[b] : ys3;
            for (int a = 0; a < nx + (xs3 >= 0); a++) {
                const int xx = a < nx ? xs[a] : xs3;
                g += lp[lin(xx, yy, zz, X, Y)];
            }
        }
    }
    return g;
}

template <int ST>
__global__ void __launch_bounds__(256) gvf_adjoint_step_kernel(const float *__restrict__ lam_in,
                                                               const typename Store<ST>::T *__restrict__ v,
                                                               const typename Store<ST>::T *__restrict__ f,
                                                               float *__restrict__ lam_out, float *__restrict__ gf,
                                                               double *__restrict__ dmu_block, int X, int Y, int Z,
                                                               float mu) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    const bool in = x < X && y < Y && z < Z;
    const int64_t n = (int64_t)X * Y * Z;
    double dmu = 0.0;
    if (in) {
        const int64_t q = lin(x, y, z, X, Y);
        float fv[3], vv[3], g[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            fv[c] = Store<ST>::load(f[c * n + q]);
            vv[c] = Store<ST>::load(v[c * n + q]);
        }
        const float s = (fv[0] * fv[0] + fv[1] * fv[1]) + fv[2] * fv[2];
        const bool interior = x >= 1 && y >= 1 && z >= 1 && x <= X - 2 && y <= Y - 2 && z <= Z - 2;
        float gdot = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float *lp = lam_in + c * n;
            g[c] = fold_at(lp, x, y, z, X, Y, Z);
            float nb = 0.0f;
            nb += fold_at(lp, x + 1, y, z, X, Y, Z);
            nb += fold_at(lp, x - 1, y, z, X, Y, Z);
            nb += fold_at(lp, x, y + 1, z, X, Y, Z);
            nb += fold_at(lp, x, y - 1, z, X, Y, Z);
            nb += fold_at(lp, x, y, z + 1, X, Y, Z);
            nb += fold_at(lp, x, y, z - 1, X, Y, Z);
            lam_out[c * n + q] = g[c] * (1.0f - 6.0f * mu - s) + mu * nb;
            gdot += g[c] * (vv[c] - fv[c]);
            if (interior && g[c] != 0.0f) {
                const typename Store<ST>::T *vc = v + c * n;
                const int64_t sx = 1, sy = X, sz = (int64_t)X * Y;
                float L = Store<ST>::load(vc[q + sx]) + Store<ST>::load(vc[q - sx]);
                L += Store<ST>::load(vc[q + sy]) + Store<ST>::load(vc[q - sy]);
                L += Store<ST>::load(vc[q + sz]) + Store<ST>::load(vc[q - sz]);
                L -= 6.0f * vv[c];
                dmu += (double)g[c] * (double)L;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) gf[c * n + q] += g[c] * s - 2.0f * fv[c] * gdot;
    }
    // deterministic per-block reduction of the mu derivative
    __shared__ double red[32];
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmu += __shfl_down_sync(0xffffffffu, dmu, o);
    if ((t & 31) == 0) red[t >> 5] = dmu;
    __syncthreads();
    if (t == 0) {
        const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) / 32;
        double sum = 0.0;
        for (int i = 0; i < nw; i++) sum += red[i];
        const int64_t b = blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
        dmu_block[b] += sum;
    }
}

// In-place fold of the cotangent along one axis: the mirror rule sends the
// update computed at 2 to index 0 and the one at size-3 to size-1, so
// g[2] += g[0], g[size-3] += g[size-1], and g[0] = g[size-1] = 0.  Applied to
// x, then y, then z it turns lambda' into fold(lambda') (the rule is separable).
// One thread per (component, face position); only the boundary planes move.
__global__ void fold_axis_kernel(float *__restrict__ g, int X, int Y, int Z, int axis) {
    pdl_trigger();
    pdl_wait();                     // launched with pdl_config: the previous kernel wrote g
    const int64_t n = (int64_t)X * Y * Z;
    int A, B;                       // extents of the face
    int64_t sa, sb, sn;             // strides: face coordinates, folded axis
    int E;                          // folded extent
    if (axis == 0) { A = Y; B = Z; sa = X; sb = (int64_t)X * Y; sn = 1; E = X; }
    else if (axis == 1) { A = X; B = Z; sa = 1; sb = (int64_t)X * Y; sn = X; E = Y; }
    else { A = X; B = Y; sa = 1; sb = X; sn = (int64_t)X * Y; E = Z; }
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)3 * A * B) return;
    const int c = (int)(t / ((int64_t)A * B));
    const int64_t r = t % ((int64_t)A * B);
    const int a = (int)(r % A), b = (int)(r / A);
    float *p = g + c * n + a * sa + b * sb;
    const float g0 = p[0], gl = p[(E - 1) * sn];
    p[2 * sn] += g0;
    p[(E - 3) * sn] += gl;
    p[0] = 0.0f;
    p[(E - 1) * sn] = 0.0f;
}

// Adjoint stencil on the folded cotangent g (zero outside [1, size-2] per
// axis), 4 consecutive voxels per thread, FP32 cotangents in 16-byte vectors,
// x-neighbours by shuffles, neighbours outside the volume read as 0:
//     lambda = g (1 - 6 mu - s) + mu sum_6 g,   gf += g s - 2 f sum_d g_d (v_d - f_d),
//     dmu += sum_c g_c L(v_c)   (L with clamped reads: g = 0 wherever L would clamp).
template <int ST>
__global__ void __launch_bounds__(256, 3) gvf_adjoint_stencil_kernel(const float *__restrict__ gin,
                                                                  const typename Store<ST>::T *__restrict__ v,
                                                                  const typename Store<ST>::T *__restrict__ f,
                                                                  float *__restrict__ lam_out, float *__restrict__ gf,
                                                                  double *__restrict__ dmu_block, int X, int Y, int Z,
                                                                  float mu) {
    using T = typename Store<ST>::T;
    constexpr int VX = 4;
    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const int x0 = (blockIdx.x * 32 + lane) * VX;
    const bool act = y < Y && x0 < X;
    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    const unsigned full = 0xffffffffu;
    const int64_t q = (int64_t)z * plane + (int64_t)(act ? y : 0) * X + (act ? x0 : 0);
    const bool hy0 = y > 0, hy1 = y < Y - 1, hz0 = z > 0, hz1 = z < Z - 1;
    double dmu = 0.0;
    float fv[3][VX], s[VX], gd[VX], gc[3][VX];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int i = 0; i < VX; i++) fv[c][i] = act ? Store<ST>::load(f[c * n + q + i]) : 0.0f;
#pragma unroll
    for (int i = 0; i < VX; i++) {
        s[i] = (fv[0][i] * fv[0][i] + fv[1][i] * fv[1][i]) + fv[2][i] * fv[2][i];
        gd[i] = 0.0f;
    }
    auto ld4 = [&](const float *p, bool ok, float o[VX]) {
        if (ok) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
            o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
        } else {
            o[0] = o[1] = o[2] = o[3] = 0.0f;
        }
    };
    auto ldv = [&](const T *p, bool ok, float o[VX]) {
#pragma unroll
        for (int i = 0; i < VX; i++) o[i] = ok ? Store<ST>::load(p[i]) : 0.0f;
    };
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float *gp = gin + c * n + q;
        const T *vp = v + c * n + q;
        float g[VX], gyp[VX], gym[VX], gzp[VX], gzm[VX], vv[VX], vyp[VX], vym[VX], vzp[VX], vzm[VX];
        ld4(gp, act, g);
        ld4(gp + X, act && hy1, gyp);
        ld4(gp - X, act && hy0, gym);
        ld4(gp + plane, act && hz1, gzp);
        ld4(gp - plane, act && hz0, gzm);
        ldv(vp, act, vv);
        ldv(vp + X, act && hy1, vyp);
        ldv(vp - X, act && hy0, vym);
        ldv(vp + plane, act && hz1, vzp);
        ldv(vp - plane, act && hz0, vzm);
        float gl = __shfl_up_sync(full, g[VX - 1], 1), gr = __shfl_down_sync(full, g[0], 1);
        float vl = __shfl_up_sync(full, vv[VX - 1], 1), vr = __shfl_down_sync(full, vv[0], 1);
        if (lane == 0) {
            gl = (act && x0 > 0) ? gp[-1] : 0.0f;
            vl = (act && x0 > 0) ? Store<ST>::load(vp[-1]) : 0.0f;
        }
        if (lane == 31 || x0 + VX >= X) {
            gr = (act && x0 + VX < X) ? gp[VX] : 0.0f;
            vr = (act && x0 + VX < X) ? Store<ST>::load(vp[VX]) : 0.0f;
        }
        float out[VX];
#pragma unroll
        for (int i = 0; i < VX; i++) {
            const float xp = i == VX - 1 ? gr : g[i + 1 < VX ? i + 1 : i];
            const float xm = i == 0 ? gl : g[i > 0 ? i - 1 : 0];
            const float nb = ((((xp + xm) + gyp[i]) + gym[i]) + gzp[i]) + gzm[i];
            out[i] = g[i] * (1.0f - 6.0f * mu - s[i]) + mu * nb;
            const float vxp = i == VX - 1 ? vr : vv[i + 1 < VX ? i + 1 : i];
            const float vxm = i == 0 ? vl : vv[i > 0 ? i - 1 : 0];
            const float L = (((((vxp + vxm) + vyp[i]) + vym[i]) + vzp[i]) + vzm[i]) - 6.0f * vv[i];
            dmu += (double)(g[i] * L);
            gd[i] += g[i] * (vv[i] - fv[c][i]);
            gc[c][i] = g[i];
        }
        if (act) *reinterpret_cast<float4 *>(lam_out + c * n + q) = make_float4(out[0], out[1], out[2], out[3]);
    }
    if (act) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float4 *gp = reinterpret_cast<float4 *>(gf + c * n + q);
            float4 a = *gp;
            a.x += gc[c][0] * s[0] - 2.0f * fv[c][0] * gd[0];
            a.y += gc[c][1] * s[1] - 2.0f * fv[c][1] * gd[1];
            a.z += gc[c][2] * s[2] - 2.0f * fv[c][2] * gd[2];
            a.w += gc[c][3] * s[3] - 2.0f * fv[c][3] * gd[3];
            *gp = a;
        }
    }
    __shared__ double red[8];
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmu += __shfl_down_sync(full, dmu, o);
    if ((t & 31) == 0) red[t >> 5] = dmu;
    __syncthreads();
    if (t == 0) {
        double sum = 0.0;
        for (int i = 0; i < (int)(blockDim.x * blockDim.y) / 32; i++) sum += red[i];
        dmu_block[blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z)] += sum;
    }
}

__global__ void add_planar_kernel(float *__restrict__ a, const float *__restrict__ b, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += b[i];
}

__global__ void reduce_double_kernel(const double *__restrict__ in, int64_t n, double *out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += in[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x / 32); i++) t += red[i];
        *out = t;
    }
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

struct AdjLayout {
    int C, nck;
    size_t state, ck, seg, lam0, lam1, dmu, dmu_out, bytes;
    int64_t nblocks;
};

static bool adj_vec(int X) { return X % 4 == 0; }
static dim3 adj_block() { return dim3(32, 4, 2); }
static dim3 adj_grid(int X, int Y, int Z) { return dim3((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2); }
static dim3 adjv_block() { return dim3(32, 8, 1); }
static dim3 adjv_grid(int X, int Y, int Z) { return dim3((X / 4 + 31) / 32, (Y + 7) / 8, Z); }

static int default_interval(int K) {
    int C = 1;
    while (C * C < K) C++;
    return C;
}

// Workspace: checkpoints v_C, v_2C, ... (v_0 is f0 itself), a segment buffer
// for the C - 1 states after a checkpoint, two cotangent buffers and the mu
// partials.  C = 1 keeps every state and recomputes nothing.
static AdjLayout adj_layout(int X, int Y, int Z, int st, int K, int C) {
    AdjLayout L;
    if (C <= 0) C = default_interval(K);
    L.C = C;
    L.nck = K > 0 ? (K + C - 1) / C : 0;
    const size_t n = (size_t)X * Y * Z;
    L.state = al256(3 * n * storage_bytes(st));
    const dim3 g = adj_grid(X, Y, Z), gv = adjv_grid(X, Y, Z);
    // partials: the per-voxel kernel's blocks, then the vector or streaming kernel's
    const int64_t nv = adj_vec(X) ? (int64_t)gv.x * gv.y * gv.z : 0, nz = gvf_adjoint_zs_max_grid();
    L.nblocks = (int64_t)g.x * g.y * g.z + (nv > nz ? nv : nz);
    size_t off = 0;
    L.ck = off; off += L.state * (size_t)(L.nck > 1 ? L.nck - 1 : 0);
    L.seg = off; off += L.state * (size_t)(C - 1);
    L.lam0 = off; off += al256(3 * n * sizeof(float));
    L.lam1 = off; off += al256(3 * n * sizeof(float));
    L.dmu = off; off += al256(sizeof(double) * (size_t)L.nblocks);
    L.dmu_out = off; off += 256;
    L.bytes = off;
    return L;
}

size_t gvf_adjoint_workspace_size(int X, int Y, int Z, int st, int K, int C) {
    return adj_layout(X, Y, Z, st, K, C).bytes;
}

// Smallest checkpoint interval whose workspace fits `budget` bytes (1 = keep
// every state); 0 if even the smallest workspace does not fit.
int gvf_adjoint_interval(int X, int Y, int Z, int st, int K, size_t budget) {
    if (K <= 0) return 1;
    for (int C = 1; C <= K; C++) {
        if (adj_layout(X, Y, Z, st, K, C).bytes <= budget) return C;
        if ((int64_t)C * C > 4 * (int64_t)K) break;   // past the minimum near sqrt(K)
    }
    return 0;
}

// state k of the segment that starts at checkpoint i (k = i*C + t)
static inline const void *ck_state(const AdjLayout &L, const void *d_f0, char *w, int i) {
    return i == 0 ? d_f0 : (const void *)(w + L.ck + (size_t)(i - 1) * L.state);
}
static inline void *seg_state(const AdjLayout &L, char *w, int t) {   // t = 1 .. C-1
    return w + L.seg + (size_t)(t - 1) * L.state;
}

// Forward pass storing the checkpoints v_C, v_2C, ... and the states of the
// last segment; v_K goes to d_v (may be NULL).  Every state is written once,
// straight into its slot.
int run_gvf_checkpointed(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int K, int st, int C, void *ws,
                         size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (K < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    const AdjLayout L = adj_layout(X, Y, Z, st, K, C);
    if (!ws || ws_bytes < L.bytes) return fail(TSF_ERR_WORKSPACE, "GVF adjoint workspace too small");
    char *w = (char *)ws;
    const size_t state_bytes = 3 * (size_t)X * Y * Z * storage_bytes(st);
    for (int i = 0; i < L.nck; i++) {
        const int k0 = i * L.C, k1 = (k0 + L.C < K) ? k0 + L.C : K;
        const bool last = i == L.nck - 1;
        const void *src = ck_state(L, d_f0, w, i);
        for (int k = k0 + 1; k <= k1; k++) {
            void *dst;
            if (k < k1) dst = seg_state(L, w, k - k0);          // inside the segment
            else if (!last) dst = (void *)ck_state(L, d_f0, w, i + 1);
            else if (d_v) dst = d_v;                            // v_K
            else break;
            r = gvf_step(st, d_f0, src, dst, X, Y, Z, mu, s);
            if (r) return r;
            src = dst;
        }
    }
    if (d_v && L.nck == 0) TSF_TRY_CUDA(cudaMemcpyAsync(d_v, d_f0, state_bytes, cudaMemcpyDeviceToDevice, s));
    return TSF_OK;
}

int run_gvf_adjoint(const void *d_f0, int X, int Y, int Z, float mu, int K, int st, const float *d_gv, float *d_gf0,
                    double *dmu_host, int C, int flags, void *ws, size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_gv || !d_gf0) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (K < 0) return fail(TSF_ERR_INVALID_ARG, "iterations must be >= 0");
    const AdjLayout L = adj_layout(X, Y, Z, st, K, C);
    if (!ws || ws_bytes < L.bytes) return fail(TSF_ERR_WORKSPACE, "GVF adjoint workspace too small");
    char *w = (char *)ws;
    const int64_t n = (int64_t)X * Y * Z;
    float *lam = (float *)(w + L.lam0), *lam2 = (float *)(w + L.lam1);
    double *dmu_b = (double *)(w + L.dmu);
    TSF_TRY_CUDA(cudaMemsetAsync(d_gf0, 0, sizeof(float) * 3 * (size_t)n, s));
    TSF_TRY_CUDA(cudaMemsetAsync(dmu_b, 0, sizeof(double) * (size_t)L.nblocks, s));
    TSF_TRY_CUDA(cudaMemcpyAsync(lam, d_gv, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, s));

    // forward pass storing the checkpoints and the last segment (unless a
    // checkpointed forward with the same arguments already did)
    if (!(flags & 1)) {
        r = run_gvf_checkpointed(d_f0, nullptr, X, Y, Z, mu, K, st, L.C, ws, ws_bytes, s);
        if (r) return r;
    }
    // the cotangent kernels move 16-byte vectors
    const bool vec = adj_vec(X) && ((uintptr_t)d_gf0 & 15) == 0 && ((uintptr_t)w & 15) == 0;
    const bool zs = vec && gvf_adjoint_zs_eligible(st, lam, d_f0, d_f0, d_gf0, lam2, X) &&
                    ((uintptr_t)(w + L.ck) & 15) == 0 && ((uintptr_t)(w + L.seg) & 15) == 0;
    const dim3 g = adj_grid(X, Y, Z);
    double *dmu_v = dmu_b + (int64_t)g.x * g.y * g.z;
    // reverse, one segment at a time
    for (int seg = L.nck - 1; seg >= 0; seg--) {
        const int k0 = seg * L.C, k1 = (k0 + L.C < K) ? k0 + L.C : K;
        // states k0+1 .. k1-1 into the segment buffer (the last segment's are
        // there from the forward pass)
        if (seg != L.nck - 1) {
            const void *src = ck_state(L, d_f0, w, seg);
            for (int k = k0 + 1; k < k1; k++) {
                void *dst = seg_state(L, w, k - k0);
                r = gvf_step(st, d_f0, src, dst, X, Y, Z, mu, s);
                if (r) return r;
                src = dst;
            }
        }
        for (int k = k1 - 1; k >= k0; k--) {
            const void *vk = k == k0 ? ck_state(L, d_f0, w, seg) : (const void *)seg_state(L, w, k - k0);
            if (vec) {
                // fold lambda' in place (boundary planes only; the streaming
                // kernel does the x part itself), then the stencil
                for (int axis = zs ? 1 : 0; axis < 3; axis++) {
                    const int64_t faces = 3 * (axis == 0 ? (int64_t)Y * Z : axis == 1 ? (int64_t)X * Z : (int64_t)X * Y);
                    cudaLaunchAttribute attr[1];
                    const cudaLaunchConfig_t cfg =
                        pdl_config(dim3((unsigned)((faces + 255) / 256)), dim3(256), 0, s, attr);
                    TSF_TRY_CUDA(cudaLaunchKernelEx(&cfg, fold_axis_kernel, lam, X, Y, Z, axis));
                }
                TSF_CHECK_LAUNCHES("fold_axis_kernel", zs ? 2 : 3);
                if (zs) {
                    r = launch_gvf_adjoint_zs(st, lam, vk, d_f0, lam2, d_gf0, dmu_v, X, Y, Z, mu, s);
                    if (r) return r;
                } else {
                    TSF_DISPATCH_STORAGE(st, ST, {
                        using T = typename Store<ST>::T;
                        gvf_adjoint_stencil_kernel<ST><<<adjv_grid(X, Y, Z), adjv_block(), 0, s>>>(
                            lam, (const T *)vk, (const T *)d_f0, lam2, d_gf0, dmu_v, X, Y, Z, mu);
                    });
                    TSF_CHECK_LAUNCH("gvf_adjoint_stencil_kernel");
                }
            } else {
                TSF_DISPATCH_STORAGE(st, ST, {
                    using T = typename Store<ST>::T;
                    gvf_adjoint_step_kernel<ST><<<g, adj_block(), 0, s>>>(lam, (const T *)vk, (const T *)d_f0, lam2,
                                                                         d_gf0, dmu_b, X, Y, Z, mu);
                });
                TSF_CHECK_LAUNCH("gvf_adjoint_step_kernel");
            }
            float *t = lam; lam = lam2; lam2 = t;
        }
    }
    // v_0 = f0
    const int64_t n3 = 3 * n;
    add_planar_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(d_gf0, lam, n3);
    TSF_CHECK_LAUNCH("add_planar_kernel");
    double *dmu_dev = (double *)(w + L.dmu_out);
    reduce_double_kernel<<<1, 1024, 0, s>>>(dmu_b, L.nblocks, dmu_dev);
    TSF_CHECK_LAUNCH("reduce_double_kernel");
    if (dmu_host) {
        TSF_TRY_CUDA(cudaMemcpyAsync(dmu_host, dmu_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
        TSF_TRY_CUDA(cudaStreamSynchronize(s));
    }
    return TSF_OK;
}

}  // namespace tsf

extern "C" size_t tsf_gvf_adjoint_workspace_size(int X, int Y, int Z, int storage, int iterations,
                                                 int checkpoint_every) {
    if (!tsf::valid_storage(storage) || X <= 0 || Y <= 0 || Z <= 0 || iterations < 0) return 0;
    return tsf::gvf_adjoint_workspace_size(X, Y, Z, storage, iterations, checkpoint_every);
}

extern "C" int tsf_gvf_adjoint_checkpoint_interval(int X, int Y, int Z, int storage, int iterations,
                                                   size_t budget_bytes) {
    if (!tsf::valid_storage(storage) || X <= 0 || Y <= 0 || Z <= 0 || iterations < 0) return 0;
    return tsf::gvf_adjoint_interval(X, Y, Z, storage, iterations, budget_bytes);
}

extern "C" int tsf_gvf_adjoint(const void *d_f0, int X, int Y, int Z, float mu, int iterations, int storage,
                               const float *d_gv, float *d_gf0, double *dmu, int checkpoint_every, int flags,
                               void *d_workspace, size_t workspace_bytes, void *stream) {
    return tsf::run_gvf_adjoint(d_f0, X, Y, Z, mu, iterations, storage, d_gv, d_gf0, dmu, checkpoint_every, flags,
                                d_workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_gvf_checkpointed(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
                                    int storage, int checkpoint_every, void *d_workspace, size_t workspace_bytes,
                                    void *stream) {
    return tsf::run_gvf_checkpointed(d_f0, d_v, X, Y, Z, mu, iterations, storage, checkpoint_every, d_workspace,
                                     workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}
