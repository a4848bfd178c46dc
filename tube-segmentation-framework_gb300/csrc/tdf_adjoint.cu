// tdf_adjoint.cu -- reverse-mode derivatives of the TDF, the vector field and
// the Gaussian blur (no counterpart in the reference, which has no
// derivatives).  Together with gvf_adjoint.cu they give dL/dI and dL/dsigma,
// dL/dmu for a loss L on the TDF response.
//
// TDF.  T(x) = max over the swept radii of S(r) = (1/32) sum_j -V(x + r a_j).a_j,
// a_j = cos(j) e3 + sin(j) e2, (e2, e3) eigenvectors of the Hessian H(x) of the
// field.  The sweep's arg-max r* is held fixed (sub-gradient of the max); a
// voxel whose response stayed 0 has zero gradient.  With gS = dL/dT / 32:
//  * texels: dL/dV_t += -gS w_t a_j for the 8 trilinear corners of each sample;
//  * directions: dL/da_j = gS (-V(p_j) - r* J(p_j)^T a_j), J = dV/dp of the
//    trilinear interpolant, so dL/de3 += cos(j) dL/da_j, dL/de2 += sin(j) dL/da_j;
//  * eigenvectors: de_i = sum_{k != i} e_k (e_k^T dH e_i) / (l_i - l_k), so
//    dL/dH = sum_{i in {2,3}} sum_{k != i} (dL/de_i . e_k) / (l_i - l_k) e_k e_i^T
//    (terms with l_i == l_k are skipped: the eigenvectors are not
//    differentiable there);
//  * H entries are central differences of the neighbours' (normalised) field,
//    u = v / |v| when rmax >= 4, so dL/dv = (dL/du - u (u . dL/du)) / |v|.
// Scatter to the texels uses float4 atomics into an interleaved accumulator.
//
// Vector field.  f = F / Fmax if |F| < Fmax else F / |F|, F = s 0.5 (central
// differences of the blurred volume b, clamp to edge): gathered, no atomics.
// Blur.  b = sum_t m_t I(clamp(x + t)): gathered per axis with the clamp
// folded; dL/dsigma uses the analytic derivative of the normalised mask.
#include <vector>

#include "tdf_common.cuh"

namespace tsf {

constexpr int kMaxRadiiBwd = 4096;

// One voxel's backward pass (the voxel has a gradient: gT != 0 and, GIVEN,
// a positive response).  GIVEN: the forward's response T and arg-max radius R
// are read instead of re-running the sweep (the forward computed them with the
// same arithmetic).
template <int ST, bool NORM, bool GIVEN>
__device__ __forceinline__ void tdf_backward_voxel(const void *__restrict__ F, int X, int Y, int Z, int x, int y,
                                                   int z, float g, float rmin, float rmax, float rstep,
                                                   const CircleTable &tab, const float *__restrict__ Tin,
                                                   const float *__restrict__ Rin, float4 *__restrict__ gV) {
    const int64_t vi = lin(x, y, z, X, Y);
    float H[3][3], V[3][3], d[3];
    hessian<ST, NORM>(F, X, Y, Z, x, y, z, H);
    eig3<float>(H, V, d);
    const float e2[3] = {V[0][1], V[1][1], V[2][1]};
    const float e3[3] = {V[0][2], V[1][2], V[2][2]};
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    // forward sweep: the arg-max radius
    float maxSum = GIVEN ? Tin[vi] : 0.0f, rstar = GIVEN ? Rin[vi] : 0.0f;
    int nr = 0;
    for (float radius = rmin; !GIVEN && radius <= rmax && nr < kMaxRadiiBwd; radius = radius + rstep, nr++) {
        float rs = 0.0f;
        for (int j = 0; j < 32; j++) {
            const float c = tab.c[j], s = tab.s[j];
            const float va0 = c * e3[0] + s * e2[0], va1 = c * e3[1] + s * e2[1], va2 = c * e3[2] + s * e2[2];
            const float3 smp = sample_linear<ST>(F, X, Y, Z, fx + radius * va0, fy + radius * va1, fz + radius * va2);
            rs = rs + (((-smp.x) * va0 + (-smp.y) * va1) + (-smp.z) * va2);
        }
        rs = rs / 32.0f;
        if (rs > maxSum) {
            maxSum = rs;
            rstar = radius;
        } else {
            break;
        }
    }
    if (!(maxSum > 0.0f)) return;
    const float gs = g / 32.0f;
    float gE2[3] = {0.f, 0.f, 0.f}, gE3[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < 32; j++) {
        const float c = tab.c[j], s = tab.s[j];
        const float a[3] = {c * e3[0] + s * e2[0], c * e3[1] + s * e2[1], c * e3[2] + s * e2[2]};
        const float u = fx + rstar * a[0] - 0.5f, v = fy + rstar * a[1] - 0.5f, w = fz + rstar * a[2] - 0.5f;
        const float fu = floorf(u), fv = floorf(v), fw = floorf(w);
        const float A = u - fu, B = v - fv, Cc = w - fw;
        const int i0 = clampi((int)fu, X), j0 = clampi((int)fv, Y), k0 = clampi((int)fw, Z);
        const int i1 = clampi((int)fu + 1, X), j1 = clampi((int)fv + 1, Y), k1 = clampi((int)fw + 1, Z);
        const int64_t idx[8] = {lin(i0, j0, k0, X, Y), lin(i1, j0, k0, X, Y), lin(i0, j1, k0, X, Y),
                                lin(i1, j1, k0, X, Y), lin(i0, j0, k1, X, Y), lin(i1, j0, k1, X, Y),
                                lin(i0, j1, k1, X, Y), lin(i1, j1, k1, X, Y)};
        const float IA = 1.f - A, IB = 1.f - B, IC = 1.f - Cc;
        const float wt[8] = {IA * IB * IC, A * IB * IC, IA * B * IC, A * B * IC,
                             IA * IB * Cc, A * IB * Cc, IA * B * Cc, A * B * Cc};
        float4 t[8];
#pragma unroll
        for (int q = 0; q < 8; q++) t[q] = Vec4Load<ST>::load(F, idx[q]);
        float Vs[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 8; q++) {
            Vs[0] += wt[q] * t[q].x;
            Vs[1] += wt[q] * t[q].y;
            Vs[2] += wt[q] * t[q].z;
            const float k = -gs * wt[q];
            atomicAdd(&gV[idx[q]], make_float4(k * a[0], k * a[1], k * a[2], 0.0f));
        }
        // derivative of the interpolant along x, y, z (dotted with a)
#define TSF_DOTA(p) ((p).x * a[0] + (p).y * a[1] + (p).z * a[2])
        const float d000 = TSF_DOTA(t[0]), d100 = TSF_DOTA(t[1]), d010 = TSF_DOTA(t[2]), d110 = TSF_DOTA(t[3]);
        const float d001 = TSF_DOTA(t[4]), d101 = TSF_DOTA(t[5]), d011 = TSF_DOTA(t[6]), d111 = TSF_DOTA(t[7]);
#undef TSF_DOTA
        const float jx = IB * IC * (d100 - d000) + B * IC * (d110 - d010) + IB * Cc * (d101 - d001) + B * Cc * (d111 - d011);
        const float jy = IA * IC * (d010 - d000) + A * IC * (d110 - d100) + IA * Cc * (d011 - d001) + A * Cc * (d111 - d101);
        const float jz = IA * IB * (d001 - d000) + A * IB * (d101 - d100) + IA * B * (d011 - d010) + A * B * (d111 - d110);
        const float gA[3] = {gs * (-Vs[0] - rstar * jx), gs * (-Vs[1] - rstar * jy), gs * (-Vs[2] - rstar * jz)};
#pragma unroll
        for (int m = 0; m < 3; m++) {
            gE3[m] += c * gA[m];
            gE2[m] += s * gA[m];
        }
    }
    // eigenvector derivatives -> dL/dH
    float G[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    const float *gE[3] = {nullptr, gE2, gE3};
#pragma unroll
    for (int i = 1; i < 3; i++) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (k == i) continue;
            const float den = d[i] - d[k];
            if (fabsf(den) <= 1e-7f * (fabsf(d[i]) + fabsf(d[k])) + 1e-30f) continue;
            const float coef = (gE[i][0] * V[0][k] + gE[i][1] * V[1][k] + gE[i][2] * V[2][k]) / den;
#pragma unroll
            for (int m = 0; m < 3; m++)
#pragma unroll
                for (int nn = 0; nn < 3; nn++) G[m][nn] += coef * V[m][k] * V[nn][i];
        }
    }
    const float gxx = G[0][0], gyx = G[0][1] + G[1][0], gzx = G[0][2] + G[2][0];
    const float gyy = G[1][1], gzy = G[1][2] + G[2][1], gzz = G[2][2];
    // Hessian entries -> the six face neighbours
    const int64_t nb[6] = {lin(clampi(x + 1, X), y, z, X, Y), lin(clampi(x - 1, X), y, z, X, Y),
                           lin(x, clampi(y + 1, Y), z, X, Y), lin(x, clampi(y - 1, Y), z, X, Y),
                           lin(x, y, clampi(z + 1, Z), X, Y), lin(x, y, clampi(z - 1, Z), X, Y)};
    const float gu[6][3] = {{0.5f * gxx, 0.5f * gyx, 0.5f * gzx}, {-0.5f * gxx, -0.5f * gyx, -0.5f * gzx},
                            {0.f, 0.5f * gyy, 0.5f * gzy},        {0.f, -0.5f * gyy, -0.5f * gzy},
                            {0.f, 0.f, 0.5f * gzz},               {0.f, 0.f, -0.5f * gzz}};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        float o[3] = {gu[q][0], gu[q][1], gu[q][2]};
        if (NORM) {
            const float4 f4 = Vec4Load<ST>::load(F, nb[q]);
            const float iw = 1.0f / f4.w;
            const float ux = f4.x * iw, uy = f4.y * iw, uz = f4.z * iw;
            const float ug = ux * o[0] + uy * o[1] + uz * o[2];
            o[0] = (o[0] - ux * ug) * iw;
            o[1] = (o[1] - uy * ug) * iw;
            o[2] = (o[2] - uz * ug) * iw;
        }
        atomicAdd(&gV[nb[q]], make_float4(o[0], o[1], o[2], 0.0f));
    }
}

// A CTA of 128 threads covers a 16 x 8 x 4 region (four 8 x 4 x 4 blocks).
// Phase 1 lists the region's voxels that have a gradient to pass back, in
// region order (x fastest); phase 2 hands them to the threads in turn, so
// every warp works on voxels with a gradient (about half of a volume's voxels
// have a zero response and nothing to pass back) and consecutive threads on
// neighbouring voxels, whose gathers and scatters stay close.
constexpr int kBwdRX = 16, kBwdRY = 8, kBwdRZ = 4, kBwdRounds = kBwdRX * kBwdRY * kBwdRZ / 128;

template <int ST, bool NORM, bool GIVEN>
__global__ void __launch_bounds__(128) tdf_backward_kernel(const void *__restrict__ F, int X, int Y, int Z,
                                                           float rmin, float rmax, float rstep, const CircleTable tab,
                                                           const float *__restrict__ gT, const float *__restrict__ Tin,
                                                           const float *__restrict__ Rin, float4 *__restrict__ gV) {
    __shared__ short list[kBwdRounds * 128];
    __shared__ int wcount[kBwdRounds][4];
    const int t = threadIdx.x, lane = t & 31, wp = t >> 5;
    const int bx = blockIdx.x * kBwdRX, by = blockIdx.y * kBwdRY, bz = blockIdx.z * kBwdRZ;
    unsigned ballot[kBwdRounds];
#pragma unroll
    for (int k = 0; k < kBwdRounds; k++) {
        const int v = k * 128 + t;
        const int x = bx + (v % kBwdRX), y = by + (v / kBwdRX) % kBwdRY, z = bz + v / (kBwdRX * kBwdRY);
        bool act = false;
        if (x < X && y < Y && z < Z) {
            const int64_t vi = lin(x, y, z, X, Y);
            act = gT[vi] != 0.0f && (!GIVEN || Tin[vi] > 0.0f);
        }
        ballot[k] = __ballot_sync(0xffffffffu, act);
        if (lane == 0) wcount[k][wp] = __popc(ballot[k]);
    }
    __syncthreads();
    int total = 0, base[kBwdRounds];
#pragma unroll
    for (int k = 0; k < kBwdRounds; k++)
        for (int w2 = 0; w2 < 4; w2++) {
            if (w2 == wp) base[k] = total;
            total += wcount[k][w2];
        }
#pragma unroll
    for (int k = 0; k < kBwdRounds; k++)
        if ((ballot[k] >> lane) & 1u) list[base[k] + __popc(ballot[k] & ((1u << lane) - 1u))] = (short)(k * 128 + t);
    __syncthreads();
    for (int e = t; e < total; e += 128) {
        const int v = list[e];
        const int x = bx + (v % kBwdRX), y = by + (v / kBwdRX) % kBwdRY, z = bz + v / (kBwdRX * kBwdRY);
        tdf_backward_voxel<ST, NORM, GIVEN>(F, X, Y, Z, x, y, z, gT[lin(x, y, z, X, Y)], rmin, rmax, rstep, tab, Tin,
                                            Rin, gV);
    }
}

__global__ void aos4_to_planar_add_kernel(const float4 *__restrict__ a, float *__restrict__ planar, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = a[i];
    planar[i] += v.x;
    planar[n + i] += v.y;
    planar[2 * n + i] += v.z;
}

// createVectorField backward, gathered: the voxels whose central difference
// reads I at q.
__global__ void vector_field_backward_kernel(const float *__restrict__ b, const float *__restrict__ gf, int X, int Y,
                                             int Z, float fmax, float sg, float *__restrict__ gI) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    const int64_t n = (int64_t)X * Y * Z;
    // dL/dF at voxel p (recomputes the normalisation branch)
    auto gF = [&](int px, int py, int pz, float out[3]) {
        const float gx = 0.5f * (b[lin(clampi(px + 1, X), py, pz, X, Y)] - b[lin(clampi(px - 1, X), py, pz, X, Y)]);
        const float gy = 0.5f * (b[lin(px, clampi(py + 1, Y), pz, X, Y)] - b[lin(px, clampi(py - 1, Y), pz, X, Y)]);
        const float gz = 0.5f * (b[lin(px, py, clampi(pz + 1, Z), X, Y)] - b[lin(px, py, clampi(pz - 1, Z), X, Y)]);
        const float Fx = sg * gx, Fy = sg * gy, Fz = sg * gz;
        const float l = sqrtf(Fx * Fx + Fy * Fy + Fz * Fz);
        const int64_t p = lin(px, py, pz, X, Y);
        const float g0 = gf[p], g1 = gf[n + p], g2 = gf[2 * n + p];
        if (l < fmax) {
            out[0] = g0 / fmax; out[1] = g1 / fmax; out[2] = g2 / fmax;
        } else {
            const float ux = Fx / l, uy = Fy / l, uz = Fz / l;
            const float ug = ux * g0 + uy * g1 + uz * g2;
            out[0] = (g0 - ux * ug) / l; out[1] = (g1 - uy * ug) / l; out[2] = (g2 - uz * ug) / l;
        }
        // through F = sg * grad: dL/d(grad) = sg * dL/dF
        out[0] *= sg; out[1] *= sg; out[2] *= sg;
    };
    float acc = 0.0f, t[3];
    const int c[3] = {x, y, z}, E[3] = {X, Y, Z};
    for (int k = 0; k < 3; k++) {
        int q[3] = {x, y, z};
        // voxel p = q - e_k reads I(p + e_k) = I(q)
        if (c[k] >= 1) { q[k] = c[k] - 1; gF(q[0], q[1], q[2], t); acc += 0.5f * t[k]; }
        // the last voxel reads I(clamp(p + e_k)) = I(q)
        if (c[k] == E[k] - 1) { gF(x, y, z, t); acc += 0.5f * t[k]; }
        q[0] = x; q[1] = y; q[2] = z;
        // voxel p = q + e_k reads I(p - e_k) = I(q)
        if (c[k] <= E[k] - 2) { q[k] = c[k] + 1; gF(q[0], q[1], q[2], t); acc -= 0.5f * t[k]; }
        // the first voxel reads I(clamp(p - e_k)) = I(q)
        if (c[k] == 0) { gF(x, y, z, t); acc -= 0.5f * t[k]; }
    }
    gI[lin(x, y, z, X, Y)] += acc;
}

struct BlurGrad {
    float w[1331];
    float dw[1331];   // d mask / d sigma
    int m;
};

// blur backward, gathered: gI(q) += sum over (x, t) with clamp(x + t) == q of m_t gb(x);
// per-block FP64 partial of sum_x gb(x) sum_t dm_t I(clamp(x + t)) for dL/dsigma.
__global__ void __launch_bounds__(256) blur_backward_kernel(const float *__restrict__ I, const float *__restrict__ gb,
                                                            int X, int Y, int Z, const BlurGrad bg,
                                                            float *__restrict__ gI, double *__restrict__ dsig_block) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    const bool in = x < X && y < Y && z < Z;
    const int m = bg.m, S = 2 * m + 1;
    double ds = 0.0;
    if (in) {
        // per axis: the (source, tap) pairs whose clamped read lands on this
        // coordinate (at most (m+1)(m+2)/2 = 21 at an edge, 2m+1 inside)
        int srcs[3][24], taps[3][24], cnt[3] = {0, 0, 0};
        const int c[3] = {x, y, z}, E[3] = {X, Y, Z};
        for (int k = 0; k < 3; k++)
            for (int t = -m; t <= m; t++)
                for (int s = max(0, c[k] - m); s <= min(E[k] - 1, c[k] + m); s++)
                    if (clampi(s + t, E[k]) == c[k] && cnt[k] < 24) {
                        srcs[k][cnt[k]] = s;
                        taps[k][cnt[k]] = t;
                        cnt[k]++;
                    }
        float acc = 0.0f;
        for (int ic = 0; ic < cnt[2]; ic++)
            for (int ib = 0; ib < cnt[1]; ib++)
                for (int ia = 0; ia < cnt[0]; ia++) {
                    const int ti = (taps[0][ia] + m) + (taps[1][ib] + m) * S + (taps[2][ic] + m) * S * S;
                    acc += bg.w[ti] * gb[lin(srcs[0][ia], srcs[1][ib], srcs[2][ic], X, Y)];
                }
        gI[lin(x, y, z, X, Y)] += acc;
        // dL/dsigma contribution of the output voxel (x, y, z)
        float sd = 0.0f;
        for (int cz = -m; cz <= m; cz++)
            for (int cy = -m; cy <= m; cy++)
                for (int cx = -m; cx <= m; cx++)
                    sd += bg.dw[(cx + m) + (cy + m) * S + (cz + m) * S * S] *
                          I[lin(clampi(x + cx, X), clampi(y + cy, Y), clampi(z + cz, Z), X, Y)];
        ds = (double)sd * (double)gb[lin(x, y, z, X, Y)];
    }
    __shared__ double red[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ds += __shfl_down_sync(0xffffffffu, ds, o);
    const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    if ((t & 31) == 0) red[t >> 5] = ds;
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        for (int i = 0; i < 8; i++) s += red[i];
        dsig_block[blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z)] = s;
    }
}

static size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t tdf_backward_workspace_size(int X, int Y, int Z) { return a256(sizeof(float4) * (size_t)X * Y * Z); }

int run_tdf_backward(const void *F, int X, int Y, int Z, int st, float rmin, float rmax, float rstep,
                     const float *gT, const float *Tin, const float *Rin, float *gfield, void *ws, size_t ws_bytes,
                     cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!F || !gT || !gfield) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    const int64_t n = (int64_t)X * Y * Z;
    if (!ws || ws_bytes < tdf_backward_workspace_size(X, Y, Z)) return fail(TSF_ERR_WORKSPACE, "TDF backward workspace too small");
    float4 *acc = (float4 *)ws;
    TSF_TRY_CUDA(cudaMemsetAsync(acc, 0, sizeof(float4) * (size_t)n, s));
    const CircleTable tab = host_circle_table();
    const dim3 b(128), g((X + kBwdRX - 1) / kBwdRX, (Y + kBwdRY - 1) / kBwdRY, (Z + kBwdRZ - 1) / kBwdRZ);
    if (g.y > 65535u || g.z > 65535u) return fail(TSF_ERR_INVALID_ARG, "volume too large for the grid");
    const bool norm = !(rmax < 4.0f);
    if ((Tin == nullptr) != (Rin == nullptr)) return fail(TSF_ERR_INVALID_ARG, "give both T and R, or neither");
    const bool given = Tin != nullptr;
#define TSF_TDFB(NORM_, GIVEN_) \
    tdf_backward_kernel<ST, NORM_, GIVEN_><<<g, b, 0, s>>>(F, X, Y, Z, rmin, rmax, rstep, tab, gT, Tin, Rin, acc)
    TSF_DISPATCH_STORAGE(st, ST, {
        if (norm) {
            if (given) TSF_TDFB(true, true); else TSF_TDFB(true, false);
        } else {
            if (given) TSF_TDFB(false, true); else TSF_TDFB(false, false);
        }
    });
#undef TSF_TDFB
    TSF_CHECK_LAUNCH("tdf_backward_kernel");
    aos4_to_planar_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(acc, gfield, n);
    TSF_CHECK_LAUNCH("aos4_to_planar_add_kernel");
    return TSF_OK;
}

int run_vector_field_backward(const float *b, const float *gf, int X, int Y, int Z, float fmax, int vsign, float *gI,
                              cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!b || !gf || !gI) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    const dim3 bl(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    vector_field_backward_kernel<<<g, bl, 0, s>>>(b, gf, X, Y, Z, fmax, (float)vsign, gI);
    TSF_CHECK_LAUNCH("vector_field_backward_kernel");
    return TSF_OK;
}

int host_blur_mask(float sigma, float *mask, int *half_width);

size_t blur_backward_workspace_size(int X, int Y, int Z) {
    const dim3 g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    return a256(sizeof(double) * (size_t)g.x * g.y * g.z) + 256;
}

int run_blur_backward(const float *I, const float *gb, int X, int Y, int Z, float sigma, float *gI, double *dsigma,
                      void *ws, size_t ws_bytes, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!I || !gb || !gI) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!ws || ws_bytes < blur_backward_workspace_size(X, Y, Z)) return fail(TSF_ERR_WORKSPACE, "blur backward workspace too small");
    BlurGrad bg;
    r = host_blur_mask(sigma, bg.w, &bg.m);
    if (r) return r;
    // analytic d(mask)/d(sigma) of the normalised Gaussian (same half width)
    const int m = bg.m, S = 2 * m + 1;
    double e[1331], de[1331], se = 0.0, sde = 0.0;
    for (int c = -m; c <= m; c++)
        for (int bb = -m; bb <= m; bb++)
            for (int a = -m; a <= m; a++) {
                const int i = (a + m) + (bb + m) * S + (c + m) * S * S;
                const double r2 = (double)(a * a + bb * bb + c * c);
                e[i] = exp(-r2 / (2.0 * sigma * sigma));
                de[i] = e[i] * r2 / ((double)sigma * sigma * sigma);
                se += e[i];
                sde += de[i];
            }
    for (int i = 0; i < S * S * S; i++) bg.dw[i] = (float)((de[i] * se - e[i] * sde) / (se * se));
    const dim3 bl(32, 4, 2), g((X + 31) / 32, (Y + 3) / 4, (Z + 1) / 2);
    double *blocks = (double *)ws;
    blur_backward_kernel<<<g, bl, 0, s>>>(I, gb, X, Y, Z, bg, gI, blocks);
    TSF_CHECK_LAUNCH("blur_backward_kernel");
    if (dsigma) {
        const size_t nb = (size_t)g.x * g.y * g.z;
        std::vector<double> h(nb);
        TSF_TRY_CUDA(cudaMemcpyAsync(h.data(), blocks, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
        TSF_TRY_CUDA(cudaStreamSynchronize(s));
        double acc = 0.0;
        for (double v : h) acc += v;
        *dsigma = acc;
    }
    return TSF_OK;
}

}  // namespace tsf

extern "C" size_t tsf_tdf_backward_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return tsf::tdf_backward_workspace_size(X, Y, Z);
}

extern "C" int tsf_tdf_circle_backward(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                                       float rstep, const float *d_gT, const float *d_T, const float *d_R,
                                       float *d_gfield, void *d_workspace, size_t workspace_bytes, void *stream) {
    return tsf::run_tdf_backward(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_gT, d_T, d_R, d_gfield,
                                 d_workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int tsf_vector_field_backward(const float *d_in, const float *d_gf, int X, int Y, int Z, float fmax,
                                         int vsign, float *d_gin, void *stream) {
    return tsf::run_vector_field_backward(d_in, d_gf, X, Y, Z, fmax, vsign, d_gin,
                                          reinterpret_cast<cudaStream_t>(stream));
}

extern "C" size_t tsf_blur_backward_workspace_size(int X, int Y, int Z) {
    if (X <= 0 || Y <= 0 || Z <= 0) return 0;
    return tsf::blur_backward_workspace_size(X, Y, Z);
}

extern "C" int tsf_blur_backward(const float *d_in, const float *d_gout, int X, int Y, int Z, float sigma,
                                 float *d_gin, double *dsigma, void *d_workspace, size_t workspace_bytes,
                                 void *stream) {
    return tsf::run_blur_backward(d_in, d_gout, X, Y, Z, sigma, d_gin, dsigma, d_workspace, workspace_bytes,
                                  reinterpret_cast<cudaStream_t>(stream));
}
