// gvf_adjoint_zs.cu -- one reverse GVF step as a z-streaming kernel fed by
// TMA copies (the transpose of GVF3DIteration, kernels.cl:1464-1493; no
// counterpart in the reference, which has no derivatives).
//
// Given the folded cotangent g = fold(lambda') (zero outside the volume; the
// y and z parts of the fold are applied to lambda' beforehand, the x part by
// this kernel as it loads), the
// state v_k and the data term f0, per component c and voxel r:
//     lambda_c = g_c (1 - 6 mu - s) + mu nb_c,   nb_c = sum of g_c over the 6 neighbours
//     dL/df0_c += g_c s - 2 f_c sum_d g_d (v_d - f_d),   s = |f0|^2
//     dL/dmu  += sum_c v_c (nb_c - 6 g_c)
// The last line is sum_q g(q) L(v)(q) summed by parts (the neighbour sum of
// g is already at hand), so the state is read at the voxel only.
//
// Layout as in the forward streaming kernel: a CTA walks z-planes of 128 x 8
// tiles; thread 0 keeps TMA copies of the next planes in flight -- g with a
// 16-byte x-halo and a 1-row y-halo (ring of RG slots; planes -1 and Z read
// as zero, which is the "zero outside" rule), and v, f0, dL/df0 tiles (ring of
// RT slots, one barrier per plane) -- while the 8 warps compute the current
// plane.  Tiles at the +x / +y edges are ragged (lanes outside write nothing):
// dL/df0 is read-modify-write, so tiles must not overlap.  Work is one
// contiguous range of (tile, plane) units per CTA over a grid of one CTA per
// resident slot, so every CTA gets the same number of planes; a range may span
// two tiles.  dL/dmu: each lane sums a plane's 12 products in FP32 (fixed
// order) and adds that to an FP64 total; the CTA's total is added to its own
// slot of the partials, so the result does not depend on scheduling.
#include <mutex>

#include "packed.cuh"
#include "tma.cuh"

namespace tsf {

template <int ST> struct AdjZsCfg {
    using T = typename Store<ST>::T;
    static constexpr int ES = (int)sizeof(T);
    static constexpr int TX = 128, TY = 8;
    static constexpr int H = 4;                            // g halo: 16 bytes of FP32
    static constexpr int BW = TX + 2 * H;
    static constexpr int RG = 4, RT = 3;
    static constexpr int GBOX = BW * (TY + 2) * 3 * 4;
    static constexpr int VBOX = TX * TY * 3 * ES;          // v and f0 tiles
    static constexpr int GFBOX = TX * TY * 3 * 4;          // dL/df0 tile
    static constexpr int r128(int b) { return (b + 127) / 128 * 128; }
    static constexpr int GSLOT = r128(GBOX);
    static constexpr int VOFF = 0, FOFF = r128(VBOX), GFOFF = 2 * r128(VBOX);
    static constexpr int TSLOT = 2 * r128(VBOX) + r128(GFBOX);
    static constexpr int SMEM = RG * GSLOT + RT * TSLOT + (RG + RT) * 8 + 16;
    static constexpr int THREADS = 32 * TY;
    static constexpr int BYTES = 4 * ES;
};

__device__ int g_gvf_adj_zs_error;

struct AdjSeg {
    int col, qa, n;                                       // tile, first plane, planes
};

__device__ __forceinline__ AdjSeg adj_seg(int64_t w, int64_t w1, int Z) {
    AdjSeg s;
    s.col = (int)(w / Z);
    s.qa = (int)(w - (int64_t)s.col * Z);
    const int64_t end = min(w1, (int64_t)(s.col + 1) * Z);
    s.n = (int)(end - w);
    return s;
}

template <int ST>
__global__ void __launch_bounds__(AdjZsCfg<ST>::THREADS, 1)
    gvf_adjoint_zs_kernel(const __grid_constant__ CUtensorMap tg, const __grid_constant__ CUtensorMap tv,
                          const __grid_constant__ CUtensorMap tf, const __grid_constant__ CUtensorMap tgf,
                          float *__restrict__ lam_out, float *__restrict__ gf, double *__restrict__ dmu_block, int X,
                          int Y, int Z, float mu, int ntx, int64_t W) {
    using C = AdjZsCfg<ST>;
    using T = typename Store<ST>::T;
    using P = PackedV<ST, C::BYTES>;
    using PF = PackedV<TSF_STORE_F32, 16>;
    constexpr int TX = C::TX, TY = C::TY, H = C::H, BW = C::BW, RG = C::RG, RT = C::RT;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *gring = smem;
    unsigned char *tring = smem + RG * C::GSLOT;
    uint64_t *gbar = reinterpret_cast<uint64_t *>(tring + RT * C::TSLOT);
    uint64_t *tbar = gbar + RG;

    const int64_t w0 = W * blockIdx.x / gridDim.x, w1 = W * (blockIdx.x + 1) / gridDim.x;
    const int tid = threadIdx.x;

    // producer (thread 0): cursors over this CTA's g loads and tile loads
    int64_t pg_w = w0, pt_w = w0;
    int pg_k = 0, pt_k = 0, gseq = 0, tseq = 0;
    auto more_g = [&]() { return pg_w < w1; };
    auto more_t = [&]() { return pt_w < w1; };
    auto issue_g = [&]() {
        const AdjSeg s = adj_seg(pg_w, w1, Z);
        const int x0 = (s.col % ntx) * TX, y0 = (s.col / ntx) * TY;
        const int sl = gseq % RG;
        mbar_arrive_expect_tx(gbar + sl, (uint32_t)C::GBOX);
        tma_load_4d(gring + sl * C::GSLOT, &tg, gbar + sl, x0 - H, y0 - 1, s.qa - 1 + pg_k, 0);
        gseq++;
        if (++pg_k == s.n + 2) {
            pg_w += s.n;
            pg_k = 0;
        }
    };
    auto issue_t = [&]() {
        const AdjSeg s = adj_seg(pt_w, w1, Z);
        const int x0 = (s.col % ntx) * TX, y0 = (s.col / ntx) * TY, q = s.qa + pt_k;
        const int sl = tseq % RT;
        unsigned char *slot = tring + sl * C::TSLOT;
        mbar_arrive_expect_tx(tbar + sl, (uint32_t)(2 * C::VBOX + C::GFBOX));
        tma_load_4d(slot + C::VOFF, &tv, tbar + sl, x0, y0, q, 0);
        tma_load_4d(slot + C::FOFF, &tf, tbar + sl, x0, y0, q, 0);
        tma_load_4d(slot + C::GFOFF, &tgf, tbar + sl, x0, y0, q, 0);
        tseq++;
        if (++pt_k == s.n) {
            pt_w += s.n;
            pt_k = 0;
        }
    };
    pdl_trigger();
    if (tid == 0) {
        tma_prefetch_desc(&tg);
        tma_prefetch_desc(&tv);
        tma_prefetch_desc(&tf);
        tma_prefetch_desc(&tgf);
        for (int i = 0; i < RG; i++) mbar_init(gbar + i, 1);
        for (int i = 0; i < RT; i++) mbar_init(tbar + i, 1);
        fence_mbar_init();
        // the previous kernel (the fold of g) has completed; every other global
        // access of this CTA follows the barrier below
        pdl_wait();
        while (gseq < RG && more_g()) issue_g();
        while (tseq < RT && more_t()) issue_t();
    }
    __syncthreads();

    const int lane = tid & 31, r = tid >> 5;
    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    const float k1 = 1.0f - 6.0f * mu;
    double dmu = 0.0;
    bool ok = true;
    int gbase = 0, tbase = 0;                             // sequence numbers of the segment's first loads
    for (int64_t w = w0; w < w1;) {
        const AdjSeg s = adj_seg(w, w1, Z);
        const int x0 = (s.col % ntx) * TX, y0 = (s.col / ntx) * TY;
        const int xc = x0 + 4 * lane, y = y0 + r;
        const bool act = xc < X && y < Y;
        const int goff = (r + 1) * BW + H + 4 * lane;      // component c at goff + c * (TY + 2) * BW
        // the x part of the fold happens here, on every g vector a lane loads:
        // its vector holds x = 0 and 2 (or X-3 and X-1) together
        const bool fx_lo = xc == 0, fx_hi = xc + 4 == X;
        auto xfold = [&](float a[4]) {
            if (fx_lo) { a[2] = a[2] + a[0]; a[0] = 0.0f; }
            if (fx_hi) { a[1] = a[1] + a[3]; a[3] = 0.0f; }
        };
        const int toff = r * TX + 4 * lane;                // component c at toff + c * TY * TX
        float gm[3][4], gc[3][4];                          // g at planes q-1 and q (lane's column)
        ok &= mbar_wait(gbar + gbase % RG, (gbase / RG) & 1);
        ok &= mbar_wait(gbar + (gbase + 1) % RG, ((gbase + 1) / RG) & 1);
        {
            const float *a = reinterpret_cast<const float *>(gring + (gbase % RG) * C::GSLOT);
            const float *b = reinterpret_cast<const float *>(gring + ((gbase + 1) % RG) * C::GSLOT);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                PF::unpack(PF::load_plain(a + goff + c * (TY + 2) * BW), gm[c]);
                PF::unpack(PF::load_plain(b + goff + c * (TY + 2) * BW), gc[c]);
                xfold(gm[c]);
                xfold(gc[c]);
            }
        }
        float *lo = lam_out + (int64_t)y * X + xc + (int64_t)s.qa * plane;
        float *go = gf + (int64_t)y * X + xc + (int64_t)s.qa * plane;
        for (int k = 0; k < s.n; k++) {
            const int jg = gbase + k + 2, jt = tbase + k;
            ok &= mbar_wait(gbar + jg % RG, (jg / RG) & 1);
            ok &= mbar_wait(tbar + jt % RT, (jt / RT) & 1);
            const float *g0 = reinterpret_cast<const float *>(gring + ((gbase + k + 1) % RG) * C::GSLOT) + goff;
            const float *gp = reinterpret_cast<const float *>(gring + (jg % RG) * C::GSLOT) + goff;
            const unsigned char *ts = tring + (jt % RT) * C::TSLOT;
            const T *vs = reinterpret_cast<const T *>(ts + C::VOFF) + toff;
            const T *fs = reinterpret_cast<const T *>(ts + C::FOFF) + toff;
            const float *gfs = reinterpret_cast<const float *>(ts + C::GFOFF) + toff;

            float fv[3][4], vv[3][4], sq[4], gd[4], part = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                P::unpack(P::load_plain(fs + c * TY * TX), fv[c]);
                P::unpack(P::load_plain(vs + c * TY * TX), vv[c]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                sq[i] = (fv[0][i] * fv[0][i] + fv[1][i] * fv[1][i]) + fv[2][i] * fv[2][i];
                gd[i] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float *pc = g0 + c * (TY + 2) * BW;
                float zp[4], yp[4], ym[4];
                PF::unpack(PF::load_plain(gp + c * (TY + 2) * BW), zp);
                PF::unpack(PF::load_plain(pc + BW), yp);
                PF::unpack(PF::load_plain(pc - BW), ym);
                xfold(zp);
                xfold(yp);
                xfold(ym);
                // x-neighbours outside the lane's vector are never fold targets
                // (x = -1 / X read as 0; x = 3 / X-4 are unchanged by the fold)
                const float xr = pc[4], xl = pc[-1];
                const float *g = gc[c];
                float out[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float xp = i == 3 ? xr : g[i < 3 ? i + 1 : i];
                    const float xm = i == 0 ? xl : g[i > 0 ? i - 1 : 0];
                    const float nb = ((((xp + xm) + yp[i]) + ym[i]) + zp[i]) + gm[c][i];
                    out[i] = g[i] * (k1 - sq[i]) + mu * nb;
                    part = part + vv[c][i] * (nb - 6.0f * g[i]);
                    gd[i] = gd[i] + g[i] * (vv[c][i] - fv[c][i]);
                }
                if (act) *reinterpret_cast<float4 *>(lo + c * n) = make_float4(out[0], out[1], out[2], out[3]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    gm[c][i] = g[i];
                    gc[c][i] = zp[i];
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float a[4];
                PF::unpack(PF::load_plain(gfs + c * TY * TX), a);
                // gm now holds this plane's g
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = a[i] + (gm[c][i] * sq[i] - 2.0f * fv[c][i] * gd[i]);
                if (act) *reinterpret_cast<float4 *>(go + c * n) = make_float4(a[0], a[1], a[2], a[3]);
            }
            if (act) dmu += (double)part;
            lo += plane;
            go += plane;
            // the plane's slots are free once every thread is here
            if (__syncthreads_or(!ok)) {
                ok = false;
                break;
            }
            if (tid == 0) {
                fence_proxy_async_smem();
                const int rel_g = (k == s.n - 1) ? gbase + s.n + 2 : gbase + k + 1;
                const int rel_t = tbase + k + 1;
                while (gseq < rel_g + RG && more_g()) issue_g();
                while (tseq < rel_t + RT && more_t()) issue_t();
            }
        }
        if (!ok) break;
        gbase += s.n + 2;
        tbase += s.n;
        w += s.n;
    }
    if (!ok) {
        if (tid == 0) {
            atomicOr(&g_gvf_adj_zs_error, 1);
            for (int sl = 0; sl < RG; sl++) {
                const int j = gseq - 1 - ((gseq - 1 - sl) % RG + RG) % RG;
                if (j >= 0) mbar_wait(gbar + sl, (j / RG) & 1);
            }
            for (int sl = 0; sl < RT; sl++) {
                const int j = tseq - 1 - ((tseq - 1 - sl) % RT + RT) % RT;
                if (j >= 0) mbar_wait(tbar + sl, (j / RT) & 1);
            }
        }
        return;
    }
    // the CTA's dL/dmu, in a fixed order
    __shared__ double red[C::THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmu += __shfl_down_sync(0xffffffffu, dmu, o);
    if (lane == 0) red[r] = dmu;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int i = 0; i < C::THREADS / 32; i++) t += red[i];
        dmu_block[blockIdx.x] += t;
    }
}

// Whether the streaming adjoint applies: rows a multiple of 16 bytes in the
// storage format and in FP32, 16-byte aligned buffers, a tensor-map encoder.
bool gvf_adjoint_zs_eligible(int st, const void *g, const void *v, const void *f, const void *gf, const void *lam,
                             int X) {
    const int es = (int)storage_bytes(st);
    if (es == 0 || (X * es) % 16 != 0 || (X * 4) % 16 != 0) return false;
    if (((uintptr_t)g | (uintptr_t)v | (uintptr_t)f | (uintptr_t)gf | (uintptr_t)lam) & 15) return false;
    return tensor_map_encoder() != nullptr;
}

// Upper bound of the grid (entries of the mu partials the caller provides).
int gvf_adjoint_zs_max_grid() {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess) {
        cudaGetLastError();
        return 4096;
    }
    return 4 * nsm;
}

template <int ST>
static int adj_zs_slots(int &slots) {
    using C = AdjZsCfg<ST>;
    // per device: the shared-memory attribute applies to the current device
    static int cached[kMaxDevices];
    static std::mutex mu;
    int dev = 0;
    TSF_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(TSF_ERR_INVALID_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (cached[dev] <= 0) {
        TSF_TRY_CUDA(cudaFuncSetAttribute(gvf_adjoint_zs_kernel<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          C::SMEM));
        int bps = 0, nsm = 0;
        TSF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, gvf_adjoint_zs_kernel<ST>, C::THREADS,
                                                                   C::SMEM));
        TSF_TRY_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        cached[dev] = (bps > 0 ? (bps > 4 ? 4 : bps) : 1) * nsm;
    }
    slots = cached[dev];
    return TSF_OK;
}

// One reverse step with the streaming kernel (caller checked eligibility and
// provides gvf_adjoint_zs_max_grid() partials at dmu_block).
int launch_gvf_adjoint_zs(int st, const float *g, const void *v, const void *f, float *lam_out, float *gf,
                          double *dmu_block, int X, int Y, int Z, float mu, cudaStream_t s) {
    int r = TSF_OK;
    TSF_DISPATCH_STORAGE(st, ST, {
        using C = AdjZsCfg<ST>;
        int slots = 0;
        r = adj_zs_slots<ST>(slots);
        if (r) return r;
        const int ntx = (X + C::TX - 1) / C::TX, nty = (Y + C::TY - 1) / C::TY;
        const int64_t W = (int64_t)ntx * nty * Z;
        const int grid = (int)(W < slots ? W : slots);
        CUtensorMap mg, mv, mf, mgf;
        if (!encode_planar(&mg, g, X, Y, Z, 4, C::BW, C::TY + 2) || !encode_planar(&mv, v, X, Y, Z, C::ES, C::TX, C::TY) ||
            !encode_planar(&mf, f, X, Y, Z, C::ES, C::TX, C::TY) || !encode_planar(&mgf, gf, X, Y, Z, 4, C::TX, C::TY))
            return fail(TSF_ERR_CUDA, "tensor map encoding failed");
        cudaLaunchAttribute attr[1];
        const cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)grid), dim3(C::THREADS), C::SMEM, s, attr);
        TSF_TRY_CUDA(cudaLaunchKernelEx(&cfg, gvf_adjoint_zs_kernel<ST>, mg, mv, mf, mgf, lam_out, gf, dmu_block, X,
                                        Y, Z, mu, ntx, W));
    });
    TSF_CHECK_LAUNCH("gvf_adjoint_zs_kernel");
    return r;
}

int gvf_adjoint_zs_error(int clear) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_gvf_adj_zs_error, sizeof(int));
    if (e != cudaSuccess) {
        check_cuda(e, "read GVF adjoint device error word");
        return -1;
    }
    if (clear && v) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_gvf_adj_zs_error, &z, sizeof(int));
        if (e != cudaSuccess) {
            check_cuda(e, "clear GVF adjoint device error word");
            return -1;
        }
    }
    return v;
}

}  // namespace tsf
