// gvf_tb2.cu -- two GVF Jacobi iterations per launch (temporal blocking) of
// the reference's GVF3DIteration (kernels.cl:1464-1493): a z-streaming kernel
// that keeps the first iteration's result for three planes in shared memory
// and computes the second iteration from it, so the field crosses HBM once
// per two iterations.
//
// A CTA owns an x-y tile of TX x TY outputs and a chunk [qa, qb] of the
// evaluation planes 1 .. Z-2 (as the one-iteration kernel, gvf_zs.cu).  Per
// step t, separated by a CTA barrier:
//   * stage A (iteration k+1) evaluates plane w = wa + t on the tile plus a
//     one-voxel ring: rows y0-1 .. y0+TY, columns x0-4 .. x0+TX+3 in 4-voxel
//     vectors (TY + 2 row warps cover columns x0 .. x0+TX-1, one more warp the
//     two edge vectors of every row), reading v_k from a ring of TMA-loaded
//     boxes (planes w-1, w, w+1; TX + 16 columns, TY + 4 rows) and f0 from a
//     ring of f0 boxes (plane w; TX + 16 columns, TY + 2 rows).  Each result is
//     rounded to the storage format -- it is v_{k+1}, as the one-iteration
//     kernel would have stored it -- and kept as FP32 in a ring of A planes;
//   * stage B (iteration k+2, TY warps) evaluates plane q = wa + t - 2 on the
//     tile from the A planes q-1, q, q+1 (complete since the last barrier)
//     and f0 plane q, and stores it to global memory.
// Only interior planes are evaluated by A (wa = max(qa-1, 1), wb = min(qb+1,
// Z-2)); the mirror rule gives A at plane 0 / Z-1 = A at plane 2 / Z-3, which
// B reads in their place.  Rows and columns follow the rule as in gvf_zs.cu:
// rows evaluate at mirror(y); the vector holding x = 0 / X-1 copies x = 2 /
// X-3; B's planes 2 / Z-3 are also written to planes 0 / Z-1.  Per voxel the
// arithmetic is exactly gvf_plain_kernel's, each iteration rounded to the
// storage format, so two launches of the one-iteration kernel and one launch
// of this one give the same bits.
//
// Rings (depth 4): v load j = plane wa-1+j in slot j % 4, issued one step
// before it is first needed; f0 load j = plane wa+j likewise; A plane
// wa+t in slot t % 4.  Every barrier wait is bounded (tma.cuh); a timeout sets
// bit 0 of the streaming kernels' device error word and the CTA stops after
// draining its copies.
#include <mutex>

#include "packed.cuh"
#include "tma.cuh"

namespace tsf {

template <int ST> struct Tb2Cfg {
    using T = typename Store<ST>::T;
    static constexpr int ES = (int)sizeof(T);
    static constexpr int TX = 128, TY = 8;
    static constexpr int H = 8;                             // x halo of the boxes, elements
    static constexpr int BW = TX + 2 * H;                   // box width: x0-8 .. x0+TX+7
    static constexpr int VROWS = TY + 4;                    // v box rows: y0-2 .. y0+TY+1
    static constexpr int FROWS = TY + 2;                    // f0 box rows: y0-1 .. y0+TY
    static constexpr int AW = TX + 8;                       // A plane columns: x0-4 .. x0+TX+3
    static constexpr int AROWS = TY + 2;                    // A plane rows: y0-1 .. y0+TY
    static constexpr int R = 4;                             // ring depth
    static constexpr int VBOX = BW * VROWS * 3 * ES;
    static constexpr int FBOX = BW * FROWS * 3 * ES;
    static constexpr int VSLOT = (VBOX + 127) / 128 * 128;
    static constexpr int FSLOT = (FBOX + 127) / 128 * 128;
    static constexpr int ASLOT = (AW * AROWS * 3 * 4 + 127) / 128 * 128;
    static constexpr int AWARPS = TY + 3;                   // TY + 2 row warps + the edge warp
    static constexpr int BWARPS = TY;
    static constexpr int THREADS = 32 * (AWARPS + BWARPS);
    static constexpr int SMEM = R * (VSLOT + FSLOT + ASLOT) + 2 * R * 8 + 16;
};

__device__ int g_gvf_tb2_error;

// One 4-voxel vector of one iteration: centre c[4], x neighbours xl / xr of
// the vector's ends, y and z neighbours, f0 of the component, |f0|^2.
// Exactly gvf_plain_kernel's arithmetic per voxel.
__device__ __forceinline__ void tb2_update(const float c[4], float xl, float xr, const float yp[4],
                                           const float ym[4], const float zp[4], const float zm[4],
                                           const float fc[4], const float sqr[4], float mu, float res[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float lap = -6.0f * c[i];
        lap = lap + (i == 3 ? xr : c[i + (i < 3 ? 1 : 0)]);
        lap = lap + (i == 0 ? xl : c[i - (i > 0 ? 1 : 0)]);
        lap = lap + yp[i];
        lap = lap + ym[i];
        lap = lap + zp[i];
        lap = lap + zm[i];
        const float upd = mu * lap - (c[i] - fc[i]) * sqr[i];
        res[i] = c[i] + upd;
    }
}

template <int ST>
__global__ void __launch_bounds__(Tb2Cfg<ST>::THREADS, 1)
    gvf_tb2_kernel(const __grid_constant__ CUtensorMap tv, const __grid_constant__ CUtensorMap tf,
                   typename Store<ST>::T *__restrict__ dst, int X, int Y, int Z, float mu, int ntx, int K,
                   long long wait_limit) {
    using C = Tb2Cfg<ST>;
    using T = typename Store<ST>::T;
    using P = PackedV<ST, 4 * C::ES>;
    constexpr int TX = C::TX, TY = C::TY, BW = C::BW, AW = C::AW, R = C::R;
    constexpr int VROWS = C::VROWS, FROWS = C::FROWS, AROWS = C::AROWS;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *vring = smem;
    unsigned char *fring = vring + R * C::VSLOT;
    float *aring = reinterpret_cast<float *>(fring + R * C::FSLOT);
    uint64_t *vbar = reinterpret_cast<uint64_t *>(reinterpret_cast<unsigned char *>(aring) + R * C::ASLOT);
    uint64_t *fbar = vbar + R;

    const int col = blockIdx.x / K, chunk = blockIdx.x % K;
    const int x0 = min((col % ntx) * TX, X - TX);
    const int y0 = min((col / ntx) * TY, Y - TY);
    const int ZI = Z - 2;
    const int qa = 1 + (int)((int64_t)ZI * chunk / K), qb = (int)((int64_t)ZI * (chunk + 1) / K);
    const int wa = max(qa - 1, 1), wb = min(qb + 1, Z - 2);
    const int nA = wb - wa + 1, nV = nA + 2, nF = nA;       // v planes wa-1 .. wb+1, f0 planes wa .. wb
    const int nsteps = nA + 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int issued_v = 0, issued_f = 0;                          // in thread 0

    pdl_trigger();
    if (tid == 0) {
        tma_prefetch_desc(&tv);
        tma_prefetch_desc(&tf);
        for (int i = 0; i < R; i++) {
            mbar_init(vbar + i, 1);
            mbar_init(fbar + i, 1);
        }
        fence_mbar_init();
        pdl_wait();
        for (; issued_v < R && issued_v < nV; issued_v++) {
            mbar_arrive_expect_tx(vbar + issued_v, (uint32_t)C::VBOX);
            tma_load_4d(vring + issued_v * C::VSLOT, &tv, vbar + issued_v, x0 - C::H, y0 - 2, wa - 1 + issued_v, 0);
        }
        for (; issued_f < 2 && issued_f < nF; issued_f++) {
            mbar_arrive_expect_tx(fbar + issued_f, (uint32_t)C::FBOX);
            tma_load_4d(fring + issued_f * C::FSLOT, &tf, fbar + issued_f, x0 - C::H, y0 - 1, wa + issued_f, 0);
        }
    }
    __syncthreads();

    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    const int vcs = VROWS * BW, fcs = FROWS * BW, acs = AROWS * AW;   // component strides
    bool ok = true;
    for (int t = 0; t < nsteps; t++) {
        if (t >= 1 && tid == 0) {
            // slots (t-1) % R of the v ring and (t+1) % R of the f0 ring were
            // last read in step t-1
            fence_proxy_async_smem();
            if (issued_v < nV) {
                const int sl = issued_v % R;
                mbar_arrive_expect_tx(vbar + sl, (uint32_t)C::VBOX);
                tma_load_4d(vring + sl * C::VSLOT, &tv, vbar + sl, x0 - C::H, y0 - 2, wa - 1 + issued_v, 0);
                issued_v++;
            }
            if (issued_f < nF) {
                const int sl = issued_f % R;
                mbar_arrive_expect_tx(fbar + sl, (uint32_t)C::FBOX);
                tma_load_4d(fring + sl * C::FSLOT, &tf, fbar + sl, x0 - C::H, y0 - 1, wa + issued_f, 0);
                issued_f++;
            }
        }
        if (warp < C::AWARPS) {
            // ---- stage A: iteration k+1 on plane w, rows y0-1 .. y0+TY ----
            if (t < nA) {
                ok &= mbar_wait(vbar + t % R, (t / R) & 1, wait_limit);
                ok &= mbar_wait(vbar + (t + 1) % R, ((t + 1) / R) & 1, wait_limit);
                ok &= mbar_wait(vbar + (t + 2) % R, ((t + 2) / R) & 1, wait_limit);
                ok &= mbar_wait(fbar + t % R, (t / R) & 1, wait_limit);
                // this lane's vector: row warps -> (row y0-1+warp, columns x0+4 lane);
                // the edge warp -> lane l < 2 (TY+2): row y0-1+l/2, columns x0-4 (l even)
                // or x0+TX (l odd)
                int r, c0;
                bool act;
                if (warp < TY + 2) {
                    r = y0 - 1 + warp;
                    c0 = x0 + 4 * lane;
                    act = true;
                } else {
                    r = y0 - 1 + (lane >> 1);
                    c0 = (lane & 1) ? x0 + TX : x0 - 4;
                    act = lane < 2 * (TY + 2);
                }
                act = act && r >= 0 && r < Y && c0 >= 0 && c0 < X;
                if (act) {
                    const int er = mirror(r, Y);
                    const T *vm = reinterpret_cast<const T *>(vring + (t % R) * C::VSLOT);
                    const T *vc = reinterpret_cast<const T *>(vring + ((t + 1) % R) * C::VSLOT);
                    const T *vp = reinterpret_cast<const T *>(vring + ((t + 2) % R) * C::VSLOT);
                    const T *fs = reinterpret_cast<const T *>(fring + (t % R) * C::FSLOT);
                    const int vo = (er - (y0 - 2)) * BW + (c0 - (x0 - C::H));   // centre of component 0
                    const int fo = (er - (y0 - 1)) * BW + (c0 - (x0 - C::H));
                    float f[3][4], sqr[4];
#pragma unroll
                    for (int k = 0; k < 3; k++) P::unpack(P::load_plain(fs + fo + k * fcs), f[k]);
#pragma unroll
                    for (int i = 0; i < 4; i++) sqr[i] = (f[0][i] * f[0][i] + f[1][i] * f[1][i]) + f[2][i] * f[2][i];
                    float *ao = aring + (t % R) * (C::ASLOT / 4) + (r - (y0 - 1)) * AW + (c0 - (x0 - 4));
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const T *pc = vc + vo + k * vcs;
                        float cc[4], yp[4], ym[4], zp[4], zm[4], res[4];
                        P::unpack(P::load_plain(pc), cc);
                        P::unpack(P::load_plain(pc + BW), yp);
                        P::unpack(P::load_plain(pc - BW), ym);
                        P::unpack(P::load_plain(vp + vo + k * vcs), zp);
                        P::unpack(P::load_plain(vm + vo + k * vcs), zm);
                        const float xr = Store<ST>::load(pc[4]), xl = Store<ST>::load(pc[-1]);
                        tb2_update(cc, xl, xr, yp, ym, zp, zm, f[k], sqr, mu, res);
                        if (c0 == 0) res[0] = res[2];
                        if (c0 + 4 == X) res[3] = res[1];
                        float4 q4;
                        q4.x = quantize<ST>(res[0]);
                        q4.y = quantize<ST>(res[1]);
                        q4.z = quantize<ST>(res[2]);
                        q4.w = quantize<ST>(res[3]);
                        *reinterpret_cast<float4 *>(ao + k * acs) = q4;
                    }
                }
            }
        } else if (t >= 2) {
            // ---- stage B: iteration k+2 on plane q from the A planes ----
            const int q = wa + t - 2;
            if (q >= qa && q <= qb) {
                const int y = y0 + (warp - C::AWARPS), xc = x0 + 4 * lane;
                const int ey = mirror(y, Y);
                const int qm = q - 1 == 0 ? 2 : q - 1, qp = q + 1 == Z - 1 ? Z - 3 : q + 1;
                const int jc = q - wa, jm = qm - wa, jp = qp - wa;              // A indices (ring slot = j % R)
                ok &= mbar_wait(fbar + jc % R, (jc / R) & 1, wait_limit);
                const T *fs = reinterpret_cast<const T *>(fring + (jc % R) * C::FSLOT) +
                              (ey - (y0 - 1)) * BW + (xc - (x0 - C::H));
                float f[3][4], sqr[4];
#pragma unroll
                for (int k = 0; k < 3; k++) P::unpack(P::load_plain(fs + k * fcs), f[k]);
#pragma unroll
                for (int i = 0; i < 4; i++) sqr[i] = (f[0][i] * f[0][i] + f[1][i] * f[1][i]) + f[2][i] * f[2][i];
                const int ao = (ey - (y0 - 1)) * AW + (xc - (x0 - 4));
                const float *ac = aring + (jc % R) * (C::ASLOT / 4) + ao;
                const float *am = aring + (jm % R) * (C::ASLOT / 4) + ao;
                const float *ap = aring + (jp % R) * (C::ASLOT / 4) + ao;
                T *o = dst + (int64_t)q * plane + (int64_t)y * X + xc;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float *pc = ac + k * acs;
                    const float4 c4 = *reinterpret_cast<const float4 *>(pc);
                    const float4 yp4 = *reinterpret_cast<const float4 *>(pc + AW);
                    const float4 ym4 = *reinterpret_cast<const float4 *>(pc - AW);
                    const float4 zp4 = *reinterpret_cast<const float4 *>(ap + k * acs);
                    const float4 zm4 = *reinterpret_cast<const float4 *>(am + k * acs);
                    const float cc[4] = {c4.x, c4.y, c4.z, c4.w}, yp[4] = {yp4.x, yp4.y, yp4.z, yp4.w};
                    const float ym[4] = {ym4.x, ym4.y, ym4.z, ym4.w}, zp[4] = {zp4.x, zp4.y, zp4.z, zp4.w};
                    const float zm[4] = {zm4.x, zm4.y, zm4.z, zm4.w};
                    float res[4];
                    tb2_update(cc, pc[-1], pc[4], yp, ym, zp, zm, f[k], sqr, mu, res);
                    if (xc == 0) res[0] = res[2];
                    if (xc + 4 == X) res[3] = res[1];
                    T *oc = o + k * n;
                    P::store(oc, res);
                    if (q == 2) P::store(oc - 2 * plane, res);
                    if (q == Z - 3) P::store(oc + 2 * plane, res);
                }
            }
        }
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
    }
    if (!ok) {
        if (tid == 0) {
            atomicOr(&g_gvf_tb2_error, 1);
            // wait (bounded) for this CTA's copies in flight
            for (int s = 0; s < R; s++) {
                int j = issued_v - 1 - ((issued_v - 1 - s) % R + R) % R;
                if (j >= 0) mbar_wait(vbar + s, (j / R) & 1, wait_limit);
                j = issued_f - 1 - ((issued_f - 1 - s) % R + R) % R;
                if (j >= 0) mbar_wait(fbar + s, (j / R) & 1, wait_limit);
            }
        }
    }
}

bool encode_planar(CUtensorMap *m, const void *base, int X, int Y, int Z, int es, int bx, int by);
bool gvf_zs_eligible(int st, const void *d_f0, const void *a, const void *b, int X, int Y, int Z);

// Whether the two-iteration kernel can run this volume: the streaming
// kernel's conditions plus a tile that fits (X >= 128, Y >= 8, Z >= 5).
bool gvf_tb2_eligible(int st, const void *d_f0, const void *a, const void *b, int X, int Y, int Z) {
    return X >= 128 && Y >= 8 && Z >= 5 && gvf_zs_eligible(st, d_f0, a, b, X, Y, Z);
}

template <int ST> static int tb2_geometry(int X, int Y, int Z, int &grid, int &ntx, int &K) {
    using C = Tb2Cfg<ST>;
    static int blocks_per_sm[kMaxDevices];
    static int nsm[kMaxDevices];
    static std::mutex mu;
    int dev = 0;
    TSF_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(TSF_ERR_INVALID_ARG, "device ordinal out of range");
    {
        std::lock_guard<std::mutex> lock(mu);
        if (blocks_per_sm[dev] <= 0) {
            TSF_TRY_CUDA(cudaFuncSetAttribute(gvf_tb2_kernel<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
            int bps = 0;
            TSF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, gvf_tb2_kernel<ST>, C::THREADS, C::SMEM));
            TSF_TRY_CUDA(cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev));
            blocks_per_sm[dev] = bps > 0 ? bps : 1;
        }
    }
    ntx = (X + C::TX - 1) / C::TX;
    const int nty = (Y + C::TY - 1) / C::TY;
    const int64_t cols = (int64_t)ntx * nty;
    const int64_t slots = (int64_t)blocks_per_sm[dev] * nsm[dev];
    int64_t k = slots / cols;
    if (k < 1 || cols * k * 5 < slots * 4) k = (6 * slots + cols - 1) / cols;
    const int64_t kmax = (Z - 2) / 8 > 1 ? (Z - 2) / 8 : 1;
    if (k > kmax) k = kmax;
    if (k < 1) k = 1;
    if (cols * k > 0x7fffffff) return fail(TSF_ERR_INVALID_ARG, "volume too large for the two-iteration GVF kernel");
    K = (int)k;
    grid = (int)(cols * k);
    return TSF_OK;
}

// Two iterations src -> dst (caller checked gvf_tb2_eligible).
int launch_gvf_tb2(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu,
                   cudaStream_t s) {
    int r = TSF_OK;
    TSF_DISPATCH_STORAGE(st, ST, {
        using C = Tb2Cfg<ST>;
        using T = typename Store<ST>::T;
        int grid = 0, ntx = 0, K = 0;
        r = tb2_geometry<ST>(X, Y, Z, grid, ntx, K);
        if (r) return r;
        CUtensorMap tv, tf;
        if (!encode_planar(&tv, src, X, Y, Z, C::ES, C::BW, C::VROWS) ||
            !encode_planar(&tf, d_f0, X, Y, Z, C::ES, C::BW, C::FROWS))
            return fail(TSF_ERR_CUDA, "tensor map encoding failed");
        cudaLaunchAttribute attr[1];
        const cudaLaunchConfig_t cfg = pdl_config(dim3((unsigned)grid), dim3(C::THREADS), C::SMEM, s, attr);
        TSF_TRY_CUDA(cudaLaunchKernelEx(&cfg, gvf_tb2_kernel<ST>, tv, tf, (T *)dst, X, Y, Z, mu, ntx, K, kWaitCycles));
    });
    TSF_CHECK_LAUNCH("gvf_tb2_kernel");
    return r;
}

int gvf_tb2_error(int clear) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_gvf_tb2_error, sizeof(int));
    if (e != cudaSuccess) {
        check_cuda(e, "read GVF two-iteration device error word");
        return -1;
    }
    if (clear && v) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_gvf_tb2_error, &z, sizeof(int));
        if (e != cudaSuccess) {
            check_cuda(e, "clear GVF two-iteration device error word");
            return -1;
        }
    }
    return v;
}

}  // namespace tsf
