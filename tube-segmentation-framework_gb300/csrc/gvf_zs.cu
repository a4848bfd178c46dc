// gvf_zs.cu -- one GVF Jacobi iteration (reference GVF3DIteration,
// kernels.cl:1464-1493) as a z-streaming kernel fed by tensor-memory-access
// (TMA) copies into a shared-memory ring of planes.
//
// Why: the register-vector kernel (gvf_vec_kernel) issues all of a thread's
// loads, waits, computes and exits; the resident blocks of an SM move through
// those phases together, so HBM idles while they compute and the issue slots
// idle while they wait.  Here a CTA owns an x-y tile and a run of z planes;
// one thread keeps the copies of the next planes in flight while the compute
// warps work on the current one, so memory traffic and arithmetic overlap.
// Synchronisation (template flag WS): FP32 / snorm16 -- thread 0 of the
// compute warps issues the copies and the CTA meets at a barrier after every
// plane, which frees that plane's slots; FP16 / BF16 -- a ninth warp issues
// the copies and each compute warp releases a slot on the slot's "empty"
// mbarrier (arrival count 8) when done with it, so warps drift up to three
// planes apart instead of waiting for the slowest every plane.  Both stream
// downwards (rev) on every other iteration, so each iteration starts on the
// planes the previous one wrote last, which are still in L2; downwards the
// newest ring slot holds plane q-1 and the oldest plane q+1, and the sums
// keep the reference's order (z+1 before z-1).
//
// Work: tile TX x TY = 128 x 8 outputs, one warp per tile row, 4 consecutive
// voxels per lane.  The tiles of
// a row / column that would run past the volume are shifted back inside it
// (they overlap their neighbour and write identical values).  Each tile's z
// range of evaluation planes [1, Z-2] is split into K chunks, K chosen so that
// tiles x chunks fills the resident-CTA slots once (or, where one wave would
// leave many slots idle, about six times); CTAs of neighbouring tiles
// stream the same planes at the same time and share their halo rows in L2.
//
// Per evaluation plane q the CTA needs planes q-1, q, q+1 of v (box: TX + 2H
// columns, H = 16 bytes of halo each side, TY + 2 rows, 3 components) and
// plane q of f0 (TX x TY x 3).  v planes live in a ring of RV slots, f0 planes
// in a ring of RF slots; slot i of a ring is reused every RV (RF) planes and
// its mbarrier phase parity is (load index / ring size) & 1.
//
// Mirror rule (v'[w] = U(m(w)), m: 0 -> 2, size-1 -> size-3 per axis): a
// lane's rows are evaluated at mirror(y) (inside the loaded box because edge
// tiles are shifted inward); in x the vector holding x = 0 / X-1 copies the
// result of x = 2 / X-3; the plane q = 2 (Z-3) is also written to plane 0
// (Z-1).  Per voxel the arithmetic is exactly gvf_plain_kernel's, so the
// result is bit-identical to the other GVF kernels.  For FP16 and BF16 the
// y neighbours, the outer x neighbours and f0 enter the arithmetic through
// mixed-precision add / subtract / fma (16-bit source, FP32 result, one
// rounding), which saves the separate half -> float conversions: the
// conversion is exact, so each such instruction rounds like convert-then-op,
// and (f0 - v)|f0|^2 added equals (v - f0)|f0|^2 subtracted bit for bit.
// snorm16 has no such shortcut: each stored value costs three instructions to
// read exactly (snorm16_pair2), so that iteration is bound by instruction
// issue, not bytes; there the voxel pairs (0, 1) and (2, 3) go through paired
// FP32 instructions (.f32x2: two operations, each rounded like its scalar
// twin), with every sum that follows a paired product done one at a time --
// the assembler contracts a paired product feeding a paired sum into a paired
// fma despite .rn, which would change the rounding.  (For the 16-bit float
// formats, which are bound by bytes, paired sums gained nothing.)
#include <mutex>

#include "packed.cuh"
#include "tma.cuh"

namespace tsf {

template <int ST> struct ZsCfg {
    using T = typename Store<ST>::T;
    static constexpr int ES = (int)sizeof(T);
    static constexpr int TX = 128;
    static constexpr int TY = 8;
    static constexpr int H = 16 / ES;                      // x halo, elements
    static constexpr int BW = TX + 2 * H;                  // v box width
    // ring slots: 16-bit formats 68 KB per CTA (3 per SM), FP32 102 KB (2 per SM)
    static constexpr int RV = ES == 2 ? 5 : 4, RF = ES == 2 ? 4 : 3;
    static constexpr int VBOX = BW * (TY + 2) * 3 * ES;    // bytes of one v box
    static constexpr int FBOX = TX * TY * 3 * ES;
    static constexpr int VSLOT = (VBOX + 127) / 128 * 128;
    static constexpr int FSLOT = (FBOX + 127) / 128 * 128;
    static constexpr int SMEM = RV * VSLOT + RF * FSLOT + 2 * (RV + RF) * 8 + 16;
    static constexpr int THREADS = 32 * TY;
    static constexpr int MIN_CTAS = ES == 2 ? 3 : 2;       // resident CTAs per SM the shared memory allows
    static constexpr int BYTES = 4 * ES;                   // one lane's 4 voxels
};

// Device-side error word: bit 0 = a copy did not land within kWaitCycles.
__device__ int g_gvf_zs_error;

// one box copy: announce its bytes on the slot's barrier, then start it
__device__ __forceinline__ void zs_issue(unsigned char *slot, uint64_t *bar, int bytes, const CUtensorMap *map,
                                         int x, int y, int z) {
    mbar_arrive_expect_tx(bar, (uint32_t)bytes);
    tma_load_4d(slot, map, bar, x, y, z, 0);
}

template <int ST, bool WS, bool REV>
__global__ void __launch_bounds__(ZsCfg<ST>::THREADS + 32 * WS, ZsCfg<ST>::MIN_CTAS) gvf_zs_kernel(const __grid_constant__ CUtensorMap tv,
                                                                   const __grid_constant__ CUtensorMap tf,
                                                                   typename Store<ST>::T *__restrict__ dst, int X,
                                                                   int Y, int Z, float mu, int ntx, int K,
                                                                   long long wait_limit, int no_copies) {
    constexpr bool rev = REV;   // stream downwards (compile-time: no selects in the sums)
    using C = ZsCfg<ST>;
    using T = typename Store<ST>::T;
    using P = PackedV<ST, C::BYTES>;
    // FP16 / BF16: 16-bit operands enter the sums through mixed-precision
    // instructions instead of separate conversions (same bits)
    constexpr bool MIX = ST == TSF_STORE_F16 || ST == TSF_STORE_BF16;
    constexpr int TX = C::TX, TY = C::TY, H = C::H, BW = C::BW, RV = C::RV, RF = C::RF;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *vring = smem;
    unsigned char *fring = smem + RV * C::VSLOT;
    uint64_t *vbar = reinterpret_cast<uint64_t *>(fring + RF * C::FSLOT);
    uint64_t *fbar = vbar + RV;
    uint64_t *vemp = fbar + RF;                           // WS: slot released by the 8 compute warps
    uint64_t *femp = vemp + RV;

    // this CTA's tile and plane range
    const int col = blockIdx.x / K, chunk = blockIdx.x % K;
    const int tx = col % ntx, ty = col / ntx;
    const int x0 = X >= TX ? min(tx * TX, X - TX) : 0;
    const int y0 = Y >= TY ? min(ty * TY, Y - TY) : 0;
    const int ZI = Z - 2;
    const int qa = 1 + (int)((int64_t)ZI * chunk / K), qb = (int)((int64_t)ZI * (chunk + 1) / K);
    const int nf = qb - qa + 1, nv = nf + 2;               // f planes qa..qb, v planes qa-1..qb+1
    const int tid = threadIdx.x;

    // v load j = plane qa-1+j into slot j % RV; f load j = plane qa+j into slot j % RF
    int issued_v = 0, issued_f = 0;                       // meaningful in the issuing thread only
    // The next iteration's CTAs may be scheduled as this grid's CTAs exit
    // (programmatic dependent launch): they run this prologue, then wait below.
    pdl_trigger();
    if (WS && tid == 0) {
        for (int i = 0; i < RV; i++) mbar_init(vbar + i, 1);
        for (int i = 0; i < RF; i++) mbar_init(fbar + i, 1);
        for (int i = 0; i < RV; i++) mbar_init(vemp + i, TY);
        for (int i = 0; i < RF; i++) mbar_init(femp + i, TY);
        fence_mbar_init();
    }
    if (!WS && tid == 0) {
        tma_prefetch_desc(&tv);
        tma_prefetch_desc(&tf);
        for (int i = 0; i < RV; i++) mbar_init(vbar + i, 1);
        for (int i = 0; i < RF; i++) mbar_init(fbar + i, 1);
        fence_mbar_init();
        // the previous grid (which wrote src and reads dst) has completed and its
        // writes are visible; every other global access of this CTA follows the
        // barrier below
        pdl_wait();
        for (; !no_copies && issued_v < RV && issued_v < nv; issued_v++)
            zs_issue(vring + issued_v * C::VSLOT, vbar + issued_v, C::VBOX, &tv, x0 - H, y0 - 1,
                     rev ? qb + 1 - issued_v : qa - 1 + issued_v);
        for (; !no_copies && issued_f < RF && issued_f < nf; issued_f++)
            zs_issue(fring + issued_f * C::FSLOT, fbar + issued_f, C::FBOX, &tf, x0, y0,
                     rev ? qb - issued_f : qa + issued_f);
    }
    __syncthreads();

    const int lane = tid & 31, r = tid >> 5;
    if constexpr (WS) {
        if (r == TY) {
            // the copy warp: one lane issues v load j (plane qa-1+j) into slot
            // j % RV and f load j (plane qa+j) into slot j % RF, each once the
            // compute warps have released the slot's previous load; order v0,
            // v1, then (v_{i+2}, f_i), the order of need
            if (lane == 0) {
                tma_prefetch_desc(&tv);
                tma_prefetch_desc(&tf);
                // the previous grid (which wrote src and reads dst) has
                // completed and its writes are visible; the compute warps
                // touch global memory only after copies issued below land
                pdl_wait();
                bool pok = true;
                for (int i = -2; pok && !no_copies && i < nf; i++) {
                    const int j = i + 2, sv = j % RV;
                    if (j >= RV) pok = mbar_wait(vemp + sv, ((j / RV) - 1) & 1, wait_limit);
                    if (!pok) break;
                    fence_proxy_async_smem();
                    zs_issue(vring + sv * C::VSLOT, vbar + sv, C::VBOX, &tv, x0 - H, y0 - 1,
                             rev ? qb + 1 - j : qa - 1 + j);
                    issued_v = j + 1;
                    if (i < 0) continue;
                    const int sf_ = i % RF;
                    if (i >= RF) pok = mbar_wait(femp + sf_, ((i / RF) - 1) & 1, wait_limit);
                    if (!pok) break;
                    fence_proxy_async_smem();
                    zs_issue(fring + sf_ * C::FSLOT, fbar + sf_, C::FBOX, &tf, x0, y0, rev ? qb - i : qa + i);
                    issued_f = i + 1;
                }
                if (!pok) {
                    // record the failure and wait (bounded) for the copies in flight
                    atomicOr(&g_gvf_zs_error, 1);
                    for (int sl = 0; sl < RV; sl++) {
                        int j = issued_v - 1 - ((issued_v - 1 - sl) % RV + RV) % RV;
                        if (j >= 0) mbar_wait(vbar + sl, (j / RV) & 1, wait_limit);
                    }
                    for (int sl = 0; sl < RF; sl++) {
                        int j = issued_f - 1 - ((issued_f - 1 - sl) % RF + RF) % RF;
                        if (j >= 0) mbar_wait(fbar + sl, (j / RF) & 1, wait_limit);
                    }
                }
            }
            return;
        }
    }
    const int xc = x0 + 4 * lane, y = y0 + r;
    const bool out_ok = xc < X && y < Y;
    const bool fix_lo = xc == 0, fix_hi = xc + 4 == X;   // vectors holding x = 0 / X-1
    const int ey = mirror(y, Y);
    const int lr = ey - y0 + 1, fr = ey - y0;            // row in the v box / f box
    const int e = H + 4 * lane;                           // column of xc in the v box
    const int64_t n = (int64_t)X * Y * Z, plane = (int64_t)X * Y;
    T *o = dst + (int64_t)y * X + xc + (int64_t)(rev ? qb : qa) * plane;   // component 0, plane q
    const int voff = lr * BW + e, vstride = (TY + 2) * BW;    // component c at voff + c * vstride
    const int foff = fr * TX + 4 * lane;
    bool ok = true;
    // FP32 / snorm16: the lane's z column (centre values of the previous and
    // the current plane) is carried from plane to plane so each stored value
    // is loaded and converted once as a centre.  FP16 / BF16 read both
    // neighbour planes from the ring each plane: they enter the sums
    // unconverted.
    // FP32 / snorm16: the lane's z column in three register sets that take
    // the roles of planes q-1, q and q+1 in turn (the plane loop is unrolled
    // three times, so no values move)
    float A[3][4], B[3][4], Cz[3][4];
    int sm = 0, sc = 1, sp = 2, sf = 0;                   // slots: previous, current, next v plane; f plane
    uint32_t pp = 0, pf = 0;                              // phase parity of the waits on sp, sf
    ok &= mbar_wait(vbar + 0, 0, wait_limit);
    ok &= mbar_wait(vbar + 1, 0, wait_limit);
    if constexpr (!MIX) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            P::unpack(P::load_plain(reinterpret_cast<const T *>(vring) + voff + c * vstride), A[c]);
            P::unpack(P::load_plain(reinterpret_cast<const T *>(vring + C::VSLOT) + voff + c * vstride), B[c]);
        }
    }

    // One plane; cm, cc = the z column at planes q-1 and q, zn receives plane
    // q+1 (q+1 and q-1 downwards).  False: stop (a wait ran out).
    auto step = [&](int k, float (&cm)[3][4], float (&cc)[3][4], float (&zn)[3][4]) -> bool {
        const int q = rev ? qb - k : qa + k;
        ok &= mbar_wait(vbar + sp, pp, wait_limit);
        ok &= mbar_wait(fbar + sf, pf, wait_limit);
        if constexpr (WS) {
            if (__any_sync(0xffffffffu, !ok)) {
                ok = false;
                return false;
            }
        }
        const T *vm = reinterpret_cast<const T *>(vring + sm * C::VSLOT) + voff;
        const T *vc = reinterpret_cast<const T *>(vring + sc * C::VSLOT) + voff;
        const T *vp = reinterpret_cast<const T *>(vring + sp * C::VSLOT) + voff;
        const T *fs = reinterpret_cast<const T *>(fring + sf * C::FSLOT) + foff;
        const bool dup_lo = q == 2, dup_hi = q == Z - 3;

        float fv[3][4], sqr[4];
        typename P::Raw fraw[3];
#pragma unroll
        for (int c = 0; c < 3; c++) fraw[c] = P::load_plain(fs + c * TY * TX);
        if constexpr (MIX && ST == TSF_STORE_F16) {
            sqr[0] = sqadd16v<0>(fraw[2].u, sqadd16v<0>(fraw[1].u, sqadd16v<0>(fraw[0].u, -0.0f)));
            sqr[1] = sqadd16v<1>(fraw[2].u, sqadd16v<1>(fraw[1].u, sqadd16v<1>(fraw[0].u, -0.0f)));
            sqr[2] = sqadd16v<2>(fraw[2].u, sqadd16v<2>(fraw[1].u, sqadd16v<2>(fraw[0].u, -0.0f)));
            sqr[3] = sqadd16v<3>(fraw[2].u, sqadd16v<3>(fraw[1].u, sqadd16v<3>(fraw[0].u, -0.0f)));
        } else if constexpr (ST == TSF_STORE_SNORM16) {
            // voxel pairs (0, 1) and (2, 3): two FP32 operations per instruction
            float2 f2[3][2];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                f2[c][0] = snorm16_pair2(fraw[c].u[0]);
                f2[c][1] = snorm16_pair2(fraw[c].u[1]);
                fv[c][0] = f2[c][0].x; fv[c][1] = f2[c][0].y; fv[c][2] = f2[c][1].x; fv[c][3] = f2[c][1].y;
            }
            // products paired, the sums after them one at a time: the
            // assembler contracts a paired product that feeds a paired sum
            // into a paired fma, although .rn asks it not to
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float2 a = mul2(f2[0][h], f2[0][h]), b = mul2(f2[1][h], f2[1][h]), d = mul2(f2[2][h], f2[2][h]);
                sqr[2 * h] = (a.x + b.x) + d.x;
                sqr[2 * h + 1] = (a.y + b.y) + d.y;
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++) P::unpack(fraw[c], fv[c]);
#pragma unroll
            for (int i = 0; i < 4; i++) sqr[i] = (fv[0][i] * fv[0][i] + fv[1][i] * fv[1][i]) + fv[2][i] * fv[2][i];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const T *pc = vc + c * vstride;
            float res[4];
            float *zp = zn[c];
            if constexpr (MIX) {
                // The centre plane q is converted once; its y neighbours, the
                // outer x neighbours, planes q -+ 1 and f0 enter the sums
                // unconverted (mixed-precision add / subtract, same bits).
                // planes q+1 and q-1: the newest and the oldest slot upwards,
                // the other way round downwards (rev)
                const T *pzp = (rev ? vm : vp) + c * vstride, *pzm = (rev ? vp : vm) + c * vstride;
                const typename P::Raw cr = P::load_plain(pc), zr = P::load_plain(pzp),
                                      mr = P::load_plain(pzm), yp = P::load_plain(pc + BW),
                                      ym = P::load_plain(pc - BW);
                const unsigned xr = *reinterpret_cast<const unsigned short *>(pc + 4);
                const unsigned xl = *reinterpret_cast<const unsigned short *>(pc - 1);
                float cen[4], lap[4];
                P::unpack(cr, cen);
#pragma unroll
                for (int i = 0; i < 4; i++) lap[i] = -6.0f * cen[i];
                lap[0] = lap[0] + cen[1];
                lap[1] = lap[1] + cen[2];
                lap[2] = lap[2] + cen[3];
                lap[3] = add16<ST, 0>(xr, lap[3]);
                lap[0] = add16<ST, 0>(xl, lap[0]);
                lap[1] = lap[1] + cen[0];
                lap[2] = lap[2] + cen[1];
                lap[3] = lap[3] + cen[2];
                lap[0] = add16v<ST, 0>(yp.u, lap[0]);
                lap[1] = add16v<ST, 1>(yp.u, lap[1]);
                lap[2] = add16v<ST, 2>(yp.u, lap[2]);
                lap[3] = add16v<ST, 3>(yp.u, lap[3]);
                lap[0] = add16v<ST, 0>(ym.u, lap[0]);
                lap[1] = add16v<ST, 1>(ym.u, lap[1]);
                lap[2] = add16v<ST, 2>(ym.u, lap[2]);
                lap[3] = add16v<ST, 3>(ym.u, lap[3]);
                lap[0] = add16v<ST, 0>(zr.u, lap[0]);
                lap[1] = add16v<ST, 1>(zr.u, lap[1]);
                lap[2] = add16v<ST, 2>(zr.u, lap[2]);
                lap[3] = add16v<ST, 3>(zr.u, lap[3]);
                lap[0] = add16v<ST, 0>(mr.u, lap[0]);
                lap[1] = add16v<ST, 1>(mr.u, lap[1]);
                lap[2] = add16v<ST, 2>(mr.u, lap[2]);
                lap[3] = add16v<ST, 3>(mr.u, lap[3]);
                // (f0 - v) * |f0|^2 added is (v - f0) * |f0|^2 subtracted, bit for bit
                float d[4];
                d[0] = sub16v<ST, 0>(fraw[c].u, cen[0]);
                d[1] = sub16v<ST, 1>(fraw[c].u, cen[1]);
                d[2] = sub16v<ST, 2>(fraw[c].u, cen[2]);
                d[3] = sub16v<ST, 3>(fraw[c].u, cen[3]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float upd = mu * lap[i] + d[i] * sqr[i];
                    res[i] = cen[i] + upd;
                }
            } else if constexpr (ST == TSF_STORE_SNORM16) {
                // voxel pairs (0, 1) and (2, 3) through paired FP32 operations;
                // the x neighbours, which straddle the pairs, one at a time.
                // Per voxel the operations and their order are the scalar path's.
                const typename P::Raw zr = P::load_plain(vp + c * vstride), yr = P::load_plain(pc + BW),
                                      mr = P::load_plain(pc - BW);
                const float2 z01 = snorm16_pair2(zr.u[0]), z23 = snorm16_pair2(zr.u[1]);
                const float2 y01 = snorm16_pair2(yr.u[0]), y23 = snorm16_pair2(yr.u[1]);
                const float2 m01 = snorm16_pair2(mr.u[0]), m23 = snorm16_pair2(mr.u[1]);
                const float xr = Store<ST>::load(pc[4]);
                const float xl = Store<ST>::load(pc[-1]);
                const float2 v01 = make_float2(cc[c][0], cc[c][1]), v23 = make_float2(cc[c][2], cc[c][3]);
                const float2 c01 = make_float2(cm[c][0], cm[c][1]), c23 = make_float2(cm[c][2], cm[c][3]);
                float2 l01 = mul2(v01, make_float2(-6.0f, -6.0f)), l23 = mul2(v23, make_float2(-6.0f, -6.0f));
                l01.x = l01.x + cc[c][1];
                l01.y = l01.y + cc[c][2];
                l23.x = l23.x + cc[c][3];
                l23.y = l23.y + xr;
                l01.x = l01.x + xl;
                l01.y = l01.y + cc[c][0];
                l23.x = l23.x + cc[c][1];
                l23.y = l23.y + cc[c][2];
                l01 = add2(l01, y01);
                l23 = add2(l23, y23);
                l01 = add2(l01, m01);
                l23 = add2(l23, m23);
                l01 = add2(l01, rev ? c01 : z01);   // plane q+1
                l23 = add2(l23, rev ? c23 : z23);
                l01 = add2(l01, rev ? z01 : c01);   // plane q-1
                l23 = add2(l23, rev ? z23 : c23);
                const float2 mu2 = make_float2(mu, mu);
                const float2 a01 = mul2(mu2, l01), a23 = mul2(mu2, l23);
                const float2 b01 = mul2(sub2(v01, make_float2(fv[c][0], fv[c][1])), make_float2(sqr[0], sqr[1]));
                const float2 b23 = mul2(sub2(v23, make_float2(fv[c][2], fv[c][3])), make_float2(sqr[2], sqr[3]));
                const float2 u01 = make_float2(a01.x - b01.x, a01.y - b01.y);   // one at a time (see sqr)
                const float2 u23 = make_float2(a23.x - b23.x, a23.y - b23.y);
                const float2 r01 = add2(v01, u01), r23 = add2(v23, u23);
                res[0] = r01.x; res[1] = r01.y; res[2] = r23.x; res[3] = r23.y;
                zp[0] = z01.x; zp[1] = z01.y; zp[2] = z23.x; zp[3] = z23.y;
            } else {
                float yp[4], ym[4];
                P::unpack(P::load_plain(vp + c * vstride), zp);
                P::unpack(P::load_plain(pc + BW), yp);
                P::unpack(P::load_plain(pc - BW), ym);
                const float xr = Store<ST>::load(pc[4]);
                const float xl = Store<ST>::load(pc[-1]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float v = cc[c][i];
                    float lap = -6.0f * v;
                    lap = lap + (i == 3 ? xr : cc[c][i < 3 ? i + 1 : i]);
                    lap = lap + (i == 0 ? xl : cc[c][i > 0 ? i - 1 : 0]);
                    lap = lap + yp[i];
                    lap = lap + ym[i];
                    lap = lap + (rev ? cm[c][i] : zp[i]);   // plane q+1
                    lap = lap + (rev ? zp[i] : cm[c][i]);   // plane q-1
                    const float upd = mu * lap - (v - fv[c][i]) * sqr[i];
                    res[i] = v + upd;
                }
            }
            if (fix_lo) res[0] = res[2];
            if (fix_hi) res[3] = res[1];
            if (out_ok) {
                T *oc = o + c * n;
                P::store(oc, res);
                if (__builtin_expect(dup_lo | dup_hi, 0)) {     // uniform: two planes of the volume
                    if (dup_lo) P::store(oc - 2 * plane, res);
                    if (dup_hi) P::store(oc + 2 * plane, res);
                }
            }
        }
        o += rev ? -plane : plane;
        if constexpr (WS) {
            // this warp is done with v load k (plane q-1) and f load k
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(vemp + sm);
                mbar_arrive(femp + sf);
            }
        }
        sm = sc;
        sc = sp;
        sp = sp + 1 == RV ? 0 : sp + 1;
        pp ^= sp == 0;
        sf = sf + 1 == RF ? 0 : sf + 1;
        pf ^= sf == 0;
        if constexpr (WS) return true;
        // slots k % RV (v) and k % RF (f) are free once every thread is here
        if (__syncthreads_or(!ok)) {
            ok = false;
            return false;
        }
        if (tid == 0) {
            fence_proxy_async_smem();
            if (issued_v < nv) {                          // issued_v == k + RV: the slot just freed
                const int sl = issued_v % RV;
                zs_issue(vring + sl * C::VSLOT, vbar + sl, C::VBOX, &tv, x0 - H, y0 - 1,
                         rev ? qb + 1 - issued_v : qa - 1 + issued_v);
                issued_v++;
            }
            if (issued_f < nf) {
                const int sl = issued_f % RF;
                zs_issue(fring + sl * C::FSLOT, fbar + sl, C::FBOX, &tf, x0, y0,
                         rev ? qb - issued_f : qa + issued_f);
                issued_f++;
            }
        }
        return true;
    };
    if constexpr (MIX) {
        for (int k = 0; k < nf; k++)
            if (!step(k, A, B, Cz)) break;
    } else {
        for (int k = 0; k < nf; k += 3) {
            if (!step(k, A, B, Cz)) break;
            if (k + 1 >= nf || !step(k + 1, B, Cz, A)) break;
            if (k + 2 >= nf || !step(k + 2, Cz, A, B)) break;
        }
    }
    if (!ok && lane == 0) atomicOr(&g_gvf_zs_error, 1);
    if (!WS && !ok && tid == 0) {
        // wait (bounded) for this CTA's copies in flight
        for (int s = 0; s < RV; s++) {
            int j = issued_v - 1 - ((issued_v - 1 - s) % RV + RV) % RV;
            if (j >= 0) mbar_wait(vbar + s, (j / RV) & 1, wait_limit);
        }
        for (int s = 0; s < RF; s++) {
            int j = issued_f - 1 - ((issued_f - 1 - s) % RF + RF) % RF;
            if (j >= 0) mbar_wait(fbar + s, (j / RF) & 1, wait_limit);
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// 4-D map (x, y, z, component) over a planar field, box (bx, by, 1, 3).
bool encode_planar(CUtensorMap *m, const void *base, int X, int Y, int Z, int es, int bx, int by) {
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, 3};
    const cuuint64_t strides[3] = {(cuuint64_t)X * es, (cuuint64_t)X * Y * es, (cuuint64_t)X * Y * Z * es};
    const cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)by, 1, 3};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(m, es == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                           const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Whether the streaming kernel can run this volume: rows a multiple of 16
// bytes (TMA strides), 16-byte aligned buffers, a driver tensor-map encoder.
bool gvf_zs_eligible(int st, const void *d_f0, const void *a, const void *b, int X, int Y, int Z) {
    const int es = (int)storage_bytes(st);
    if (es == 0 || (X * es) % 16 != 0) return false;
    if (((uintptr_t)d_f0 | (uintptr_t)a | (uintptr_t)b) & 15) return false;
    if ((int64_t)X * Y * Z * es * 3 >= ((int64_t)1 << 40)) return false;
    return tensor_map_encoder() != nullptr;
}

template <int ST> struct ZsLaunch {
    int grid = 0, ntx = 0, K = 0;
};

template <int ST, bool WS>
static int zs_geometry(int X, int Y, int Z, ZsLaunch<ST> &g) {
    using C = ZsCfg<ST>;
    // The shared-memory attribute applies to the device that is current when
    // it is set, so it and the occupancy figures are kept per device.
    static int blocks_per_sm[kMaxDevices];
    static int nsm[kMaxDevices];
    static std::mutex mu;
    int dev = 0;
    TSF_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(TSF_ERR_INVALID_ARG, "device ordinal out of range");
    {
        std::lock_guard<std::mutex> lock(mu);
        if (blocks_per_sm[dev] <= 0) {
            TSF_TRY_CUDA(cudaFuncSetAttribute(gvf_zs_kernel<ST, WS, false>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
            TSF_TRY_CUDA(cudaFuncSetAttribute(gvf_zs_kernel<ST, WS, true>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
            int bps = 0;
            TSF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, gvf_zs_kernel<ST, WS, false>, C::THREADS + 32 * WS,
                                                                       C::SMEM));
            TSF_TRY_CUDA(cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev));
            blocks_per_sm[dev] = bps > 0 ? bps : 1;
        }
    }
    g.ntx = (X + C::TX - 1) / C::TX;
    const int nty = (Y + C::TY - 1) / C::TY;
    const int64_t cols = (int64_t)g.ntx * nty;
    const int64_t slots = (int64_t)blocks_per_sm[dev] * nsm[dev];
    // One wave (tiles x chunks = the resident-CTA slots) when it fills at
    // least 80 % of the slots; otherwise (e.g. 256 tiles on 456 slots at
    // 512^3) about six waves of shorter chunks, so the scheduler backfills
    // freed slots and the tail stays small (512^3 f16: 520 -> 367 us per
    // iteration; one wave at 256^3: 7 chunks, 47.0 us, while 14 chunks take
    // 48.7 us).
    int64_t K = slots / cols;
    if (K < 1 || cols * K * 5 < slots * 4) K = (6 * slots + cols - 1) / cols;
    const int64_t kmax = (Z - 2) / 8 > 1 ? (Z - 2) / 8 : 1;   // chunks of at least 8 planes
    if (K > kmax) K = kmax;
    if (K < 1) K = 1;
    if (cols * K > 0x7fffffff) return fail(TSF_ERR_INVALID_ARG, "volume too large for the streaming GVF kernel");
    g.K = (int)K;
    g.grid = (int)(cols * K);
    return TSF_OK;
}

// One iteration src -> dst with the streaming kernel (caller checked
// gvf_zs_eligible).
template <int ST, bool WS>
static int launch_zs_typed(const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu,
                           cudaStream_t s, int rev, long long wait_limit = kWaitCycles, int no_copies = 0) {
    using C = ZsCfg<ST>;
    using T = typename Store<ST>::T;
    ZsLaunch<ST> g;
    int r = zs_geometry<ST, WS>(X, Y, Z, g);
    if (r) return r;
    CUtensorMap tv, tf;
    if (!encode_planar(&tv, src, X, Y, Z, C::ES, C::BW, C::TY + 2) ||
        !encode_planar(&tf, d_f0, X, Y, Z, C::ES, C::TX, C::TY))
        return fail(TSF_ERR_CUDA, "tensor map encoding failed");
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg =
        pdl_config(dim3((unsigned)g.grid), dim3(C::THREADS + 32 * WS), C::SMEM, s, attr);
    if (rev)
        TSF_TRY_CUDA(cudaLaunchKernelEx(&cfg, gvf_zs_kernel<ST, WS, true>, tv, tf, (T *)dst, X, Y, Z, mu, g.ntx, g.K,
                                        wait_limit, no_copies));
    else
        TSF_TRY_CUDA(cudaLaunchKernelEx(&cfg, gvf_zs_kernel<ST, WS, false>, tv, tf, (T *)dst, X, Y, Z, mu, g.ntx, g.K,
                                        wait_limit, no_copies));
    return TSF_OK;
}

int launch_gvf_zs(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z, float mu,
                  cudaStream_t s, int rev) {
    int r = TSF_OK;
    // 16-bit float formats: a copy warp and per-slot release barriers (the
    // compute warps drift up to three planes apart instead of meeting at a
    // CTA barrier every plane).  FP32 and snorm16 measured faster with the
    // CTA barrier (FP32 is at the copy bandwidth).
    TSF_DISPATCH_STORAGE(st, ST, {
        r = launch_zs_typed<ST, ST == TSF_STORE_F16 || ST == TSF_STORE_BF16>(d_f0, src, dst, X, Y, Z, mu, s, rev);
    });
    TSF_CHECK_LAUNCH("gvf_zs_kernel");
    return r;
}

// Self-test of the bounded waits: one launch with every copy suppressed, so
// each wait runs out after wait_cycles; returns the error word afterwards
// (cleared), or a negative value if the launch itself failed.
int gvf_zs_error(int clear);
int gvf_zs_wait_selftest(int st, const void *d_f0, const void *src, void *dst, int X, int Y, int Z,
                         long long wait_cycles, cudaStream_t s) {
    if (wait_cycles <= 0) return -fail(TSF_ERR_INVALID_ARG, "wait_cycles must be > 0");
    if (!gvf_zs_eligible(st, d_f0, src, dst, X, Y, Z))
        return -fail(TSF_ERR_INVALID_ARG, "the streaming GVF kernel cannot run these buffers");
    if (gvf_zs_error(1) < 0) return -TSF_ERR_CUDA;
    int r = TSF_OK;
    TSF_DISPATCH_STORAGE(st, ST, {
        r = launch_zs_typed<ST, ST == TSF_STORE_F16 || ST == TSF_STORE_BF16>(d_f0, src, dst, X, Y, Z, 0.05f, s, 0,
                                                                              wait_cycles, 1);
    });
    if (r) return -r;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return -check_cuda(e, "GVF wait self-test");
    count_launches(1);
    return gvf_zs_error(1);
}

// Reads (and optionally clears) the streaming kernel's device error word;
// -1 if the read itself failed.
int gvf_zs_error(int clear) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_gvf_zs_error, sizeof(int));
    if (e != cudaSuccess) {
        check_cuda(e, "read GVF device error word");
        return -1;
    }
    if (clear && v) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_gvf_zs_error, &z, sizeof(int));
        if (e != cudaSuccess) {
            check_cuda(e, "clear GVF device error word");
            return -1;
        }
    }
    return v;
}

}  // namespace tsf

namespace tsf {
int gvf_adjoint_zs_error(int clear);
}

extern "C" int tsf_gvf_wait_selftest(const void *d_f0, void *d_v, int X, int Y, int Z, int storage,
                                     long long wait_cycles, void *d_workspace, size_t workspace_bytes, void *stream) {
    using namespace tsf;
    int r = check_dims(X, Y, Z);
    if (r) return -r;
    if (!valid_storage(storage)) return -fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!d_f0 || !d_v) return -fail(TSF_ERR_INVALID_ARG, "null buffer");
    const size_t need = (size_t)X * Y * Z * 3 * storage_bytes(storage);
    if (!d_workspace || workspace_bytes < need) return -fail(TSF_ERR_WORKSPACE, "workspace too small");
    return gvf_zs_wait_selftest(storage, d_f0, d_v, d_workspace, X, Y, Z, wait_cycles,
                                reinterpret_cast<cudaStream_t>(stream));
}

namespace tsf {
int gvf_tb2_error(int clear);
}

extern "C" int tsf_gvf_device_error(int clear) {
    const int a = tsf::gvf_zs_error(clear), b = tsf::gvf_adjoint_zs_error(clear), c = tsf::gvf_tb2_error(clear);
    if (a < 0 || b < 0 || c < 0) return -1;
    return (a || c ? 1 : 0) | (b ? 2 : 0);
}
