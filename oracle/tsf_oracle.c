/*
 * tsf_oracle.c -- CPU restatement of the Tube Segmentation Framework hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker; see tsf_oracle.h).  Parity
 * against the reference's own outputs is UNPINNED: the reference is OpenCL and
 * cannot run here, and it has no golden vectors.
 *
 * This file holds the precision-independent pieces (storage conversions, the
 * sample-direction table, the blur mask, the histogram pyramid) and includes
 * tsf_oracle_impl.h twice to instantiate the float and double kernels.
 *
 * Build: cc -O2 -std=c11 -fopenmp -ffp-contract=off -fPIC -shared (see Makefile).
 * -ffp-contract=off is required: the float oracle must round every product and
 * sum separately, exactly like the CUDA kernels (built with -fmad=false).
 */
#include "tsf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* closed-form eigensolver cores (tsf_oracle_eigc.h), float and double */
#define EIGC_R float
#define EIGC_SFX _f
#define EIGC_SQRT sqrtf
#include "tsf_oracle_eigc.h"
#undef EIGC_R
#undef EIGC_SFX
#undef EIGC_SQRT
#define EIGC_R double
#define EIGC_SFX _d
#define EIGC_SQRT sqrt
#include "tsf_oracle_eigc.h"
#undef EIGC_R
#undef EIGC_SFX
#undef EIGC_SQRT

/* Closed-form eigen-decomposition as the TDF's eigen mode 1 uses it: the
 * float core with 5 Newton steps, redone in double with 7 when
 * 1 - |r| < 1e-3 (two eigenvalues nearly equal); then ascending |lambda| by
 * the reference's selection sort (strict <, kernels.cl:1742-1761) and each
 * eigenvector's largest-magnitude component made positive.  A row-major,
 * Vout[3 * i + k] = component i of eigenvector k. */
void orc_eig3_closed_f32(const float A[9], float Vout[9], float d[3]) {
    const float a[6] = {A[0], A[4], A[8], A[3], A[6], A[7]};
    float lam[3], vec[3][3], r = 0.0f;
    if (eigc_core_f(a, lam, vec, &r, 5) && 1.0f - (r < 0.0f ? -r : r) < 1e-3f) {
        const double ad[6] = {a[0], a[1], a[2], a[3], a[4], a[5]};
        double ld[3], vd[3][3], rd;
        eigc_core_d(ad, ld, vd, &rd, 7);
        for (int k = 0; k < 3; k++) {
            lam[k] = (float)ld[k];
            for (int i = 0; i < 3; i++) vec[k][i] = (float)vd[k][i];
        }
    }
    int idx[3] = {0, 1, 2};
    float dv[3] = {lam[0], lam[1], lam[2]};
    for (int i = 0; i < 2; i++) {
        int k = i;
        float p = dv[i];
        for (int j = i + 1; j < 3; j++)
            if (fabsf(dv[j]) < fabsf(p)) { k = j; p = dv[j]; }
        if (k != i) {
            dv[k] = dv[i];
            dv[i] = p;
            const int t = idx[k]; idx[k] = idx[i]; idx[i] = t;
        }
    }
    for (int k = 0; k < 3; k++) {
        const float *e = vec[idx[k]];
        float big = e[0];
        if (fabsf(e[1]) > fabsf(big)) big = e[1];
        if (fabsf(e[2]) > fabsf(big)) big = e[2];
        const float s = big < 0.0f ? -1.0f : 1.0f;
        for (int i = 0; i < 3; i++) Vout[3 * i + k] = s * e[i];
        d[k] = dv[k];
    }
}

static int g_threads = 0;

void orc_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Storage conversions                                                       */
/* ------------------------------------------------------------------------ */

static inline uint32_t f2u(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
static inline float u2f(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

/* IEEE binary16, round to nearest even. */
uint16_t orc_f32_to_f16_bits(float x) {
    uint32_t u = f2u(x);
    uint32_t sign = (u >> 16) & 0x8000u;
    uint32_t a = u & 0x7fffffffu;
    if (a > 0x7f800000u) return (uint16_t)(sign | 0x7e00u);       /* NaN */
    if (a >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);      /* >= 65520 -> inf */
    if (a >= 0x38800000u) {                                       /* normal half */
        uint32_t h = (a - 0x38000000u) >> 13;                     /* rebias 127 -> 15 */
        uint32_t rem = a & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    /* subnormal half: units of 2^-24 */
    int e = (int)(a >> 23) - 127;
    uint32_t m = (a & 0x7fffffu) | (a ? 0x800000u : 0u);
    int s = -(e + 1);                     /* right shift that maps m to 2^-24 units */
    if (a == 0 || s > 24) return (uint16_t)sign;
    uint32_t h = m >> s;
    uint32_t rem = m & ((1u << s) - 1u);
    uint32_t half = 1u << (s - 1);
    if (rem > half || (rem == half && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

float orc_f16_bits_to_f32(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    if (e == 0x1fu) return u2f(sign | 0x7f800000u | (m << 13));
    if (e == 0) {
        /* subnormal: m * 2^-24, exact in float */
        float v = (float)m * 5.9604644775390625e-08f;
        return sign ? -v : v;
    }
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

uint16_t orc_f32_to_bf16_bits(float x) {
    uint32_t u = f2u(x);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

/* convert_short_sat_rte(x * 32767.0f): kernels_no_3d_write.cl:9-21 and the
 * OpenCL 1.1 rule for writes to CL_SNORM_INT16 images. */
int16_t orc_f32_to_snorm16(float x) {
    float f = x * 32767.0f;
    if (f != f) return 0;
    float r = rintf(f);                   /* default rounding mode: nearest even */
    if (r >= 32767.0f) return 32767;
    if (r <= -32768.0f) return -32768;
    return (int16_t)r;
}

float orc_snorm16_to_f32(int16_t s) {
    float v = (float)s / 32767.0f;
    return v < -1.0f ? -1.0f : v;
}

uint16_t orc_f32_to_unorm16(float x) {
    float f = x * 65535.0f;
    if (f != f) return 0;
    float r = rintf(f);
    if (r >= 65535.0f) return 65535;
    if (r <= 0.0f) return 0;
    return (uint16_t)r;
}

float orc_unorm16_to_f32(uint16_t u) { return (float)u / 65535.0f; }

float orc_quantize(float x, int storage) {
    switch (storage) {
    case ORC_F16: return orc_f16_bits_to_f32(orc_f32_to_f16_bits(x));
    case ORC_BF16: return u2f((uint32_t)orc_f32_to_bf16_bits(x) << 16);
    case ORC_SNORM16: return orc_snorm16_to_f32(orc_f32_to_snorm16(x));
    default: return x;
    }
}

void orc_quantize_array(float *a, int64_t n, int storage) {
    if (storage == ORC_F32) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) a[i] = orc_quantize(a[i], storage);
}

void orc_to_unorm16_array(const float *in, uint16_t *out, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = orc_f32_to_unorm16(in[i]);
}

void orc_from_unorm16_array(const uint16_t *in, float *out, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) out[i] = orc_unorm16_to_f32(in[i]);
}

/* ------------------------------------------------------------------------ */
/* Tables                                                                    */
/* ------------------------------------------------------------------------ */

void orc_circle_table(float cosv[32], float sinv[32]) {
    char buf[64];
    for (int j = 0; j < 32; j++) {
        snprintf(buf, sizeof buf, "%.6g", cos((double)j));
        cosv[j] = strtof(buf, NULL);
        snprintf(buf, sizeof buf, "%.6g", sin((double)j));
        sinv[j] = strtof(buf, NULL);
    }
}

void orc_arm_table(float cosv[12], float sinv[12]) {
    const float two_pi = 2.0f * 3.14159265358979323846f;   /* 2 * M_PI_F */
    for (int j = 0; j < 12; j++) {
        const float alpha = two_pi * (float)j / 12.0f;
        cosv[j] = (float)cos((double)alpha);
        sinv[j] = (float)sin((double)alpha);
    }
}

/* createBlurMask, tube-segmentation.cpp:188-211: half width m = ceil(sigma/0.5)
 * clamped to [1,5]; weights exp(-(a^2+b^2+c^2)/(2 sigma^2)) normalised to sum 1.
 * The exponential is evaluated in double (C exp) and rounded to float; the
 * running sum is kept in float, as in the reference host code. */
int orc_blur_mask(float sigma, float *mask) {
    int m = (int)ceilf(sigma / 0.5f);
    if (m < 1) m = 1;
    if (m > 5) m = 5;
    int S = 2 * m + 1;
    float sum = 0.0f;
    float two_s2 = (2.0f * sigma) * sigma;
    for (int a = -m; a <= m; a++)
        for (int b = -m; b <= m; b++)
            for (int c = -m; c <= m; c++) {
                float arg = -((float)(a * a + b * b + c * c) / two_s2);
                double w = exp((double)arg);
                sum = (float)((double)sum + w);
                mask[(a + m) + (b + m) * S + (c + m) * S * S] = (float)w;
            }
    for (int i = 0; i < S * S * S; i++) mask[i] = mask[i] / sum;
    return m;
}

/* ------------------------------------------------------------------------ */
/* Histogram pyramid (kernels.cl:63-299; oul::HistogramPyramid3D)            */
/* ------------------------------------------------------------------------ */

/* Child visiting order of one pyramid cell, cubeOffsets (kernels.cl:70-79). */
static const int k_cube[8][3] = {
    {0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1},
    {0, 1, 0}, {1, 1, 0}, {0, 1, 1}, {1, 1, 1},
};

int64_t orc_hp_compact(const int8_t *mask, int X, int Y, int Z, int32_t *pos, int64_t cap) {
    int hp = 8;
    int mx = X > Y ? X : Y;
    if (Z > mx) mx = Z;
    while (hp < mx) hp *= 2;
    int L = 0;
    while ((1 << L) < hp) L++;          /* levels 0..L-1, level k has size hp>>k */

    int32_t **lev = (int32_t **)calloc((size_t)L, sizeof(int32_t *));
    /* level 0: the mask, zero outside the volume */
    int64_t n0 = (int64_t)hp * hp * hp;
    lev[0] = (int32_t *)calloc((size_t)n0, sizeof(int32_t));
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++)
                lev[0][x + (int64_t)hp * (y + (int64_t)hp * z)] =
                    mask[x + (int64_t)X * (y + (int64_t)Y * z)] != 0;
    /* constructHPLevel3D: each cell = sum of its 8 children */
    for (int k = 1; k < L; k++) {
        int s = hp >> k, sp = hp >> (k - 1);
        lev[k] = (int32_t *)calloc((size_t)s * s * s, sizeof(int32_t));
        for (int z = 0; z < s; z++)
            for (int y = 0; y < s; y++)
                for (int x = 0; x < s; x++) {
                    int32_t acc = 0;
                    for (int c = 0; c < 8; c++) {
                        int xx = 2 * x + k_cube[c][0], yy = 2 * y + k_cube[c][1],
                            zz = 2 * z + k_cube[c][2];
                        acc += lev[k - 1][xx + (int64_t)sp * (yy + (int64_t)sp * zz)];
                    }
                    lev[k][x + (int64_t)s * (y + (int64_t)s * z)] = acc;
                }
    }
    int64_t sum = 0;
    {
        int s = hp >> (L - 1); /* == 2 */
        for (int i = 0; i < s * s * s; i++) sum += lev[L - 1][i];
    }
    /* traverseHP3D / scanHPLevel3D for every target rank */
    int64_t nout = sum < cap ? sum : cap;
    for (int64_t t = 0; t < nout; t++) {
        int cx = 0, cy = 0, cz = 0;
        int64_t acc0 = 0;
        for (int k = L - 1; k >= 0; k--) {
            int s = hp >> k;
            int64_t nb[8];
            for (int c = 0; c < 8; c++) {
                int xx = cx + k_cube[c][0], yy = cy + k_cube[c][1], zz = cz + k_cube[c][2];
                nb[c] = (xx < s && yy < s && zz < s)
                            ? lev[k][xx + (int64_t)s * (yy + (int64_t)s * zz)] : 0;
            }
            int64_t acc = acc0;
            int idx = 0;
            int64_t add = 0;
            for (int c = 0; c < 7; c++) {
                acc += nb[c];
                if (acc <= t) { idx++; add += nb[c]; }
            }
            cx += k_cube[idx][0]; cy += k_cube[idx][1]; cz += k_cube[idx][2];
            cx *= 2; cy *= 2; cz *= 2;
            acc0 += add;
        }
        pos[3 * t + 0] = cx / 2;
        pos[3 * t + 1] = cy / 2;
        pos[3 * t + 2] = cz / 2;
    }
    for (int k = 0; k < L; k++) free(lev[k]);
    free(lev);
    return sum;
}

static inline int orc_mirror(int w, int n) {
    int p = w == 0 ? 2 : w;
    return p >= n - 1 ? n - 3 : p;
}

void orc_gvf_residual_norm(const float *f0, const float *v, int X, int Y, int Z, float mu, int kind, double out[5]) {
    const int64_t n = (int64_t)X * Y * Z, sx = 1, sy = X, sz = (int64_t)X * Y;
    double acc[3] = {0.0, 0.0, 0.0};
    float amax = 0.0f;
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                const int64_t p = orc_mirror(x, X) + (int64_t)X * (orc_mirror(y, Y) + (int64_t)Y * orc_mirror(z, Z));
                const float fx = f0[p], fy = f0[n + p], fz = f0[2 * n + p];
                const float sqr = (fx * fx + fy * fy) + fz * fz;
                for (int c = 0; c < 3; c++) {
                    const float *vc = v + c * n;
                    const float fc = c == 0 ? fx : (c == 1 ? fy : fz);
                    float r;
                    if (kind == 0) {
                        float lap = -6.0f * vc[p];
                        lap = lap + vc[p + sx];
                        lap = lap + vc[p - sx];
                        lap = lap + vc[p + sy];
                        lap = lap + vc[p - sy];
                        lap = lap + vc[p + sz];
                        lap = lap + vc[p - sz];
                        r = mu * lap - (vc[p] - fc) * sqr;
                    } else {
                        float s6 = vc[p + sx] + vc[p - sx];
                        s6 = s6 + vc[p + sy];
                        s6 = s6 + vc[p - sy];
                        s6 = s6 + vc[p + sz];
                        s6 = s6 + vc[p - sz];
                        const float residue = (mu * (s6 - 6.0f * vc[p])) / 1.0f;
                        r = -sqr * fc - (residue - sqr * vc[p]);
                    }
                    acc[c] += (double)r * (double)r;
                    if (fabsf(r) > amax) amax = fabsf(r);
                }
            }
    out[0] = sqrt(acc[0]);
    out[1] = sqrt(acc[1]);
    out[2] = sqrt(acc[2]);
    out[3] = sqrt((acc[0] + acc[1]) + acc[2]);
    out[4] = amax;
}

void orc_threshold_f32(const float *T, int64_t n, float thr, int8_t *mask) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) mask[i] = (T[i] < thr) ? 0 : 1;
}

/* ------------------------------------------------------------------------ */
/* Centerline linking (runNewCenterlineAlg back half,                       */
/* parallelCenterlineExtraction.cpp:911-1332; kernels.cl:327-559)           */
/* ------------------------------------------------------------------------ */

#define CLAMPI(v, n) ((v) < 0 ? 0 : ((v) >= (n) ? (n) - 1 : (v)))

static float orc_vdist(const int32_t *v, int a, int b) {
    const float dx = (float)v[3 * a] - (float)v[3 * b];
    const float dy = (float)v[3 * a + 1] - (float)v[3 * b + 1];
    const float dz = (float)v[3 * a + 2] - (float)v[3 * b + 2];
    return sqrtf((dx * dx + dy * dy) + dz * dz);
}

/* the TDF through OpenCL's linear sampler (unnormalised, clamp to edge) */
static float orc_sample_tdf(const float *T, int X, int Y, int Z, float u, float v, float w) {
    const float uu = u - 0.5f, vv = v - 0.5f, ww = w - 0.5f;
    const float fu = floorf(uu), fv = floorf(vv), fw = floorf(ww);
    const float a = uu - fu, b = vv - fv, c = ww - fw;
    int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const int i1 = CLAMPI(i0 + 1, X), j1 = CLAMPI(j0 + 1, Y), k1 = CLAMPI(k0 + 1, Z);
    i0 = CLAMPI(i0, X); j0 = CLAMPI(j0, Y); k0 = CLAMPI(k0, Z);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
#define TT(i, j, k) T[(int64_t)(i) + (int64_t)X * ((int64_t)(j) + (int64_t)Y * (int64_t)(k))]
    float o = ((ia * ib) * ic) * TT(i0, j0, k0);
    o = o + ((a * ib) * ic) * TT(i1, j0, k0);
    o = o + ((ia * b) * ic) * TT(i0, j1, k0);
    o = o + ((a * b) * ic) * TT(i1, j1, k0);
    o = o + ((ia * ib) * c) * TT(i0, j0, k1);
    o = o + ((a * ib) * c) * TT(i1, j0, k1);
    o = o + ((ia * b) * c) * TT(i0, j1, k1);
    o = o + ((a * b) * c) * TT(i1, j1, k1);
#undef TT
    return o;
}

static float orc_mean_tdf(const float *T, int X, int Y, int Z, const float xa[3], const float s[3], int d) {
    float sum = 0.0f;
    for (int k = 0; k <= d; k++) {
        const float alpha = (float)k / (float)d;
        sum = sum + orc_sample_tdf(T, X, Y, Z, xa[0] + s[0] * alpha, xa[1] + s[1] * alpha, xa[2] + s[2] * alpha);
    }
    return sum / (float)(d + 1);
}

static uint32_t orc_hp2d_key(uint32_t x, uint32_t y) {
    uint32_t k = 0;
    for (int bit = 0; bit < 16; bit++) k |= (((y >> bit) & 1u) | (((x >> bit) & 1u) << 1)) << (2 * bit);
    return k;
}

static int orc_cmp_u32(const void *a, const void *b) {
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static int orc_find(int *parent, int i) {
    while (parent[i] != i) i = parent[i];
    return i;
}

int orc_link_centerpoints(const int32_t *v, int n, const float *T, int X, int Y, int Z, float min_avg, float maxd,
                          int32_t *edges, int32_t *labels, int32_t *sizes) {
    /* candidate lists, ascending partner (linkLengths + compact) */
    int *cnt = (int *)calloc((size_t)n, sizeof(int));
    int *lst = (int *)malloc(sizeof(int) * (size_t)n * (size_t)n);
    float *len = (float *)malloc(sizeof(float) * (size_t)n * (size_t)n);
    int *partner = (int *)malloc(sizeof(int) * 2 * (size_t)n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int a = 0; a < n; a++) {
        int c = 0;
        for (int b = 0; b < n; b++) {
            const float d = orc_vdist(v, a, b);
            if (d < maxd && d > 0.0f) {
                lst[(size_t)a * n + c] = b;
                len[(size_t)a * n + c] = d;
                c++;
            }
        }
        cnt[a] = c;
    }
    /* linkCenterpoints */
#pragma omp parallel for schedule(dynamic, 16)
    for (int a = 0; a < n; a++) {
        const float xa[3] = {(float)v[3 * a], (float)v[3 * a + 1], (float)v[3 * a + 2]};
        float shortest = maxd * 2.0f;
        int best_b = -1, best_c = -1;
        for (int i = 0; i < cnt[a]; i++) {
            const int b = lst[(size_t)a * n + i];
            const int db = (int)roundf(len[(size_t)a * n + i]);
            if ((float)db >= shortest) continue;
            const float ab[3] = {(float)v[3 * b] - xa[0], (float)v[3 * b + 1] - xa[1], (float)v[3 * b + 2] - xa[2]};
            for (int j = 0; j < i; j++) {
                const int c = lst[(size_t)a * n + j];
                if (c == b) continue;
                const int dc = (int)roundf(len[(size_t)a * n + j]);
                if (!((float)(db + dc) < shortest)) continue;
                const float ac[3] = {(float)v[3 * c] - xa[0], (float)v[3 * c + 1] - xa[1],
                                     (float)v[3 * c + 2] - xa[2]};
                const float lb = sqrtf((ab[0] * ab[0] + ab[1] * ab[1]) + ab[2] * ab[2]);
                const float lc = sqrtf((ac[0] * ac[0] + ac[1] * ac[1]) + ac[2] * ac[2]);
                const float dot =
                    ((ab[0] / lb) * (ac[0] / lc) + (ab[1] / lb) * (ac[1] / lc)) + (ab[2] / lb) * (ac[2] / lc);
                if (dot > -0.41614684f) continue; /* acos(dot) < 2 */
                if (orc_mean_tdf(T, X, Y, Z, xa, ab, db) < min_avg) continue;
                if (orc_mean_tdf(T, X, Y, Z, xa, ac, dc) < min_avg) continue;
                best_b = b;
                best_c = c;
                shortest = (float)(db + dc);
            }
        }
        partner[2 * a] = best_b;
        partner[2 * a + 1] = best_c;
    }
    /* removeDuplicateEdges, then the 2-D pyramid order */
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)n);
    int ne = 0;
    for (int t = 0; t < 2 * n; t++) {
        const int a = t >> 1, b = partner[t];
        if (b < 0) continue;
        const int back = partner[2 * b] == a || partner[2 * b + 1] == a;
        if (a <= b || !back) keys[ne++] = orc_hp2d_key((uint32_t)a, (uint32_t)b);
    }
    qsort(keys, (size_t)ne, sizeof(uint32_t), orc_cmp_u32);
    for (int e = 0; e < ne; e++) {
        uint32_t x = 0, y = 0;
        for (int bit = 0; bit < 16; bit++) {
            y |= ((keys[e] >> (2 * bit)) & 1u) << bit;
            x |= ((keys[e] >> (2 * bit + 1)) & 1u) << bit;
        }
        edges[2 * e] = (int32_t)x;
        edges[2 * e + 1] = (int32_t)y;
    }
    /* components labelled by their smallest vertex; sizes */
    int *parent = (int *)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < n; i++) parent[i] = i;
    for (int e = 0; e < ne; e++) {
        const int ra = orc_find(parent, edges[2 * e]), rb = orc_find(parent, edges[2 * e + 1]);
        if (ra < rb) parent[rb] = ra;
        else if (rb < ra) parent[ra] = rb;
    }
    for (int i = 0; i < n; i++) {
        labels[i] = orc_find(parent, i);
        sizes[i] = 0;
    }
    for (int i = 0; i < n; i++) sizes[labels[i]]++;
    free(cnt); free(lst); free(len); free(partner); free(keys); free(parent);
    return ne;
}

void orc_rasterize_trees(const int32_t *v, const int32_t *edges, int ne, const int32_t *labels,
                         const int32_t *sizes, int min_tree, int8_t *out, int X, int Y, int Z) {
    for (int e = 0; e < ne; e++) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        if (sizes[labels[a]] < min_tree) continue;
        const float xa[3] = {(float)v[3 * a], (float)v[3 * a + 1], (float)v[3 * a + 2]};
        const float d[3] = {(float)v[3 * b] - xa[0], (float)v[3 * b + 1] - xa[1], (float)v[3 * b + 2] - xa[2]};
        const int l = (int)roundf(sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]));
        for (int i = 0; i < l; i++) {
            const float alpha = (float)i / (float)l;
            const int x = (int)roundf(xa[0] + d[0] * alpha), y = (int)roundf(xa[1] + d[1] * alpha),
                      z = (int)roundf(xa[2] + d[2] * alpha);
            if (x >= 0 && y >= 0 && z >= 0 && x < X && y < Y && z < Z)
                out[(int64_t)x + (int64_t)X * ((int64_t)y + (int64_t)Y * z)] = 1;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Segmentation (segmentation.cpp:5-307; kernels_no_3d_write.cl:1100-1235,   */
/* 1370-1412).  Reads clamp to the edge (the reference's sampler), writes    */
/* outside the volume are dropped (the buffer kernels' bounds checks).       */
/* ------------------------------------------------------------------------ */

#define SEG_IDX(x, y, z) ((int64_t)(x) + (int64_t)X * ((int64_t)(y) + (int64_t)Y * (int64_t)(z)))
#define SEG_IN(x, y, z) ((x) >= 0 && (y) >= 0 && (z) >= 0 && (x) < X && (y) < Y && (z) < Z)

/* initGrowing (kernels_no_3d_write.cl:1100-1124) on state = copy of cl */
static void seg_init_growing(const int8_t *cl, const float *radius, int8_t *state, int X, int Y, int Z) {
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                if (cl[SEG_IDX(x, y, z)] != 1) continue;
                int N = (int)roundf(radius[SEG_IDX(x, y, z)] / 2.0f);
                if (N < 1) N = 1;
                if (N > 4) N = 4;
                for (int a = -N; a <= N; a++)
                    for (int b = -N; b <= N; b++)
                        for (int c = -N; c <= N; c++) {
                            const int nx = x + a, ny = y + b, nz = z + c;
                            if (!SEG_IN(nx, ny, nz)) continue;
                            if (cl[SEG_IDX(nx, ny, nz)] == 0) state[SEG_IDX(nx, ny, nz)] = 2;
                        }
            }
}

/* One grow iteration (kernels_no_3d_write.cl:1128-1207): decide from `cur`,
 * then apply with the precedence accepted > to check > dropped (the reference
 * races these writes).  Returns 1 if anything was accepted. */
static int seg_grow_once(int8_t *cur, int8_t *acc, int8_t *mark, const float *F, int X, int Y, int Z) {
    int any = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : any)
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                const int64_t i = SEG_IDX(x, y, z);
                if (cur[i] != 2) continue;
                const float wX = F[4 * i + 3];
                int grew = 0;
                for (int a = -1; a < 2; a++)
                    for (int b = -1; b < 2; b++)
                        for (int c = -1; c < 2; c++) {
                            if (a == 0 && b == 0 && c == 0) continue;
                            const int yx = x + a, yy = y + b, yz = z + c;
                            const int64_t j = SEG_IDX(CLAMPI(yx, X), CLAMPI(yy, Y), CLAMPI(yz, Z));
                            if (cur[j] == 1) continue;
                            const float w = F[4 * j + 3];
                            const float fx = F[4 * j] / w, fy = F[4 * j + 1] / w, fz = F[4 * j + 2] / w;
                            if (!(w > wX)) continue;
                            /* the neighbour of Y whose direction best matches F(Y) */
                            float best = -2.0f;
                            int zx = 0, zy = 0, zz = 0;
                            for (int a2 = -1; a2 < 2; a2++)
                                for (int b2 = -1; b2 < 2; b2++)
                                    for (int c2 = -1; c2 < 2; c2++) {
                                        if (a2 == 0 && b2 == 0 && c2 == 0) continue;
                                        const float l = sqrtf((float)(a2 * a2 + b2 * b2 + c2 * c2));
                                        const float dx = (float)a2 / l, dy = (float)b2 / l, dz = (float)c2 / l;
                                        const float v = (fx * dx + fy * dy) + fz * dz;
                                        if (v > best) {
                                            best = v;
                                            zx = yx + a2;
                                            zy = yy + b2;
                                            zz = yz + c2;
                                        }
                                    }
                            if (zx != x || zy != y || zz != z) continue;
                            if (!SEG_IN(yx, yy, yz)) continue;  /* accepted only through Y inside */
#pragma omp atomic write
                            mark[SEG_IDX(yx, yy, yz)] = 1;
                            grew = 1;
                        }
                if (grew) {
                    acc[i] = 1;
                    any = 1;
                }
            }
    const int64_t n = (int64_t)X * Y * Z;
    for (int64_t i = 0; i < n; i++) {
        cur[i] = (cur[i] == 1 || acc[i]) ? 1 : (mark[i] ? 2 : 0);
        acc[i] = 0;
        mark[i] = 0;
    }
    return any;
}

int orc_segment_inverse_gradient(const int8_t *cl, const float *field4, const float *radius, int X, int Y, int Z,
                                 int8_t *out) {
    const int64_t n = (int64_t)X * Y * Z;
    int8_t *cur = (int8_t *)malloc((size_t)n), *acc = (int8_t *)calloc((size_t)n, 1),
           *mark = (int8_t *)calloc((size_t)n, 1), *dil = (int8_t *)calloc((size_t)n, 1);
    memcpy(cur, cl, (size_t)n);
    seg_init_growing(cl, radius, cur, X, Y, Z);
    int it = 0;
    for (;;) {
        it++;
        if (!seg_grow_once(cur, acc, mark, field4, X, Y, Z)) break;
    }
    /* dilate (kernels_no_3d_write.cl:1370-1389) into a zeroed volume */
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                if (cur[SEG_IDX(x, y, z)] != 1) continue;
                for (int a = -1; a < 2; a++)
                    for (int b = -1; b < 2; b++)
                        for (int c = -1; c < 2; c++)
                            if (SEG_IN(x + a, y + b, z + c)) dil[SEG_IDX(x + a, y + b, z + c)] = 1;
            }
    /* erode (kernels_no_3d_write.cl:1391-1412), clamp-to-edge reads */
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                int keep = dil[SEG_IDX(x, y, z)] == 1;
                for (int a = -1; a < 2; a++)
                    for (int b = -1; b < 2; b++)
                        for (int c = -1; c < 2; c++)
                            keep = keep && dil[SEG_IDX(CLAMPI(x + a, X), CLAMPI(y + b, Y), CLAMPI(z + c, Z))] == 1;
                out[SEG_IDX(x, y, z)] = keep ? 1 : 0;
            }
    free(cur);
    free(acc);
    free(mark);
    free(dil);
    return it;
}

/* sphereSegmentation (kernels_no_3d_write.cl:1209-1234) into a zeroed out */
void orc_segment_spheres(const int8_t *cl, const float *radius, int X, int Y, int Z, int8_t *out) {
    memset(out, 0, (size_t)X * Y * Z);
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                if (cl[SEG_IDX(x, y, z)] == 0) continue;
                const float r = radius[SEG_IDX(x, y, z)];
                if (!(r > 0.0f)) continue;
                const int M = X > Y ? (X > Z ? X : Z) : (Y > Z ? Y : Z);
                const int N = (int)ceilf(r < (float)M ? r : (float)M);
                for (int a = -N; a <= N; a++)
                    for (int b = -N; b <= N; b++)
                        for (int c = -N; c <= N; c++) {
                            if (!(sqrtf((float)(a * a + b * b + c * c)) < r)) continue;
                            if (SEG_IN(x + a, y + b, z + c)) out[SEG_IDX(x + a, y + b, z + c)] = 1;
                        }
            }
}

/* ------------------------------------------------------------------------ */
/* Cropping (cropDatasetThreshold / cropDatasetLung, kernels.cl:813-946),    */
/* one pass per slice direction as the reference enqueues them               */
/* (tube-segmentation.cpp:1577-1604).  type: ORC_RAW_*.                       */
/* ------------------------------------------------------------------------ */

static double crop_value(const void *vol, int type, int64_t i) {
    switch (type) {
    case ORC_RAW_U8: return (double)((const uint8_t *)vol)[i];
    case ORC_RAW_I8: return (double)((const int8_t *)vol)[i];
    case ORC_RAW_U16: return (double)((const uint16_t *)vol)[i];
    case ORC_RAW_I16: return (double)((const int16_t *)vol)[i];
    default: return (double)((const float *)vol)[i];
    }
}

void orc_crop_scan_lines(const void *vol, int type, int X, int Y, int Z, int method, float threshold,
                         int16_t *counts) {
    const int unsigned_type = type == ORC_RAW_U8 || type == ORC_RAW_U16;
    const int hu_limit = unsigned_type ? -150 + 1024 : -150;
    const int ext[3] = {X, Y, Z};
    int16_t *out[3] = {counts, counts + X, counts + X + Y};
    for (int dir = 0; dir < 3; dir++) {
        const int line_n = dir == 1 ? X : Y;      /* scanLineSize */
        const int elem_n = dir == 2 ? X : Z;      /* scanLineElementSize */
        for (int slice = 0; slice < ext[dir]; slice++) {
            int16_t lines = 0;
            for (int line = 0; line < line_n; line++) {
                int found = 0, w = 0, b = 0, dw = 0, db = 0;
                for (int e = 0; e < elem_n; e++) {
                    int x, y, z;
                    if (dir == 0) { x = slice; y = line; z = e; }
                    else if (dir == 1) { x = line; y = slice; z = e; }
                    else { x = e; y = line; z = slice; }
                    const int64_t i = (int64_t)x + (int64_t)X * ((int64_t)y + (int64_t)Y * z);
                    if (method == 0) {
                        /* integer values convert to float for the comparison */
                        const float v = type == ORC_RAW_F32 ? ((const float *)vol)[i] : (float)crop_value(vol, type, i);
                        if (v > threshold) found = 1;
                    } else {
                        /* the read value stored into a short */
                        int hu;
                        if (type == ORC_RAW_U16) hu = (int16_t)((const uint16_t *)vol)[i];
                        else hu = (int16_t)(int)crop_value(vol, type, i);
                        if (hu > hu_limit) {
                            if (w == 30) { dw++; b = 0; }
                            w++;
                        } else {
                            if (b == 30) { db++; w = 0; }
                            b++;
                        }
                    }
                }
                if (method == 0 ? found : ((dw == 2 && db == 1) || (db > 1 && dw > 1))) lines++;
            }
            out[dir][slice] = lines;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Precision-templated kernels                                               */
/* ------------------------------------------------------------------------ */

#define REAL float
#define SUFFIX _f32
#define ORC_IS_F32 1
#include "tsf_oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef ORC_IS_F32

#define REAL double
#define SUFFIX _f64
#define ORC_IS_F32 0
#include "tsf_oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef ORC_IS_F32
