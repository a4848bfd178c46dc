/*
 * tsf_oracle_impl.h -- precision-templated body of the oracle (TEST
 * INFRASTRUCTURE ONLY; included twice by tsf_oracle.c with REAL = float /
 * double).  Parity against the reference's outputs: unpinned (see
 * tsf_oracle.h).
 *
 * Float instantiation (_f32): same arithmetic, same operation order and the
 * same storage rounding as the CUDA kernels.  Double instantiation (_f64): the
 * FP64 oracle; storage rounding is skipped (the exact method).
 */

#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define FN(name) ORC_CAT(name, SUFFIX)

#if ORC_IS_F32
#define RSQRT_(x) sqrtf(x)
#define RFABS_(x) fabsf(x)
#define RFLOOR_(x) floorf(x)
#define RROUND_(x) roundf(x)
#define Q_(x, st) orc_quantize((x), (st))
#else
#define RSQRT_(x) sqrt(x)
#define RFABS_(x) fabs(x)
#define RFLOOR_(x) floor(x)
#define RROUND_(x) round(x)
#define Q_(x, st) (x)
#endif

#define IDX(x, y, z) ((int64_t)(x) + (int64_t)X * ((int64_t)(y) + (int64_t)Y * (int64_t)(z)))

static inline int FN(clampi)(int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

/* Mirror boundary rule of GVF3DIteration and the multigrid kernels
 * (kernels.cl:1472-1475): index 0 reads the stencil at 2, indices >= size-1
 * read the stencil at size-3; the two selects are applied in that order. */
static inline int FN(mirror)(int w, int n) {
    int p = (w == 0) ? 2 : w;
    return (p >= n - 1) ? n - 3 : p;
}

/* blurVolumeWithGaussian, kernels.cl:1017-1040.  Nearest read, clamp to edge.
 * Loop order c (z) outer, b (y), a (x) inner; float accumulation. */
void FN(orc_blur)(const float *in, int X, int Y, int Z, int m, const float *mask, REAL *out) {
    int S = 2 * m + 1;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                REAL sum = 0;
                for (int c = -m; c <= m; c++)
                    for (int b = -m; b <= m; b++)
                        for (int a = -m; a <= m; a++) {
                            REAL w = (REAL)mask[(a + m) + (b + m) * S + (c + m) * S * S];
                            REAL v = (REAL)in[IDX(FN(clampi)(x + a, X), FN(clampi)(y + b, Y),
                                                  FN(clampi)(z + c, Z))];
                            sum = sum + w * v;
                        }
                out[IDX(x, y, z)] = sum;
            }
}

/* createVectorField, kernels.cl:1042-1063 (with gradient, kernels.cl:756-810):
 * F = vsign * 0.5*(I(x+1)-I(x-1), ...) with clamp-to-edge reads,
 * F <- F/Fmax if |F| < Fmax else F/|F|, w = 1; stored in `storage`. */
void FN(orc_vector_field)(const REAL *in, int X, int Y, int Z, float Fmax, int vsign,
                          int storage, REAL *field4) {
    const REAL fmax = (REAL)Fmax;
    const REAL sg = (REAL)vsign;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                REAL gx = (REAL)0.5 * (in[IDX(FN(clampi)(x + 1, X), y, z)] -
                                       in[IDX(FN(clampi)(x - 1, X), y, z)]);
                REAL gy = (REAL)0.5 * (in[IDX(x, FN(clampi)(y + 1, Y), z)] -
                                       in[IDX(x, FN(clampi)(y - 1, Y), z)]);
                REAL gz = (REAL)0.5 * (in[IDX(x, y, FN(clampi)(z + 1, Z))] -
                                       in[IDX(x, y, FN(clampi)(z - 1, Z))]);
                REAL Fx = sg * gx, Fy = sg * gy, Fz = sg * gz;
                REAL l = RSQRT_((Fx * Fx + Fy * Fy) + Fz * Fz);
                if (l < fmax) {
                    Fx = Fx / fmax; Fy = Fy / fmax; Fz = Fz / fmax;
                } else {
                    Fx = Fx / l; Fy = Fy / l; Fz = Fz / l;
                }
                int64_t i = IDX(x, y, z);
                field4[4 * i + 0] = Q_(Fx, storage);
                field4[4 * i + 1] = Q_(Fy, storage);
                field4[4 * i + 2] = Q_(Fz, storage);
                field4[4 * i + 3] = Q_((REAL)1, storage);
            }
}

/* GVF3DInit, kernels.cl:1495-1503: v0 = f0.  The planar copies keep the three
 * components of f0 (the reference keeps x,y in an RG image and z in v.w). */
void FN(orc_gvf_init)(const REAL *field4, int64_t n, REAL *v_planar, REAL *f_planar) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            v_planar[c * n + i] = field4[4 * i + c];
            f_planar[c * n + i] = field4[4 * i + c];
        }
}

/* GVF3DIteration, kernels.cl:1464-1493, repeated `iterations` times with the
 * ping-pong of gradientVectorFlow.cpp:1137-1151.  Per component:
 *   L = -6 v + v(x+1) + v(x-1) + v(y+1) + v(y-1) + v(z+1) + v(z-1)
 *   v <- v + (mu L - (v - f) |f|^2),  |f|^2 = fx^2 + fy^2 + fz^2,
 * evaluated at the mirror-mapped position and stored in `storage`. */
void FN(orc_gvf)(const REAL *f, REAL *v, int X, int Y, int Z, float mu_, int iterations,
                 int storage) {
    const int64_t n = (int64_t)X * Y * Z;
    const REAL mu = (REAL)mu_;
    REAL *w = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)n);
    REAL *src = v, *dst = w;
    for (int it = 0; it < iterations; it++) {
#pragma omp parallel for schedule(static)
        for (int z = 0; z < Z; z++)
            for (int y = 0; y < Y; y++)
                for (int x = 0; x < X; x++) {
                    int px = FN(mirror)(x, X), py = FN(mirror)(y, Y), pz = FN(mirror)(z, Z);
                    int64_t p = IDX(px, py, pz);
                    REAL fx = f[p], fy = f[n + p], fz = f[2 * n + p];
                    REAL sqr = (fx * fx + fy * fy) + fz * fz;
                    int64_t xp = IDX(FN(clampi)(px + 1, X), py, pz);
                    int64_t xm = IDX(FN(clampi)(px - 1, X), py, pz);
                    int64_t yp = IDX(px, FN(clampi)(py + 1, Y), pz);
                    int64_t ym = IDX(px, FN(clampi)(py - 1, Y), pz);
                    int64_t zp = IDX(px, py, FN(clampi)(pz + 1, Z));
                    int64_t zm = IDX(px, py, FN(clampi)(pz - 1, Z));
                    int64_t o = IDX(x, y, z);
                    for (int c = 0; c < 3; c++) {
                        const REAL *s = src + c * n;
                        REAL vc = s[p];
                        REAL lap = (REAL)(-6) * vc;
                        lap = lap + s[xp];
                        lap = lap + s[xm];
                        lap = lap + s[yp];
                        lap = lap + s[ym];
                        lap = lap + s[zp];
                        lap = lap + s[zm];
                        REAL fc = f[c * n + p];
                        REAL upd = mu * lap - (vc - fc) * sqr;
                        dst[c * n + o] = Q_(vc + upd, storage);
                    }
                }
        REAL *t = src; src = dst; dst = t;
    }
    if (src != v) memcpy(v, src, sizeof(REAL) * 3 * (size_t)n);
    free(w);
}

/* GVF3DFinish, kernels.cl:1506-1515: w = |v| (1 if |v| == 0). */
void FN(orc_gvf_finish)(const REAL *v, int64_t n, int storage, REAL *field4) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        REAL x = v[i], y = v[n + i], z = v[2 * n + i];
        REAL l = RSQRT_((x * x + y * y) + z * z);
        field4[4 * i + 0] = Q_(x, storage);
        field4[4 * i + 1] = Q_(y, storage);
        field4[4 * i + 2] = Q_(z, storage);
        field4[4 * i + 3] = Q_(l > 0 ? l : (REAL)1, storage);
    }
}

/* Low-memory GVF, one component at a time (runLowMemoryGVF,
 * gradientVectorFlow.cpp:1172-1300; GVF3DInit_one_component /
 * GVF3DIteration_one_component / GVF3DFinish_one_component,
 * kernels_no_3d_write.cl:1669-1741, image variant kernels.cl:1392-1462):
 * per component c, v = f0_c and the init pair (f0_c, |f0|^2) are stored in
 * `storage`, then
 *   v <- v + (mu L - (v - f0_c) sq),  sq = the stored |f0|^2,
 * `iterations` times with the mirror rule; finally w = |v| as GVF3DFinish. */
void FN(orc_gvf_one_component)(const REAL *field4, int X, int Y, int Z, float mu_, int iterations,
                               int storage, REAL *out4) {
    const int64_t n = (int64_t)X * Y * Z;
    const REAL mu = (REAL)mu_;
    REAL *v = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)n);
    REAL *w = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    REAL *f = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    REAL *sq = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    for (int c = 0; c < 3; c++) {
        REAL *vc = v + c * n;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            const REAL a = field4[4 * i + 0], b = field4[4 * i + 1], d = field4[4 * i + 2];
            vc[i] = f[i] = Q_(field4[4 * i + c], storage);
            sq[i] = Q_((a * a + b * b) + d * d, storage);
        }
        REAL *src = vc, *dst = w;
        for (int it = 0; it < iterations; it++) {
#pragma omp parallel for schedule(static)
            for (int z = 0; z < Z; z++)
                for (int y = 0; y < Y; y++)
                    for (int x = 0; x < X; x++) {
                        int px = FN(mirror)(x, X), py = FN(mirror)(y, Y), pz = FN(mirror)(z, Z);
                        int64_t p = IDX(px, py, pz);
                        REAL vv = src[p];
                        REAL lap = (REAL)(-6) * vv;
                        lap = lap + src[IDX(FN(clampi)(px + 1, X), py, pz)];
                        lap = lap + src[IDX(FN(clampi)(px - 1, X), py, pz)];
                        lap = lap + src[IDX(px, FN(clampi)(py + 1, Y), pz)];
                        lap = lap + src[IDX(px, FN(clampi)(py - 1, Y), pz)];
                        lap = lap + src[IDX(px, py, FN(clampi)(pz + 1, Z))];
                        lap = lap + src[IDX(px, py, FN(clampi)(pz - 1, Z))];
                        REAL upd = mu * lap - (vv - f[p]) * sq[p];
                        dst[IDX(x, y, z)] = Q_(vv + upd, storage);
                    }
            REAL *t = src; src = dst; dst = t;
        }
        if (src != vc) memcpy(vc, src, sizeof(REAL) * (size_t)n);
    }
    FN(orc_gvf_finish)(v, n, storage, out4);
    free(v); free(w); free(f); free(sq);
}

/* ---------------------------------------------------------------------------
 * 3x3 symmetric eigen-decomposition: Householder tridiagonalisation followed by
 * the implicit QL method (the EISPACK tred2/tql2 procedures of Bowdler, Martin,
 * Reinsch and Wilkinson, Handbook for Automatic Computation vol. II), as used
 * by the reference at kernels.cl:1519-1773 and eigenanalysisOfHessian.cpp:10-260.
 * The tolerance is 2^-52 in both precisions (kernels.cl:1660).  The QL sweep is
 * capped at 64 iterations (the reference has no cap).  Eigenvalues are sorted
 * by ascending magnitude; eigenvectors are the columns of V (V[row*3+col]).
 * ------------------------------------------------------------------------- */
static void FN(orc_tred2)(REAL V[3][3], REAL d[3], REAL e[3]) {
    const int n = 3;
    for (int j = 0; j < n; j++) d[j] = V[n - 1][j];
    for (int i = n - 1; i > 0; i--) {
        REAL scale = 0, h = 0;
        for (int k = 0; k < i; k++) scale = scale + RFABS_(d[k]);
        if (scale == 0) {
            e[i] = d[i - 1];
            for (int j = 0; j < i; j++) {
                d[j] = V[i - 1][j];
                V[i][j] = 0;
                V[j][i] = 0;
            }
        } else {
            for (int k = 0; k < i; k++) {
                d[k] = d[k] / scale;
                h = h + d[k] * d[k];
            }
            REAL f = d[i - 1];
            REAL g = RSQRT_(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int j = 0; j < i; j++) e[j] = 0;
            for (int j = 0; j < i; j++) {
                f = d[j];
                V[j][i] = f;
                g = e[j] + V[j][j] * f;
                for (int k = j + 1; k <= i - 1; k++) {
                    g = g + V[k][j] * d[k];
                    e[k] = e[k] + V[k][j] * f;
                }
                e[j] = g;
            }
            f = 0;
            for (int j = 0; j < i; j++) {
                e[j] = e[j] / h;
                f = f + e[j] * d[j];
            }
            REAL hh = f / (h + h);
            for (int j = 0; j < i; j++) e[j] = e[j] - hh * d[j];
            for (int j = 0; j < i; j++) {
                f = d[j];
                g = e[j];
                for (int k = j; k <= i - 1; k++) V[k][j] = V[k][j] - (f * e[k] + g * d[k]);
                d[j] = V[i - 1][j];
                V[i][j] = 0;
            }
        }
        d[i] = h;
    }
    for (int i = 0; i < n - 1; i++) {
        V[n - 1][i] = V[i][i];
        V[i][i] = 1;
        REAL h = d[i + 1];
        if (h != 0) {
            for (int k = 0; k <= i; k++) d[k] = V[k][i + 1] / h;
            for (int j = 0; j <= i; j++) {
                REAL g = 0;
                for (int k = 0; k <= i; k++) g = g + V[k][i + 1] * V[k][j];
                for (int k = 0; k <= i; k++) V[k][j] = V[k][j] - g * d[k];
            }
        }
        for (int k = 0; k <= i; k++) V[k][i + 1] = 0;
    }
    for (int j = 0; j < n; j++) {
        d[j] = V[n - 1][j];
        V[n - 1][j] = 0;
    }
    V[n - 1][n - 1] = 1;
    e[0] = 0;
}

static inline REAL FN(orc_hyp)(REAL a, REAL b) { return RSQRT_(a * a + b * b); }

static void FN(orc_tql2)(REAL V[3][3], REAL d[3], REAL e[3]) {
    const int n = 3;
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = 0;
    REAL f = 0, tst1 = 0;
    const REAL eps = (REAL)2.220446049250313080847263336181640625e-16; /* 2^-52 */
    for (int l = 0; l < n; l++) {
        REAL t = RFABS_(d[l]) + RFABS_(e[l]);
        tst1 = tst1 > t ? tst1 : t;
        int m = l;
        while (m < n) {
            if (RFABS_(e[m]) <= eps * tst1) break;
            m++;
        }
        if (m > n - 1) m = n - 1; /* only with NaN input: e[n-1] == 0 ends the search */
        if (m > l) {
            int iter = 0;
            do {
                iter++;
                REAL g = d[l];
                REAL p = (d[l + 1] - g) / ((REAL)2 * e[l]);
                REAL r = FN(orc_hyp)(p, (REAL)1);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                REAL dl1 = d[l + 1];
                REAL h = g - d[l];
                for (int i = l + 2; i < n; i++) d[i] = d[i] - h;
                f = f + h;
                p = d[m];
                REAL c = 1, c2 = 1, c3 = 1;
                REAL el1 = e[l + 1];
                REAL s = 0, s2 = 0;
                for (int i = m - 1; i >= l; i--) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = FN(orc_hyp)(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < n; k++) {
                        h = V[k][i + 1];
                        V[k][i + 1] = s * V[k][i] + c * h;
                        V[k][i] = c * V[k][i] - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (RFABS_(e[l]) > eps * tst1 && iter < 64);
        }
        d[l] = d[l] + f;
        e[l] = 0;
    }
    for (int i = 0; i < n - 1; i++) {
        int k = i;
        REAL p = d[i];
        for (int j = i + 1; j < n; j++)
            if (RFABS_(d[j]) < RFABS_(p)) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int j = 0; j < n; j++) {
                p = V[j][i];
                V[j][i] = V[j][k];
                V[j][k] = p;
            }
        }
    }
}

void FN(orc_eig3)(const REAL A[9], REAL Vout[9], REAL d[3]) {
    REAL V[3][3], e[3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) V[i][j] = A[3 * i + j];
    FN(orc_tred2)(V, d, e);
    FN(orc_tql2)(V, d, e);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Vout[3 * i + j] = V[i][j];
}

/* Hessian of the vector field at (x,y,z) (kernels.cl:1081-1098 with gradient /
 * gradientNormalized, kernels.cl:700-810): central differences with
 * clamp-to-edge reads; `normalized` divides each neighbour by its w. */
static void FN(orc_hessian)(const REAL *F, int X, int Y, int Z, int x, int y, int z,
                            int normalized, REAL H[3][3]) {
    const REAL *xp = F + 4 * IDX(FN(clampi)(x + 1, X), y, z);
    const REAL *xm = F + 4 * IDX(FN(clampi)(x - 1, X), y, z);
    const REAL *yp = F + 4 * IDX(x, FN(clampi)(y + 1, Y), z);
    const REAL *ym = F + 4 * IDX(x, FN(clampi)(y - 1, Y), z);
    const REAL *zp = F + 4 * IDX(x, y, FN(clampi)(z + 1, Z));
    const REAL *zm = F + 4 * IDX(x, y, FN(clampi)(z - 1, Z));
    const REAL h = (REAL)0.5;
    REAL Fxx, Fyx, Fyy, Fzx, Fzy, Fzz;
    if (normalized) {
        Fxx = h * (xp[0] / xp[3] - xm[0] / xm[3]);
        Fyx = h * (xp[1] / xp[3] - xm[1] / xm[3]);
        Fyy = h * (yp[1] / yp[3] - ym[1] / ym[3]);
        Fzx = h * (xp[2] / xp[3] - xm[2] / xm[3]);
        Fzy = h * (yp[2] / yp[3] - ym[2] / ym[3]);
        Fzz = h * (zp[2] / zp[3] - zm[2] / zm[3]);
    } else {
        Fxx = h * (xp[0] - xm[0]);
        Fyx = h * (xp[1] - xm[1]);
        Fyy = h * (yp[1] - ym[1]);
        Fzx = h * (xp[2] - xm[2]);
        Fzy = h * (yp[2] - ym[2]);
        Fzz = h * (zp[2] - zm[2]);
    }
    H[0][0] = Fxx; H[0][1] = Fyx; H[0][2] = Fzx;
    H[1][0] = Fyx; H[1][1] = Fyy; H[1][2] = Fzy;
    H[2][0] = Fzx; H[2][1] = Fzy; H[2][2] = Fzz;
}

/* OpenCL linear sampling with unnormalised coordinates and clamp-to-edge
 * (OpenCL 1.1 section 8.2): i0 = floor(u - 0.5), a = frac(u - 0.5), weights
 * summed in the order the specification lists them.  Returns x,y,z. */
static void FN(orc_sample_linear)(const REAL *F, int X, int Y, int Z, REAL u, REAL v, REAL w,
                                  REAL out[3]) {
    REAL uu = u - (REAL)0.5, vv = v - (REAL)0.5, ww = w - (REAL)0.5;
    REAL fu = RFLOOR_(uu), fv = RFLOOR_(vv), fw = RFLOOR_(ww);
    REAL a = uu - fu, b = vv - fv, c = ww - fw;
    int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    int i1 = FN(clampi)(i0 + 1, X), j1 = FN(clampi)(j0 + 1, Y), k1 = FN(clampi)(k0 + 1, Z);
    i0 = FN(clampi)(i0, X); j0 = FN(clampi)(j0, Y); k0 = FN(clampi)(k0, Z);
    REAL ia = (REAL)1 - a, ib = (REAL)1 - b, ic = (REAL)1 - c;
    REAL w000 = (ia * ib) * ic, w100 = (a * ib) * ic, w010 = (ia * b) * ic, w110 = (a * b) * ic;
    REAL w001 = (ia * ib) * c, w101 = (a * ib) * c, w011 = (ia * b) * c, w111 = (a * b) * c;
    const REAL *t000 = F + 4 * IDX(i0, j0, k0), *t100 = F + 4 * IDX(i1, j0, k0);
    const REAL *t010 = F + 4 * IDX(i0, j1, k0), *t110 = F + 4 * IDX(i1, j1, k0);
    const REAL *t001 = F + 4 * IDX(i0, j0, k1), *t101 = F + 4 * IDX(i1, j0, k1);
    const REAL *t011 = F + 4 * IDX(i0, j1, k1), *t111 = F + 4 * IDX(i1, j1, k1);
    for (int q = 0; q < 3; q++) {
        REAL s = w000 * t000[q];
        s = s + w100 * t100[q];
        s = s + w010 * t010[q];
        s = s + w110 * t110[q];
        s = s + w001 * t001[q];
        s = s + w101 * t101[q];
        s = s + w011 * t011[q];
        s = s + w111 * t111[q];
        out[q] = s;
    }
}

/* circleFittingTDF, kernels.cl:1071-1157.  Hessian + eigen-decomposition, then
 * for r = rMin, rMin+rStep, ... <= rMax (accumulated in REAL):
 *   S(r) = (1/32) sum_j dot(-V(x + r Va_j), Va_j),  Va_j = cos(j) e3 + sin(j) e2
 * keep the maximum and stop at the first radius that does not increase it.
 * The Hessian is normalised by w when rMax >= 4 (kernels.cl:1083-1091). */
void FN(orc_tdf_circle)(const REAL *F, int X, int Y, int Z, float rMin, float rMax,
                        float rStep, REAL *T, REAL *Rout) {
    FN(orc_tdf_circle_ex)(F, X, Y, Z, rMin, rMax, rStep, 32, 1, 0, T, Rout);
}

/* circleFittingTDF with the library's options: `samples` samples per radius
 * taking entries j * stride of the 32-entry table (the reference's disabled
 * sample-count switch, kernels.cl:1120-1131; 32 / 1 is the reference) and
 * the eigensolver `eigen` (0: tred2 + tql2; 1: the closed form,
 * orc_eig3_closed_f32 -- float instantiation only, the double one keeps
 * tql2). */
void FN(orc_tdf_circle_ex)(const REAL *F, int X, int Y, int Z, float rMin, float rMax,
                           float rStep, int samples, int stride, int eigen, REAL *T, REAL *Rout) {
    float cf32[32], sf32[32], cf[32], sf[32];
    orc_circle_table(cf32, sf32);
    for (int j = 0; j < samples; j++) {
        cf[j] = cf32[j * stride];
        sf[j] = sf32[j * stride];
    }
    (void)eigen;
    const int normalized = !(rMax < 4.0f);
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                REAL H[3][3], A[9], V[9], d[3];
                FN(orc_hessian)(F, X, Y, Z, x, y, z, normalized, H);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) A[3 * i + j] = H[i][j];
#if ORC_IS_F32
                if (eigen) orc_eig3_closed_f32(A, V, d);
                else FN(orc_eig3)(A, V, d);
#else
                FN(orc_eig3)(A, V, d);
#endif
                REAL e2[3] = {V[0 * 3 + 1], V[1 * 3 + 1], V[2 * 3 + 1]};
                REAL e3[3] = {V[0 * 3 + 2], V[1 * 3 + 2], V[2 * 3 + 2]};
                REAL maxSum = 0, maxRadius = 0;
                for (REAL radius = (REAL)rMin; radius <= (REAL)rMax; radius = radius + (REAL)rStep) {
                    REAL rs = 0;
                    for (int j = 0; j < samples; j++) {
                        REAL c = (REAL)cf[j], s = (REAL)sf[j];
                        REAL va0 = c * e3[0] + s * e2[0];
                        REAL va1 = c * e3[1] + s * e2[1];
                        REAL va2 = c * e3[2] + s * e2[2];
                        REAL smp[3];
                        FN(orc_sample_linear)(F, X, Y, Z, (REAL)x + radius * va0,
                                              (REAL)y + radius * va1, (REAL)z + radius * va2, smp);
                        REAL dt = ((-smp[0]) * va0 + (-smp[1]) * va1) + (-smp[2]) * va2;
                        rs = rs + dt;
                    }
                    rs = rs / (REAL)samples;
                    if (rs > maxSum) {
                        maxSum = rs;
                        maxRadius = radius;
                    } else {
                        break;
                    }
                }
                T[IDX(x, y, z)] = maxSum;
                Rout[IDX(x, y, z)] = maxRadius;
            }
}

/* splineTDF, kernels.cl:1159-1254 (kernels_no_3d_write.cl:1574-1671), with
 * the driver's constants (tubeDetectionFilters.cpp:37-48): rMin = max(1, rMin),
 * 12 arms, minAverageMag 0.1.  Normalised Hessian, eigenvectors e1, e2, e3;
 * per arm a line search from rMin for the first border point (magnitude
 * falling after having risen, mean of the last two magnitudes above the
 * voxel's own by more than 0.1); an arm without one, or whose border field
 * points along the arm, makes the voxel invalid (T = 0).  At most 4096 radii
 * per arm (the reference loops forever for a step that does not advance). */
void FN(orc_tdf_spline)(const REAL *F, int X, int Y, int Z, float rMin, float rMax,
                        float rStep, REAL *T, REAL *Rout) {
    float cf[12], sf[12];
    orc_arm_table(cf, sf);
    if (rMin < 1.0f) rMin = 1.0f;
    const REAL minAvg = (REAL)0.1f;
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                REAL H[3][3], A[9], V[9], d[3];
                FN(orc_hessian)(F, X, Y, Z, x, y, z, 1, H);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) A[3 * i + j] = H[i][j];
                FN(orc_eig3)(A, V, d);
                const REAL e1[3] = {V[0 * 3 + 0], V[1 * 3 + 0], V[2 * 3 + 0]};
                const REAL e2[3] = {V[0 * 3 + 1], V[1 * 3 + 1], V[2 * 3 + 1]};
                const REAL e3[3] = {V[0 * 3 + 2], V[1 * 3 + 2], V[2 * 3 + 2]};
                const REAL *c4 = F + 4 * IDX(x, y, z);
                const REAL cur = RSQRT_((c4[0] * c4[0] + c4[1] * c4[1]) + c4[2] * c4[2]);
                REAL maxRadius[12], sum = 0, avgRadius = 0;
                int invalid = 0;
                for (int j = 0; j < 12; j++) {
                    maxRadius[j] = 999;
                    const REAL c = (REAL)cf[j], s = (REAL)sf[j];
                    const REAL va[3] = {c * e3[0] + s * e2[0], c * e3[1] + s * e2[1], c * e3[2] + s * e2[2]};
                    REAL smp[3];
                    FN(orc_sample_linear)(F, X, Y, Z, (REAL)x + (REAL)rMin * va[0], (REAL)y + (REAL)rMin * va[1],
                                          (REAL)z + (REAL)rMin * va[2], smp);
                    REAL prevMagnitude = RSQRT_((smp[0] * smp[0] + smp[1] * smp[1]) + smp[2] * smp[2]);
                    int up = cur > prevMagnitude ? 0 : 1;
                    int nr = 0;
                    for (REAL radius = (REAL)rMin + (REAL)rStep; radius <= (REAL)rMax && nr < 4096;
                         radius = radius + (REAL)rStep, nr++) {
                        REAL vec[3];
                        FN(orc_sample_linear)(F, X, Y, Z, (REAL)x + radius * va[0], (REAL)y + radius * va[1],
                                              (REAL)z + radius * va[2], vec);
                        const REAL magnitude = RSQRT_((vec[0] * vec[0] + vec[1] * vec[1]) + vec[2] * vec[2]);
                        if (up == 1 && magnitude < prevMagnitude &&
                            (prevMagnitude + magnitude) / (REAL)2 - cur > minAvg) {
                            maxRadius[j] = radius;
                            avgRadius = avgRadius + radius;
                            const REAL n[3] = {vec[0] / magnitude, vec[1] / magnitude, vec[2] / magnitude};
                            const REAL la = RSQRT_((va[0] * va[0] + va[1] * va[1]) + va[2] * va[2]);
                            const REAL na[3] = {-(va[0] / la), -(va[1] / la), -(va[2] / la)};
                            if ((n[0] * na[0] + n[1] * na[1]) + n[2] * na[2] < 0) {
                                invalid = 1;
                                sum = 0;
                            }
                            sum = sum + ((REAL)1 - RFABS_((n[0] * e1[0] + n[1] * e1[1]) + n[2] * e1[2]));
                            break;
                        }
                        if (magnitude > prevMagnitude) up = 1;
                        prevMagnitude = magnitude;
                    }
                    if (maxRadius[j] == 999 || invalid == 1) {
                        invalid = 1;
                        break;
                    }
                }
                Rout[IDX(x, y, z)] = avgRadius / (REAL)12;
                if (invalid) {
                    T[IDX(x, y, z)] = 0;
                } else {
                    REAL avgSymmetry = 0;
                    for (int j = 0; j < 6; j++) {
                        const REAL a = maxRadius[j], b = maxRadius[6 + j];
                        avgSymmetry = avgSymmetry + (a < b ? a : b) / (a > b ? a : b);
                    }
                    avgSymmetry = avgSymmetry / (REAL)6;
                    const REAL t = (sum / (REAL)12) * avgSymmetry + (REAL)0.2f;
                    T[IDX(x, y, z)] = t < (REAL)1 ? t : (REAL)1;
                }
            }
}

/* combine, kernels.cl:561-572 */
void FN(orc_combine)(const REAL *Ts, const REAL *Rs, REAL *Tl, REAL *Rl, int64_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++)
        if (Tl[i] < Ts[i]) {
            Tl[i] = Ts[i];
            Rl[i] = Rs[i];
        }
}

/* findCandidateCenterpoints2, kernels.cl:1309-1390, one candidate at a time.
 * maxD = clamp(round(radius), 1, 8).  For every offset r != 0 in the cube with
 * |r| < maxD whose angle to its projection on the plane orthogonal to e1 is
 * below 0.5 rad, the candidate is rejected if |v| (the w channel, clamp-to-edge)
 * at the offset is below |v| at the candidate.  The angle test acos(d) < 0.5 is
 * evaluated as d > cos(0.5) with d <= 1 (acos is NaN above 1; NaN compares
 * false), which avoids a libm-dependent acos. */
void FN(orc_candidates2)(const REAL *radius, const REAL *F, int X, int Y, int Z,
                         const int32_t *pos, int64_t count, int8_t *mask_out) {
#if ORC_IS_F32
    /* smallest float strictly above cos(0.5) */
    float cl = (float)cos(0.5);
    if ((double)cl <= cos(0.5)) cl = nextafterf(cl, 2.0f);
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < count; t++) {
        int x = pos[3 * t], y = pos[3 * t + 1], z = pos[3 * t + 2];
        REAL rad = radius[IDX(x, y, z)];
        REAL rr = RROUND_(rad);
        rr = rr < (REAL)8 ? rr : (REAL)8;
        rr = rr > (REAL)1 ? rr : (REAL)1;
        int maxD = (int)rr;
        REAL H[3][3], A[9], V[9], d[3];
        FN(orc_hessian)(F, X, Y, Z, x, y, z, 1, H);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) A[3 * i + j] = H[i][j];
        FN(orc_eig3)(A, V, d);
        REAL e1[3] = {V[0], V[3], V[6]};
        REAL mag0 = F[4 * IDX(x, y, z) + 3];
        int invalid = 0;
        for (int a = -maxD; a <= maxD; a++)
            for (int b = -maxD; b <= maxD; b++)
                for (int c = -maxD; c <= maxD; c++) {
                    if (a == 0 && b == 0 && c == 0) continue;
                    if (a * a + b * b + c * c >= maxD * maxD) continue;
                    REAL r0 = (REAL)a, r1 = (REAL)b, r2 = (REAL)c;
                    REAL dp = (e1[0] * r0 + e1[1] * r1) + e1[2] * r2;
                    REAL p0 = r0 - e1[0] * dp, p1 = r1 - e1[1] * dp, p2 = r2 - e1[2] * dp;
                    REAL lr = RSQRT_((r0 * r0 + r1 * r1) + r2 * r2);
                    REAL lp = RSQRT_((p0 * p0 + p1 * p1) + p2 * p2);
                    REAL dd = ((r0 / lr) * (p0 / lp) + (r1 / lr) * (p1 / lp)) + (r2 / lr) * (p2 / lp);
#if ORC_IS_F32
                    int close = (dd >= cl) && (dd <= 1.0f);
#else
                    int close = (dd > cos(0.5)) && (dd <= 1.0);
#endif
                    if (!close) continue;
                    REAL mag = F[4 * IDX(FN(clampi)(x + a, X), FN(clampi)(y + b, Y),
                                         FN(clampi)(z + c, Z)) + 3];
                    if (mag < mag0) invalid = 1;
                }
        mask_out[IDX(x, y, z)] = invalid ? 0 : 1;
    }
}

/* dd, kernels.cl:1260-1292: per cube of cubeSize^3 voxels, the candidate with
 * the largest TDF (strict >, starting from 0; loop x outer, y, z inner; reads
 * clamped to the edge). */
void FN(orc_dd)(const REAL *T, const int8_t *cand, int X, int Y, int Z, int cs, int8_t *out) {
    int GX = (X + cs - 1) / cs, GY = (Y + cs - 1) / cs, GZ = (Z + cs - 1) / cs;
#pragma omp parallel for schedule(static)
    for (int gz = 0; gz < GZ; gz++)
        for (int gy = 0; gy < GY; gy++)
            for (int gx = 0; gx < GX; gx++) {
                REAL best = 0;
                int found = 0, bx = 0, by = 0, bz = 0;
                for (int a = 0; a < cs; a++)
                    for (int b = 0; b < cs; b++)
                        for (int c = 0; c < cs; c++) {
                            int x = gx * cs + a, y = gy * cs + b, z = gz * cs + c;
                            int64_t i = IDX(FN(clampi)(x, X), FN(clampi)(y, Y), FN(clampi)(z, Z));
                            if (cand[i] == 1) {
                                REAL g = T[i];
                                if (g > best) {
                                    found = 1;
                                    best = g;
                                    bx = x; by = y; bz = z;
                                }
                            }
                        }
                if (found && bx < X && by < Y && bz < Z) out[IDX(bx, by, bz)] = 1;
            }
}

/* ---------------------------------------------------------------------------
 * Full-multigrid GVF (gradientVectorFlow.cpp:5-441, 631-1005; kernels
 * kernels.cl:1775-2061).  Every image is stored in `storage` after each kernel.
 * Images outside their bounds read 0 where the reference uses the CLAMP
 * sampler (restrict, prolongate, residual) and the edge value where it uses
 * clamp-to-edge (Gauss-Seidel, fmgResidual's field read).
 * ------------------------------------------------------------------------- */
typedef struct { int x, y, z; } FN(orc_dim);

static inline REAL FN(rd0)(const REAL *a, FN(orc_dim) d, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= d.x || y >= d.y || z >= d.z) return 0;
    return a[(int64_t)x + (int64_t)d.x * ((int64_t)y + (int64_t)d.y * z)];
}
static inline REAL FN(rdc)(const REAL *a, FN(orc_dim) d, int x, int y, int z) {
    x = FN(clampi)(x, d.x); y = FN(clampi)(y, d.y); z = FN(clampi)(z, d.z);
    return a[(int64_t)x + (int64_t)d.x * ((int64_t)y + (int64_t)d.y * z)];
}
#define DN(d) ((int64_t)(d).x * (d).y * (d).z)
#define DI(d, i_, j_, k_) ((int64_t)(i_) + (int64_t)(d).x * ((int64_t)(j_) + (int64_t)(d).y * (k_)))

/* calculateNewSize, gradientVectorFlow.cpp:371-395 */
static FN(orc_dim) FN(fmg_new_size)(FN(orc_dim) s) {
    int ok = 0;
    if (s.x == s.y && s.x == s.z) {
        int p = 1;
        while (p < s.x) p *= 2;
        ok = (p == s.x);
    }
    int ns;
    if (!ok) {
        int mx = s.x > s.y ? s.x : s.y;
        if (s.z > mx) mx = s.z;
        int i = 1;
        while ((1 << i) < mx) i++;
        ns = 1 << (i - 1);
    } else {
        ns = s.x / 2;
    }
    FN(orc_dim) r = {ns, ns, ns};
    return r;
}

/* GVFgaussSeidel / GVFgaussSeidel2 half-sweeps; `iterations` full sweeps. */
static void FN(fmg_gs)(REAL *v, const REAL *r, const REAL *sq, FN(orc_dim) d, REAL mu, REAL h,
                       int iterations, int st) {
    if (iterations <= 0) return;
    int64_t n = DN(d);
    REAL *v2 = (REAL *)calloc((size_t)n, sizeof(REAL));
    const REAL two_mu = (REAL)2 * mu, twelve_mu = (REAL)12 * mu, hh = h * h;
    const REAL two_hh = ((REAL)2 * h) * h;
    for (int it = 0; it < 2 * iterations; it++) {
        const int red_pass = (it % 2 == 0);
        const REAL *src = red_pass ? v : v2;
        REAL *dst = red_pass ? v2 : v;
#pragma omp parallel for schedule(static)
        for (int z = 0; z < d.z; z++)
            for (int y = 0; y < d.y; y++)
                for (int x = 0; x < d.x; x++) {
                    int px = FN(mirror)(x, d.x), py = FN(mirror)(y, d.y), pz = FN(mirror)(z, d.z);
                    int red = ((px + py + pz) % 2 == 0);
                    if (red_pass && !red) continue;
                    REAL value;
                    if (!red_pass && red) {
                        value = src[DI(d, px, py, pz)];
                    } else {
                        REAL s = FN(rdc)(src, d, px + 1, py, pz);
                        s = s + FN(rdc)(src, d, px - 1, py, pz);
                        s = s + FN(rdc)(src, d, px, py + 1, pz);
                        s = s + FN(rdc)(src, d, px, py - 1, pz);
                        s = s + FN(rdc)(src, d, px, py, pz + 1);
                        s = s + FN(rdc)(src, d, px, py, pz - 1);
                        REAL num = two_mu * s - two_hh * r[DI(d, px, py, pz)];
                        REAL den = twelve_mu + hh * sq[DI(d, px, py, pz)];
                        value = num / den;
                    }
                    dst[DI(d, x, y, z)] = Q_(value, st);
                }
    }
    free(v2);
}

/* residual, kernels.cl:1973-2006 */
static void FN(fmg_residual)(const REAL *r, const REAL *v, const REAL *sq, FN(orc_dim) d, REAL mu,
                             REAL h, int st, REAL *out) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.z; z++)
        for (int y = 0; y < d.y; y++)
            for (int x = 0; x < d.x; x++) {
                int px = FN(mirror)(x, d.x), py = FN(mirror)(y, d.y), pz = FN(mirror)(z, d.z);
                REAL vc = FN(rd0)(v, d, px, py, pz);
                REAL s = FN(rd0)(v, d, px + 1, py, pz);
                s = s + FN(rd0)(v, d, px - 1, py, pz);
                s = s + FN(rd0)(v, d, px, py + 1, pz);
                s = s + FN(rd0)(v, d, px, py - 1, pz);
                s = s + FN(rd0)(v, d, px, py, pz + 1);
                s = s + FN(rd0)(v, d, px, py, pz - 1);
                s = s - (REAL)6 * vc;
                REAL lap = (mu * s) / (h * h);
                REAL value = FN(rd0)(r, d, px, py, pz) - (lap - FN(rd0)(sq, d, px, py, pz) * vc);
                out[DI(d, x, y, z)] = Q_(value, st);
            }
}

/* restrictVolume, kernels.cl:1923-1951: mean of the 2x2x2 children; `fd` is
 * the fine image's extent (reads outside it are 0), the mirror clamp uses
 * twice the coarse extent. */
static void FN(fmg_restrict)(const REAL *fine, FN(orc_dim) fd, FN(orc_dim) cd, int st, REAL *out) {
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                  {1, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
#pragma omp parallel for schedule(static)
    for (int z = 0; z < cd.z; z++)
        for (int y = 0; y < cd.y; y++)
            for (int x = 0; x < cd.x; x++) {
                int px = 2 * x, py = 2 * y, pz = 2 * z;
                if (px >= 2 * cd.x - 1) px = 2 * cd.x - 3;
                if (py >= 2 * cd.y - 1) py = 2 * cd.y - 3;
                if (pz >= 2 * cd.z - 1) pz = 2 * cd.z - 3;
                REAL s = FN(rd0)(fine, fd, px + off[0][0], py + off[0][1], pz + off[0][2]);
                for (int k = 1; k < 8; k++)
                    s = s + FN(rd0)(fine, fd, px + off[k][0], py + off[k][1], pz + off[k][2]);
                out[DI(cd, x, y, z)] = Q_((REAL)0.125 * s, st);
            }
}

/* prolongate (add == 1, kernels.cl:1953-1961) and prolongate2 (add == 0,
 * kernels.cl:1963-1970): injection from floor(x/2). */
static void FN(fmg_prolong)(const REAL *fine_in, const REAL *coarse, FN(orc_dim) fd, FN(orc_dim) cd,
                            int add, int st, REAL *out) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < fd.z; z++)
        for (int y = 0; y < fd.y; y++)
            for (int x = 0; x < fd.x; x++) {
                REAL c = FN(rd0)(coarse, cd, x / 2, y / 2, z / 2);
                REAL value = add ? fine_in[DI(fd, x, y, z)] + c : c;
                out[DI(fd, x, y, z)] = Q_(value, st);
            }
}

static void FN(fmg_vcycle)(const REAL *r, REAL *v, const REAL *sq, FN(orc_dim) d, int l, int v1,
                           int v2, int lmax, REAL mu, REAL h, int st) {
    FN(fmg_gs)(v, r, sq, d, mu, h, v1, st);
    if (l < lmax) {
        FN(orc_dim) nd = FN(fmg_new_size)(d);
        int64_t n = DN(d), nn = DN(nd);
        REAL *p = (REAL *)malloc(sizeof(REAL) * (size_t)n);
        REAL *r1 = (REAL *)malloc(sizeof(REAL) * (size_t)nn);
        REAL *s1 = (REAL *)malloc(sizeof(REAL) * (size_t)nn);
        REAL *v1p = (REAL *)calloc((size_t)nn, sizeof(REAL));
        FN(fmg_residual)(r, v, sq, d, mu, h, st, p);
        FN(fmg_restrict)(p, d, nd, st, r1);
        FN(fmg_restrict)(sq, d, nd, st, s1);
        FN(fmg_vcycle)(r1, v1p, s1, nd, l + 1, v1, v2, lmax, mu, h * (REAL)2, st);
        FN(fmg_prolong)(v, v1p, d, nd, 1, st, p);
        memcpy(v, p, sizeof(REAL) * (size_t)n);
        free(p); free(r1); free(s1); free(v1p);
    }
    FN(fmg_gs)(v, r, sq, d, mu, h, v2, st);
}

static REAL *FN(fmg_full)(const REAL *r, const REAL *sq, FN(orc_dim) d, int l, int v0, int v1,
                          int v2, int lmax, REAL mu, REAL h, int st) {
    int64_t n = DN(d);
    REAL *v = (REAL *)calloc((size_t)n, sizeof(REAL));
    if (l < lmax) {
        FN(orc_dim) nd = FN(fmg_new_size)(d);
        int64_t nn = DN(nd);
        REAL *r1 = (REAL *)malloc(sizeof(REAL) * (size_t)nn);
        REAL *s1 = (REAL *)malloc(sizeof(REAL) * (size_t)nn);
        FN(fmg_restrict)(r, d, nd, st, r1);
        FN(fmg_restrict)(sq, d, nd, st, s1);
        REAL *vc = FN(fmg_full)(r1, s1, nd, l + 1, v0, v1, v2, lmax, mu, h * (REAL)2, st);
        FN(fmg_prolong)(NULL, vc, d, nd, 0, st, v);
        free(r1); free(s1); free(vc);
    }
    for (int i = 0; i < v0; i++) FN(fmg_vcycle)(r, v, sq, d, l, v1, v2, lmax, mu, h, st);
    return v;
}

/* runFMGGVF, gradientVectorFlow.cpp:729-1005 with v0=1, v1=2, v2=2, l_max=2 and
 * spacing 1; `iterations` FMG cycles per component.  field4 is the vector field
 * (RGBA, as produced by createVectorField); out4 gets (vx, vy, vz, |v|). */
void FN(orc_fmg_gvf)(const REAL *field4, int X, int Y, int Z, float mu_, int iterations, int st,
                     REAL *out4) {
    FN(orc_dim) d = {X, Y, Z};
    const int64_t n = DN(d);
    const REAL mu = (REAL)mu_;
    REAL *sq = (REAL *)malloc(sizeof(REAL) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const REAL *q = field4 + 4 * i;
        sq[i] = Q_((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2], st);   /* createSqrMag */
    }
    REAL *comp[3];
    REAL *rr = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    for (int c = 0; c < 3; c++) {
        REAL *f = (REAL *)calloc((size_t)n, sizeof(REAL));
        for (int it = 0; it < iterations; it++) {
            /* fmgResidual, kernels.cl:2008-2053 */
#pragma omp parallel for schedule(static)
            for (int z = 0; z < Z; z++)
                for (int y = 0; y < Y; y++)
                    for (int x = 0; x < X; x++) {
                        int px = FN(mirror)(x, X), py = FN(mirror)(y, Y), pz = FN(mirror)(z, Z);
                        const REAL *q = field4 + 4 * DI(d, px, py, pz);
                        REAL v0 = q[c];
                        REAL sqm = (q[0] * q[0] + q[1] * q[1]) + q[2] * q[2];
                        REAL fc = FN(rd0)(f, d, px, py, pz);
                        REAL s = FN(rd0)(f, d, px + 1, py, pz);
                        s = s + FN(rd0)(f, d, px - 1, py, pz);
                        s = s + FN(rd0)(f, d, px, py + 1, pz);
                        s = s + FN(rd0)(f, d, px, py - 1, pz);
                        s = s + FN(rd0)(f, d, px, py, pz + 1);
                        s = s + FN(rd0)(f, d, px, py, pz - 1);
                        s = s - (REAL)6 * fc;
                        REAL res = (mu * s) / ((REAL)1 * (REAL)1);
                        REAL value = (-sqm) * v0 - (res - sqm * fc);
                        rr[DI(d, x, y, z)] = Q_(value, st);
                    }
            REAL *f2 = FN(fmg_full)(rr, sq, d, 0, 1, 2, 2, 2, mu, (REAL)1, st);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) f[i] = Q_(f[i] + f2[i], st);   /* addTwoImages */
            free(f2);
        }
        comp[c] = f;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {                                     /* MGGVFFinish */
        REAL x = comp[0][i], y = comp[1][i], z = comp[2][i];
        out4[4 * i + 0] = Q_(x, st);
        out4[4 * i + 1] = Q_(y, st);
        out4[4 * i + 2] = Q_(z, st);
        out4[4 * i + 3] = Q_(RSQRT_((x * x + y * y) + z * z), st);
    }
    for (int c = 0; c < 3; c++) free(comp[c]);
    free(rr);
    free(sq);
}

#undef FN
#undef ORC_CAT
#undef ORC_CAT2
#undef RSQRT_
#undef RFABS_
#undef RFLOOR_
#undef RROUND_
#undef Q_
#undef IDX
#undef DN
#undef DI
