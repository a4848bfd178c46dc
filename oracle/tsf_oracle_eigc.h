/*
 * tsf_oracle_eigc.h -- TEST INFRASTRUCTURE ONLY: the oracle's restatement of
 * the closed-form 3x3 symmetric eigensolver of the TDF's eigen mode 1 (the
 * library's alternative to the reference's tred2 + tql2, kernels.cl:1519-1773,
 * which has no closed form).  Included twice by tsf_oracle.c with
 * EIGC_R = float / double and EIGC_SFX = _f / _d.
 *
 * Method: the trigonometric method for symmetric 3x3 matrices (O. K. Smith,
 * CACM 4(4), 1961) with the isolated root of b^3 - 3b - 2r = 0 found by a fixed
 * number of Newton steps from +-2 and the other two from the remaining
 * quadratic; eigenvectors as in D. Eberly, "A Robust Eigensolver for 3 x 3
 * Symmetric Matrices" (2014): the isolated eigenvalue's vector from the
 * longest cross product of two rows of A - lambda I, the middle one from the
 * 2x2 restriction to the orthogonal complement, the third as a cross product.
 * Only +, -, *, / and sqrt, in a fixed order, so the float result is the
 * CUDA kernel's bit for bit (both without contraction into fused
 * multiply-adds).
 */

#define EIGC_CAT2(a, b) a##b
#define EIGC_CAT(a, b) EIGC_CAT2(a, b)
#define EIGC_FN(name) EIGC_CAT(name, EIGC_SFX)

static EIGC_R EIGC_FN(eigc_abs)(EIGC_R x) { return x < (EIGC_R)0 ? -x : x; }

static EIGC_R EIGC_FN(eigc_top_root)(EIGC_R r, int nit) {
    EIGC_R b = (EIGC_R)2;
    for (int i = 0; i < nit; i++) {
        const EIGC_R b2 = b * b;
        const EIGC_R g = (b2 - (EIGC_R)3) * b - (EIGC_R)2 * r;
        const EIGC_R gp = (EIGC_R)3 * b2 - (EIGC_R)3;
        b = b - g / gp;
    }
    return b;
}

/* a = (a00, a11, a22, a01, a02, a12); lam ascending by value, vec[k] its unit
 * eigenvector, *r_out = det((A - m I) / p) / 2.  Returns 0 when p == 0. */
static int EIGC_FN(eigc_core)(const EIGC_R a[6], EIGC_R lam[3], EIGC_R vec[3][3], EIGC_R *r_out, int nit) {
    typedef EIGC_R R;
    const R m = ((a[0] + a[1]) + a[2]) / (R)3;
    const R b00 = a[0] - m, b11 = a[1] - m, b22 = a[2] - m;
    const R off = (a[3] * a[3] + a[4] * a[4]) + a[5] * a[5];
    const R p2 = (((b00 * b00 + b11 * b11) + b22 * b22) + (R)2 * off) / (R)6;
    if (!(p2 > (R)0)) {
        for (int k = 0; k < 3; k++) {
            lam[k] = m;
            for (int i = 0; i < 3; i++) vec[k][i] = i == k ? (R)1 : (R)0;
        }
        *r_out = (R)0;
        return 0;
    }
    const R p = EIGC_SQRT(p2);
    const R c00 = b00 / p, c11 = b11 / p, c22 = b22 / p, c01 = a[3] / p, c02 = a[4] / p, c12 = a[5] / p;
    const R det = (c00 * (c11 * c22 - c12 * c12) - c01 * (c01 * c22 - c12 * c02)) + c02 * (c01 * c12 - c11 * c02);
    R r = det / (R)2;
    if (r > (R)1) r = (R)1;
    else if (r < (R)-1) r = (R)-1;
    *r_out = r;
    const int top = r >= (R)0;
    const R biso = top ? EIGC_FN(eigc_top_root)(r, nit) : -EIGC_FN(eigc_top_root)(-r, nit);
    R disc = (R)12 - (R)3 * (biso * biso);
    if (!(disc > (R)0)) disc = (R)0;
    const R sq = EIGC_SQRT(disc);
    const R blo = (-biso - sq) / (R)2, bhi = (-biso + sq) / (R)2;
    const R l_iso = m + p * biso, l_mid = m + p * (top ? bhi : blo), l_far = m + p * (top ? blo : bhi);
    lam[0] = top ? l_far : l_iso;
    lam[1] = l_mid;
    lam[2] = top ? l_iso : l_far;
    /* rows of A - l_iso I and their pairwise cross products */
    const R r0[3] = {a[0] - l_iso, a[3], a[4]}, r1[3] = {a[3], a[1] - l_iso, a[5]};
    const R r2[3] = {a[4], a[5], a[2] - l_iso};
    R x[3][3];
    x[0][0] = r0[1] * r1[2] - r0[2] * r1[1]; x[0][1] = r0[2] * r1[0] - r0[0] * r1[2]; x[0][2] = r0[0] * r1[1] - r0[1] * r1[0];
    x[1][0] = r0[1] * r2[2] - r0[2] * r2[1]; x[1][1] = r0[2] * r2[0] - r0[0] * r2[2]; x[1][2] = r0[0] * r2[1] - r0[1] * r2[0];
    x[2][0] = r1[1] * r2[2] - r1[2] * r2[1]; x[2][1] = r1[2] * r2[0] - r1[0] * r2[2]; x[2][2] = r1[0] * r2[1] - r1[1] * r2[0];
    int kb = 0;
    R nb = (x[0][0] * x[0][0] + x[0][1] * x[0][1]) + x[0][2] * x[0][2];
    for (int k = 1; k < 3; k++) {
        const R nk = (x[k][0] * x[k][0] + x[k][1] * x[k][1]) + x[k][2] * x[k][2];
        if (nk > nb) { kb = k; nb = nk; }
    }
    R e[3];
    if (nb > (R)0) {
        const R l = EIGC_SQRT(nb);
        for (int i = 0; i < 3; i++) e[i] = x[kb][i] / l;
    } else {
        e[0] = (R)1; e[1] = (R)0; e[2] = (R)0;
    }
    /* orthonormal basis (U, V) of the complement of e */
    R U[3];
    if (EIGC_FN(eigc_abs)(e[0]) > EIGC_FN(eigc_abs)(e[1])) {
        const R l = EIGC_SQRT(e[0] * e[0] + e[2] * e[2]);
        U[0] = -e[2] / l; U[1] = (R)0; U[2] = e[0] / l;
    } else {
        const R l = EIGC_SQRT(e[1] * e[1] + e[2] * e[2]);
        U[0] = (R)0; U[1] = e[2] / l; U[2] = -e[1] / l;
    }
    const R V[3] = {e[1] * U[2] - e[2] * U[1], e[2] * U[0] - e[0] * U[2], e[0] * U[1] - e[1] * U[0]};
    const R AU[3] = {(a[0] * U[0] + a[3] * U[1]) + a[4] * U[2], (a[3] * U[0] + a[1] * U[1]) + a[5] * U[2],
                     (a[4] * U[0] + a[5] * U[1]) + a[2] * U[2]};
    const R AV[3] = {(a[0] * V[0] + a[3] * V[1]) + a[4] * V[2], (a[3] * V[0] + a[1] * V[1]) + a[5] * V[2],
                     (a[4] * V[0] + a[5] * V[1]) + a[2] * V[2]};
    const R m00 = ((U[0] * AU[0] + U[1] * AU[1]) + U[2] * AU[2]) - l_mid;
    const R m01 = (U[0] * AV[0] + U[1] * AV[1]) + U[2] * AV[2];
    const R m11 = ((V[0] * AV[0] + V[1] * AV[1]) + V[2] * AV[2]) - l_mid;
    R w0, w1;
    if (EIGC_FN(eigc_abs)(m00) >= EIGC_FN(eigc_abs)(m11)) { w0 = -m01; w1 = m00; }
    else { w0 = m11; w1 = -m01; }
    R wl = w0 * w0 + w1 * w1;
    if (wl > (R)0) {
        wl = EIGC_SQRT(wl);
        w0 = w0 / wl; w1 = w1 / wl;
    } else {
        w0 = (R)1; w1 = (R)0;
    }
    R g[3] = {w0 * U[0] + w1 * V[0], w0 * U[1] + w1 * V[1], w0 * U[2] + w1 * V[2]};
    const R gl = EIGC_SQRT((g[0] * g[0] + g[1] * g[1]) + g[2] * g[2]);
    g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl;
    const R h[3] = {e[1] * g[2] - e[2] * g[1], e[2] * g[0] - e[0] * g[2], e[0] * g[1] - e[1] * g[0]};
    for (int i = 0; i < 3; i++) {
        vec[0][i] = top ? h[i] : e[i];
        vec[1][i] = g[i];
        vec[2][i] = top ? e[i] : h[i];
    }
    return 1;
}

#undef EIGC_FN
#undef EIGC_CAT
#undef EIGC_CAT2
