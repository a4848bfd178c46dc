// eigen_closed.cuh -- closed-form eigen-decomposition of a symmetric 3x3
// matrix, held in registers: the alternative to the reference's iterative
// tred2 + tql2 (kernels.cl:1519-1773, eigen3.cuh), for the TDF's eigen mode 1.
//
// Method (no transcendental function, so every step is an IEEE +, -, *, / or
// sqrt and the float oracle can reproduce it bit for bit):
//  1. Eigenvalues by the trigonometric method for symmetric 3x3 matrices
//     (O. K. Smith, "Eigenvalues of a symmetric 3 x 3 matrix", CACM 4(4),
//     1961): m = tr(A) / 3, p = sqrt(|A - m I|_F^2 / 6), B = (A - m I) / p,
//     r = det(B) / 2; the eigenvalues of B are the roots of
//     b^3 - 3 b - 2 r = 0, namely 2 cos((acos r + 2 pi k) / 3).  Instead of
//     acos and cos, the root that is isolated from the other two (the
//     largest when r >= 0, the smallest when r < 0) is found by Newton's
//     method from +-2 (the cubic is convex there, so the iterates decrease
//     monotonically onto the root at a quadratic rate: kEigNewtonF32 / kEigNewtonF64 steps suffice),
//     and the other two come from the remaining quadratic,
//     (-b_iso -+ sqrt(12 - 3 b_iso^2)) / 2.
//  2. Eigenvectors as in D. Eberly, "A Robust Eigensolver for 3 x 3
//     Symmetric Matrices" (Geometric Tools, 2014): the isolated eigenvalue's
//     vector is the longest cross product of two rows of A - lambda I; its
//     orthogonal complement gets an orthonormal basis (U, V); the middle
//     eigenvalue's vector is the null vector of the 2x2 restriction of
//     A - lambda I to (U, V), which stays well defined when the two remaining
//     eigenvalues coincide; the third is the cross product of the first two.
//  3. Near-degenerate branch: when 1 - |r| < kNearDegenerate (a small cubic
//     discriminant, 27 (1 - r^2) in units of p^6: two eigenvalues within a few
//     percent of p), steps 1-2 are redone in FP64 and rounded to float.
//  4. Order and signs: ascending |lambda| (e1 = the smallest, the tube
//     direction, as tql2 sorts: a selection sort with strict <, started from
//     ascending values), each eigenvector with its largest-magnitude
//     component positive.  tql2's signs follow its rotation sequence and have
//     no closed-form rule; the TDF's circle samples (angles j radians) are not
//     symmetric, so TDF values of this mode agree with the tql2 mode to the
//     sampling noise of the circle, not bit for bit.
#pragma once

namespace tsf {

constexpr int kEigNewtonF32 = 5;
constexpr int kEigNewtonF64 = 7;
constexpr float kNearDegenerate = 1e-3f;

template <class R> __host__ __device__ __forceinline__ R eigc_sqrt(R x);
template <> __host__ __device__ __forceinline__ float eigc_sqrt<float>(float x) { return sqrtf(x); }
template <> __host__ __device__ __forceinline__ double eigc_sqrt<double>(double x) { return sqrt(x); }

template <class R> __host__ __device__ __forceinline__ R eigc_abs(R x) { return x < (R)0 ? -x : x; }

// Largest root of b^3 - 3 b - 2 r for r >= 0 (in [sqrt 3, 2]): Newton from 2.
template <class R, int NIT> __host__ __device__ __forceinline__ R eigc_top_root(R r) {
    R b = (R)2;
#pragma unroll
    for (int i = 0; i < NIT; i++) {
        const R b2 = b * b;
        const R g = (b2 - (R)3) * b - (R)2 * r;
        const R gp = (R)3 * b2 - (R)3;
        b = b - g / gp;
    }
    return b;
}

// a: (a00, a11, a22, a01, a02, a12).  lam[3] ascending by value, vec[k][3]
// the unit eigenvector of lam[k], *r_out = det(B) / 2.  Returns false when
// p == 0 (a multiple of the identity; lam = m, vec = the identity, r = 0).
template <class R, int NIT>
__host__ __device__ __forceinline__ bool eigc_core(const R a[6], R lam[3], R vec[3][3], R *r_out) {
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
        return false;
    }
    const R p = eigc_sqrt<R>(p2);
    const R c00 = b00 / p, c11 = b11 / p, c22 = b22 / p, c01 = a[3] / p, c02 = a[4] / p, c12 = a[5] / p;
    // det(B) / 2, clamped to [-1, 1]
    const R det = (c00 * (c11 * c22 - c12 * c12) - c01 * (c01 * c22 - c12 * c02)) + c02 * (c01 * c12 - c11 * c02);
    R r = det / (R)2;
    r = r > (R)1 ? (R)1 : (r < (R)-1 ? (R)-1 : r);
    *r_out = r;
    // the isolated root (largest for r >= 0, smallest for r < 0) and the pair
    const bool top = r >= (R)0;
    const R biso = top ? eigc_top_root<R, NIT>(r) : -eigc_top_root<R, NIT>(-r);
    R disc = (R)12 - (R)3 * (biso * biso);
    disc = disc > (R)0 ? disc : (R)0;
    const R sq = eigc_sqrt<R>(disc);
    const R blo = (-biso - sq) / (R)2, bhi = (-biso + sq) / (R)2;
    // eigenvalues ascending; iso = index of the isolated one (2 or 0)
    const R l_iso = m + p * biso, l_mid = m + p * (top ? bhi : blo), l_far = m + p * (top ? blo : bhi);
    lam[0] = top ? l_far : l_iso;
    lam[1] = l_mid;
    lam[2] = top ? l_iso : l_far;

    // eigenvector of the isolated eigenvalue: the longest cross product of
    // two rows of A - l_iso I
    const R r0[3] = {a[0] - l_iso, a[3], a[4]}, r1[3] = {a[3], a[1] - l_iso, a[5]}, r2[3] = {a[4], a[5], a[2] - l_iso};
    const R x01[3] = {r0[1] * r1[2] - r0[2] * r1[1], r0[2] * r1[0] - r0[0] * r1[2], r0[0] * r1[1] - r0[1] * r1[0]};
    const R x02[3] = {r0[1] * r2[2] - r0[2] * r2[1], r0[2] * r2[0] - r0[0] * r2[2], r0[0] * r2[1] - r0[1] * r2[0]};
    const R x12[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2], r1[0] * r2[1] - r1[1] * r2[0]};
    const R n01 = (x01[0] * x01[0] + x01[1] * x01[1]) + x01[2] * x01[2];
    const R n02 = (x02[0] * x02[0] + x02[1] * x02[1]) + x02[2] * x02[2];
    const R n12 = (x12[0] * x12[0] + x12[1] * x12[1]) + x12[2] * x12[2];
    R xb0 = x01[0], xb1 = x01[1], xb2 = x01[2], nb = n01;
    if (n02 > nb) { xb0 = x02[0]; xb1 = x02[1]; xb2 = x02[2]; nb = n02; }
    if (n12 > nb) { xb0 = x12[0]; xb1 = x12[1]; xb2 = x12[2]; nb = n12; }
    R e[3];
    if (nb > (R)0) {
        const R inv = eigc_sqrt<R>(nb);
        e[0] = xb0 / inv; e[1] = xb1 / inv; e[2] = xb2 / inv;
    } else {
        e[0] = (R)1; e[1] = (R)0; e[2] = (R)0;
    }
    // orthonormal basis (U, V) of the complement of e
    R U[3];
    if (eigc_abs<R>(e[0]) > eigc_abs<R>(e[1])) {
        const R l = eigc_sqrt<R>(e[0] * e[0] + e[2] * e[2]);
        U[0] = -e[2] / l; U[1] = (R)0; U[2] = e[0] / l;
    } else {
        const R l = eigc_sqrt<R>(e[1] * e[1] + e[2] * e[2]);
        U[0] = (R)0; U[1] = e[2] / l; U[2] = -e[1] / l;
    }
    const R V[3] = {e[1] * U[2] - e[2] * U[1], e[2] * U[0] - e[0] * U[2], e[0] * U[1] - e[1] * U[0]};
    // 2x2 restriction of A - l_mid I to (U, V)
    const R AU[3] = {(a[0] * U[0] + a[3] * U[1]) + a[4] * U[2], (a[3] * U[0] + a[1] * U[1]) + a[5] * U[2],
                     (a[4] * U[0] + a[5] * U[1]) + a[2] * U[2]};
    const R AV[3] = {(a[0] * V[0] + a[3] * V[1]) + a[4] * V[2], (a[3] * V[0] + a[1] * V[1]) + a[5] * V[2],
                     (a[4] * V[0] + a[5] * V[1]) + a[2] * V[2]};
    const R m00 = ((U[0] * AU[0] + U[1] * AU[1]) + U[2] * AU[2]) - l_mid;
    const R m01 = (U[0] * AV[0] + U[1] * AV[1]) + U[2] * AV[2];
    const R m11 = ((V[0] * AV[0] + V[1] * AV[1]) + V[2] * AV[2]) - l_mid;
    R w0, w1;
    if (eigc_abs<R>(m00) >= eigc_abs<R>(m11)) {      // null vector of the row (m00, m01)
        w0 = -m01; w1 = m00;
    } else {                                          // of the row (m01, m11)
        w0 = m11; w1 = -m01;
    }
    R wl = w0 * w0 + w1 * w1;
    if (wl > (R)0) {
        wl = eigc_sqrt<R>(wl);
        w0 = w0 / wl; w1 = w1 / wl;
    } else {
        w0 = (R)1; w1 = (R)0;
    }
    R g[3] = {w0 * U[0] + w1 * V[0], w0 * U[1] + w1 * V[1], w0 * U[2] + w1 * V[2]};
    const R gl = eigc_sqrt<R>((g[0] * g[0] + g[1] * g[1]) + g[2] * g[2]);
    g[0] = g[0] / gl; g[1] = g[1] / gl; g[2] = g[2] / gl;
    const R h[3] = {e[1] * g[2] - e[2] * g[1], e[2] * g[0] - e[0] * g[2], e[0] * g[1] - e[1] * g[0]};
    for (int i = 0; i < 3; i++) {
        vec[0][i] = top ? h[i] : e[i];
        vec[1][i] = g[i];
        vec[2][i] = top ? e[i] : h[i];
    }
    return true;
}

// H row-major symmetric (the lower triangle is used as the reference builds
// it, kernels.cl:1094-1098).  V[i][k]: component i of eigenvector k (columns,
// like eig3); d ascending by |lambda|.
__host__ __device__ __forceinline__ void eig3_closed(const float H[3][3], float V[3][3], float d[3]) {
    const float a[6] = {H[0][0], H[1][1], H[2][2], H[1][0], H[2][0], H[2][1]};
    float lam[3], vec[3][3], r = 0.0f;
    // near-degenerate branch: redo in FP64 when the cubic's discriminant is
    // small (1 - |r| < kNearDegenerate)
    if (eigc_core<float, kEigNewtonF32>(a, lam, vec, &r) && 1.0f - eigc_abs<float>(r) < kNearDegenerate) {
        const double ad[6] = {(double)a[0], (double)a[1], (double)a[2], (double)a[3], (double)a[4], (double)a[5]};
        double ld[3], vd[3][3], rd;
        eigc_core<double, kEigNewtonF64>(ad, ld, vd, &rd);
        for (int k = 0; k < 3; k++) {
            lam[k] = (float)ld[k];
            for (int i = 0; i < 3; i++) vec[k][i] = (float)vd[k][i];
        }
    }
    // ascending |lambda| from ascending values: the reference's selection
    // sort with strict < (kernels.cl:1742-1761), as compare-and-swap steps on
    // registers -- step 0 moves the first smallest |lambda| to slot 0, step 1
    // orders slots 1 and 2
    float d0 = lam[0], d1 = lam[1], d2 = lam[2];
    float v0[3] = {vec[0][0], vec[0][1], vec[0][2]}, v1[3] = {vec[1][0], vec[1][1], vec[1][2]},
          v2[3] = {vec[2][0], vec[2][1], vec[2][2]};
    auto swapv = [](float &x, float &y, float a[3], float b[3]) {
        float t = x; x = y; y = t;
        for (int i = 0; i < 3; i++) { t = a[i]; a[i] = b[i]; b[i] = t; }
    };
    const bool k1 = eigc_abs<float>(d1) < eigc_abs<float>(d0);
    const bool k2 = eigc_abs<float>(d2) < eigc_abs<float>(k1 ? d1 : d0);
    if (k2) swapv(d0, d2, v0, v2);
    else if (k1) swapv(d0, d1, v0, v1);
    if (eigc_abs<float>(d2) < eigc_abs<float>(d1)) swapv(d1, d2, v1, v2);
    // signs: the largest-magnitude component positive (the first of equals)
    auto put = [&](int k, const float e[3], float dk) {
        float big = e[0];
        if (eigc_abs<float>(e[1]) > eigc_abs<float>(big)) big = e[1];
        if (eigc_abs<float>(e[2]) > eigc_abs<float>(big)) big = e[2];
        const float sgn = big < 0.0f ? -1.0f : 1.0f;
        V[0][k] = sgn * e[0];
        V[1][k] = sgn * e[1];
        V[2][k] = sgn * e[2];
        d[k] = dk;
    };
    put(0, v0, d0);
    put(1, v1, d1);
    put(2, v2, d2);
}

}  // namespace tsf
