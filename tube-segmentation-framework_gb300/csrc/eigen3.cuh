// eigen3.cuh -- 3x3 symmetric eigen-decomposition held entirely in registers.
//
// Householder tridiagonalisation followed by the implicit QL method: the
// EISPACK tred2 / tql2 procedures (Bowdler, Martin, Reinsch, Wilkinson,
// Handbook for Automatic Computation vol. II) that the reference runs per
// voxel (kernels.cl:1519-1773).  The steps and their operation order are kept
// so that the eigenvector signs -- which decide where the TDF samples its
// circle -- are the reference's.  What differs is the shape of the code: all
// loops are unrolled over the fixed size 3 and every data-dependent index
// (the QL split point m, the sort's arg-min k) is turned into predicated
// selects, so no array ever spills to local memory.  The QL sweep is capped
// at 64 iterations (the reference's loop is unbounded); `converged` reports
// whether the cap was hit.  Tolerance 2^-52 in every precision
// (kernels.cl:1660).  Output: eigenvalues d sorted by ascending |d|,
// eigenvectors in the columns of V.
#pragma once

namespace tsf {

template <typename R> __device__ __forceinline__ R rabs(R v) { return v < R(0) ? -v : v; }
__device__ __forceinline__ float rsqrt_exact(float v) { return sqrtf(v); }
__device__ __forceinline__ double rsqrt_exact(double v) { return sqrt(v); }

template <typename R>
__device__ __forceinline__ void tred2_3(R V[3][3], R d[3], R e[3]) {
    constexpr int n = 3;
#pragma unroll
    for (int j = 0; j < n; j++) d[j] = V[n - 1][j];
#pragma unroll
    for (int i = n - 1; i > 0; i--) {
        R scale = R(0), h = R(0);
#pragma unroll
        for (int k = 0; k < i; k++) scale = scale + rabs(d[k]);
        if (scale == R(0)) {
            e[i] = d[i - 1];
#pragma unroll
            for (int j = 0; j < i; j++) {
                d[j] = V[i - 1][j];
                V[i][j] = R(0);
                V[j][i] = R(0);
            }
        } else {
#pragma unroll
            for (int k = 0; k < i; k++) {
                d[k] = d[k] / scale;
                h = h + d[k] * d[k];
            }
            R f = d[i - 1];
            R g = rsqrt_exact(h);
            if (f > R(0)) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
#pragma unroll
            for (int j = 0; j < i; j++) e[j] = R(0);
#pragma unroll
            for (int j = 0; j < i; j++) {
                f = d[j];
                V[j][i] = f;
                g = e[j] + V[j][j] * f;
#pragma unroll
                for (int k = j + 1; k <= i - 1; k++) {
                    g = g + V[k][j] * d[k];
                    e[k] = e[k] + V[k][j] * f;
                }
                e[j] = g;
            }
            f = R(0);
#pragma unroll
            for (int j = 0; j < i; j++) {
                e[j] = e[j] / h;
                f = f + e[j] * d[j];
            }
            R hh = f / (h + h);
#pragma unroll
            for (int j = 0; j < i; j++) e[j] = e[j] - hh * d[j];
#pragma unroll
            for (int j = 0; j < i; j++) {
                f = d[j];
                g = e[j];
#pragma unroll
                for (int k = j; k <= i - 1; k++) V[k][j] = V[k][j] - (f * e[k] + g * d[k]);
                d[j] = V[i - 1][j];
                V[i][j] = R(0);
            }
        }
        d[i] = h;
    }
#pragma unroll
    for (int i = 0; i < n - 1; i++) {
        V[n - 1][i] = V[i][i];
        V[i][i] = R(1);
        R h = d[i + 1];
        if (h != R(0)) {
#pragma unroll
            for (int k = 0; k <= i; k++) d[k] = V[k][i + 1] / h;
#pragma unroll
            for (int j = 0; j <= i; j++) {
                R g = R(0);
#pragma unroll
                for (int k = 0; k <= i; k++) g = g + V[k][i + 1] * V[k][j];
#pragma unroll
                for (int k = 0; k <= i; k++) V[k][j] = V[k][j] - g * d[k];
            }
        }
#pragma unroll
        for (int k = 0; k <= i; k++) V[k][i + 1] = R(0);
    }
#pragma unroll
    for (int j = 0; j < n; j++) {
        d[j] = V[n - 1][j];
        V[n - 1][j] = R(0);
    }
    V[n - 1][n - 1] = R(1);
    e[0] = R(0);
}

template <typename R> __device__ __forceinline__ R hyp2(R a, R b) { return rsqrt_exact(a * a + b * b); }

template <typename R>
__device__ __forceinline__ bool tql2_3(R V[3][3], R d[3], R e[3]) {
    constexpr int n = 3;
    bool converged = true;
#pragma unroll
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = R(0);
    R f = R(0), tst1 = R(0);
    const R eps = R(2.220446049250313080847263336181640625e-16);
#pragma unroll
    for (int l = 0; l < n; l++) {
        const R t = rabs(d[l]) + rabs(e[l]);
        tst1 = tst1 > t ? tst1 : t;
        // first m >= l with |e[m]| <= eps*tst1 (e[n-1] == 0 bounds it at n-1)
        int m = n - 1;
#pragma unroll
        for (int mm = n - 2; mm >= l; mm--)
            if (rabs(e[mm]) <= eps * tst1) m = mm;
        if (l < n - 1 && m > l) {
            int iter = 0;
            do {
                iter++;
                R g = d[l];
                R p = (d[l + 1] - g) / (R(2) * e[l]);
                R r = hyp2(p, R(1));
                if (p < R(0)) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const R dl1 = d[l + 1];
                R h = g - d[l];
#pragma unroll
                for (int i = l + 2; i < n; i++) d[i] = d[i] - h;
                f = f + h;
                // p = d[m]
                p = d[l];
#pragma unroll
                for (int mm = l + 1; mm < n; mm++)
                    if (m == mm) p = d[mm];
                R c = R(1), c2 = R(1), c3 = R(1);
                const R el1 = e[l + 1];
                R s = R(0), s2 = R(0);
#pragma unroll
                for (int i = n - 2; i >= l; i--) {
                    if (i <= m - 1) {
                        c3 = c2;
                        c2 = c;
                        s2 = s;
                        g = c * e[i];
                        h = c * p;
                        r = hyp2(p, e[i]);
                        e[i + 1] = s * r;
                        s = e[i] / r;
                        c = p / r;
                        p = c * d[i] - s * g;
                        d[i + 1] = h + s * (c * g + s * d[i]);
#pragma unroll
                        for (int k = 0; k < n; k++) {
                            h = V[k][i + 1];
                            V[k][i + 1] = s * V[k][i] + c * h;
                            V[k][i] = c * V[k][i] - s * h;
                        }
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (rabs(e[l]) > eps * tst1 && iter < 64);
            if (rabs(e[l]) > eps * tst1) converged = false;
        }
        d[l] = d[l] + f;
        e[l] = R(0);
    }
    // sort by ascending |d| (selection, first minimum wins)
#pragma unroll
    for (int i = 0; i < n - 1; i++) {
        int k = i;
        R p = d[i];
#pragma unroll
        for (int j = i + 1; j < n; j++)
            if (rabs(d[j]) < rabs(p)) {
                k = j;
                p = d[j];
            }
#pragma unroll
        for (int kk = i + 1; kk < n; kk++) {
            if (k == kk) {
                d[kk] = d[i];
                d[i] = p;
#pragma unroll
                for (int j = 0; j < n; j++) {
                    const R q = V[j][i];
                    V[j][i] = V[j][kk];
                    V[j][kk] = q;
                }
            }
        }
    }
    return converged;
}

template <typename R>
__device__ __forceinline__ bool eig3(const R A[3][3], R V[3][3], R d[3]) {
    R e[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) V[i][j] = A[i][j];
    tred2_3(V, d, e);
    return tql2_3(V, d, e);
}

}  // namespace tsf
