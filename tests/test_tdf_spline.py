"""Spline TDF oracle (no GPU): splineTDF (kernels.cl:1159-1254) with the
constants of runSplineTDF (tubeDetectionFilters.cpp:37-48).

The C restatement is checked against a pure-Python restatement of the kernel
text (float32 op by op; the eigen-decomposition is the oracle's, itself pinned
against numpy) on sampled voxels, on a bright straight tube whose axis and
radius it must find, and against its own FP64 twin."""
import math

import numpy as np
import pytest

f32 = np.float32


def _sample(F, u, v, w):
    """OpenCL linear sampler, unnormalised coordinates, clamp to edge; x,y,z."""
    Z, Y, X = F.shape[:3]
    uu, vv, ww = f32(u) - f32(0.5), f32(v) - f32(0.5), f32(w) - f32(0.5)
    fu, fv, fw = np.floor(uu), np.floor(vv), np.floor(ww)
    a, b, c = f32(uu - fu), f32(vv - fv), f32(ww - fw)
    cl = lambda i, n: min(max(i, 0), n - 1)
    i0, j0, k0 = int(fu), int(fv), int(fw)
    i1, j1, k1 = cl(i0 + 1, X), cl(j0 + 1, Y), cl(k0 + 1, Z)
    i0, j0, k0 = cl(i0, X), cl(j0, Y), cl(k0, Z)
    ia, ib, ic = f32(1) - a, f32(1) - b, f32(1) - c
    ws = [(ia * ib) * ic, (a * ib) * ic, (ia * b) * ic, (a * b) * ic,
          (ia * ib) * c, (a * ib) * c, (ia * b) * c, (a * b) * c]
    cs = [(i0, j0, k0), (i1, j0, k0), (i0, j1, k0), (i1, j1, k0),
          (i0, j0, k1), (i1, j0, k1), (i0, j1, k1), (i1, j1, k1)]
    out = []
    for q in range(3):
        s = ws[0] * F[cs[0][2], cs[0][1], cs[0][0], q]
        for wgt, (i, j, k) in zip(ws[1:], cs[1:]):
            s = s + wgt * F[k, j, i, q]
        out.append(f32(s))
    return out


def _py_spline_voxel(oracle, F, x, y, z, rmin, rmax, rstep):
    Z, Y, X = F.shape[:3]
    cl = lambda i, n: min(max(i, 0), n - 1)
    g = lambda i, j, k: F[cl(k, Z), cl(j, Y), cl(i, X)]
    h = f32(0.5)
    xp, xm, yp, ym, zp, zm = g(x + 1, y, z), g(x - 1, y, z), g(x, y + 1, z), g(x, y - 1, z), g(x, y, z + 1), g(x, y, z - 1)
    Fxx = h * (xp[0] / xp[3] - xm[0] / xm[3])
    Fyx = h * (xp[1] / xp[3] - xm[1] / xm[3])
    Fyy = h * (yp[1] / yp[3] - ym[1] / ym[3])
    Fzx = h * (xp[2] / xp[3] - xm[2] / xm[3])
    Fzy = h * (yp[2] / yp[3] - ym[2] / ym[3])
    Fzz = h * (zp[2] / zp[3] - zm[2] / zm[3])
    H = np.array([[Fxx, Fyx, Fzx], [Fyx, Fyy, Fzy], [Fzx, Fzy, Fzz]], f32)
    _, V = oracle.eig3(H)
    e1, e2, e3 = V[:, 0], V[:, 1], V[:, 2]
    length = lambda p: np.sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2], dtype=f32)
    cur = length(F[z, y, x])
    rmin = max(f32(1.0), f32(rmin))
    two_pi = f32(2.0) * f32(math.pi)
    mr, s_, avg, invalid = [f32(999)] * 12, f32(0), f32(0), False
    for j in range(12):
        alpha = f32(two_pi * f32(j)) / f32(12)
        c, s = f32(math.cos(float(alpha))), f32(math.sin(float(alpha)))
        va = [c * e3[q] + s * e2[q] for q in range(3)]
        prev = length(_sample(F, f32(x) + rmin * va[0], f32(y) + rmin * va[1], f32(z) + rmin * va[2]))
        up = not (cur > prev)
        radius, nr = f32(rmin + f32(rstep)), 0
        while radius <= f32(rmax) and nr < 4096:
            v = _sample(F, f32(x) + radius * va[0], f32(y) + radius * va[1], f32(z) + radius * va[2])
            mag = length(v)
            if up and mag < prev and (prev + mag) / f32(2) - cur > f32(0.1):
                mr[j] = radius
                avg = avg + radius
                n = [v[q] / mag for q in range(3)]
                la = length(va)
                na = [-(va[q] / la) for q in range(3)]
                if (n[0] * na[0] + n[1] * na[1]) + n[2] * na[2] < 0:
                    invalid, s_ = True, f32(0)
                s_ = s_ + (f32(1) - abs((n[0] * e1[0] + n[1] * e1[1]) + n[2] * e1[2]))
                break
            if mag > prev:
                up = True
            prev = mag
            radius, nr = f32(radius + f32(rstep)), nr + 1
        if mr[j] == 999 or invalid:
            invalid = True
            break
    R = avg / f32(12)
    if invalid:
        return f32(0), R
    sym = f32(0)
    for j in range(6):
        sym = sym + min(mr[j], mr[6 + j]) / max(mr[j], mr[6 + j])
    sym = sym / f32(6)
    return min(f32(1), (s_ / f32(12)) * sym + f32(0.2)), R


def _tube_field(oracle, radius=5.0, shape=(24, 40, 40)):
    Z, Y, X = shape
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    d = np.sqrt((xx - 19.5) ** 2 + (yy - 20.0) ** 2)
    vol = (d <= radius).astype(np.float32)
    f4 = oracle.vector_field(oracle.blur(vol, 1.0), 0.2, 1, "f32")
    return oracle.gvf_finish(oracle.gvf(f4, 0.1, 80, "f32"), "f32"), d


@pytest.fixture(scope="module")
def tube(oracle):
    return _tube_field(oracle)


def test_spline_matches_python_restatement(oracle, tube):
    F, d = tube
    T, R = oracle.tdf_spline(F, 1.5, 15.0, 0.5)
    rng = np.random.default_rng(0)
    Z, Y, X = T.shape
    picks = [(19, 20, 12), (20, 20, 12), (17, 22, 5), (0, 0, 0), (39, 39, 23)]
    picks += [tuple(int(v) for v in (rng.integers(X), rng.integers(Y), rng.integers(Z))) for _ in range(12)]
    for x, y, z in picks:
        t, r = _py_spline_voxel(oracle, F, x, y, z, 1.5, 15.0, 0.5)
        assert T[z, y, x] == t and R[z, y, x] == r, (x, y, z)


def test_spline_finds_the_tube(oracle, tube):
    """Radius-5 tube: the axis responds near 1 with radius about 5; far from
    the tube no arm finds a border (T = 0)."""
    F, d = tube
    T, R = oracle.tdf_spline(F, 1.5, 15.0, 0.5)
    axis = d[12] < 1.0
    assert T[12][axis].min() > 0.9
    assert 4.5 < R[12][axis].mean() < 6.0
    assert T[:, d[0] > 14].max() == 0.0


def test_spline_f32_against_f64(oracle, synth):
    vol = oracle.blur(synth.vascular_tree((48, 48, 48), seed=3), 1.0)
    F = oracle.gvf_finish(oracle.gvf(oracle.vector_field(vol, 0.2, 1, "f32"), 0.1, 40, "f32"), "f32")
    T, R = oracle.tdf_spline(F, 1.5, 12.0, 0.5)
    T64, _ = oracle.tdf_spline(F.astype(np.float64), 1.5, 12.0, 0.5, f64=True)
    assert (T > 0).sum() > 100
    assert np.mean(np.abs(T - T64) <= 1e-3) > 0.995


def test_spline_empty_range(oracle, tube):
    """rmin beyond rmax: no radius is searched, every voxel is invalid."""
    F, _ = tube
    T, R = oracle.tdf_spline(F, 9.0, 4.0, 0.5)
    assert not T.any() and not R.any()
