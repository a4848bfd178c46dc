"""CPU tests: pin the oracle.

The reference publishes no golden vectors for GVF, TDF, eigen or the pyramid,
and its OpenCL runtime cannot run here.  The oracle is pinned two ways: to the
reference's own kernel text -- golden vectors written by running kernels.cl
under an OpenCL C shim on the CPU (tests/golden/, reproduced stage by stage
below; tests/test_reference_pin.py compares the two directly where the
reference source is present) -- and by what can be checked independently:
published algorithms against numpy, the pyramid order against its closed
form, the format conversions against numpy/IEEE, the sample-direction table
against the literals in the reference's kernels, and method-level invariants.
"""
import os
import re

import numpy as np
import pytest


def test_eigen_matches_numpy(oracle):
    rng = np.random.default_rng(0)
    for f64 in (True, False):
        tol = 1e-12 if f64 else 2e-5
        for _ in range(500):
            A = rng.normal(size=(3, 3))
            A = (A + A.T) / 2
            d, V = oracle.eig3(A, f64=f64)
            w, U = np.linalg.eigh(A.astype(np.float64))
            o = np.argsort(np.abs(w), kind="stable")
            w, U = w[o], U[:, o]
            assert np.max(np.abs(d - w)) < tol * 10
            for k in range(3):
                err = min(np.max(np.abs(V[:, k] - U[:, k])), np.max(np.abs(V[:, k] + U[:, k])))
                gap = np.min(np.abs(np.delete(w, k) - w[k]))
                if gap > 1e-3:
                    assert err < tol * 100 / gap


def test_eigen_known_answers(oracle):
    d, V = oracle.eig3(np.diag([1.0, -3.0, 2.0]), f64=True)
    assert np.allclose(d, [1.0, 2.0, -3.0])                 # ascending |lambda|
    assert np.allclose(np.abs(V), [[1, 0, 0], [0, 0, 1], [0, 1, 0]])
    d, V = oracle.eig3(np.zeros((3, 3)), f64=True)           # degenerate: identity basis
    assert np.allclose(d, 0) and np.allclose(np.abs(V), np.eye(3))


def _key(x, y, z, bits=12):
    k = np.zeros(x.shape, np.int64)
    for b in range(bits):
        k |= (((x >> b) & 1) | (((z >> b) & 1) << 1) | (((y >> b) & 1) << 2)).astype(np.int64) << (3 * b)
    return k


@pytest.mark.parametrize("shape", [(8, 8, 8), (20, 24, 17), (3, 40, 9), (33, 5, 64)])
def test_pyramid_order_is_key_sort(oracle, shape):
    rng = np.random.default_rng(1)
    m = (rng.random(shape) < 0.1).astype(np.int8)
    pos = oracle.hp_compact(m)
    z, y, x = np.nonzero(m)
    o = np.argsort(_key(x, y, z), kind="stable")
    assert np.array_equal(pos, np.stack([x[o], y[o], z[o]], 1))


def test_float16_rounding_matches_numpy(oracle):
    rng = np.random.default_rng(2)
    a = (rng.normal(size=200000) * 10.0 ** rng.integers(-9, 6, size=200000)).astype(np.float32)
    a = np.concatenate([a, np.float32([65504, 65519, 65520, 7e-8, 2.98e-8, 0.0, -0.0])])
    assert np.array_equal(oracle.quantize(a, "f16"), a.astype(np.float16).astype(np.float32))


def test_bfloat16_rounding_matches_torch(oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a = (rng.normal(size=100000) * 10.0 ** rng.integers(-20, 20, size=100000)).astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).float().numpy()
    assert np.array_equal(oracle.quantize(a, "bf16"), ref)


def test_snorm16_and_unorm16_conversions(oracle):
    # OpenCL 1.1: convert_short_sat_rte(v * 32767), read max(-1, s / 32767)
    a = np.float32([-2.0, -1.0, -0.5, 0.0, 1.5 / 32767, 2.5 / 32767, 0.25, 1.0, 3.0])
    s = np.clip(np.rint(a * np.float32(32767)), -32768, 32767)
    expect = np.maximum(np.float32(-1), (s / 32767).astype(np.float32))
    assert np.array_equal(oracle.quantize(a, "snorm16"), expect)
    u = oracle.to_unorm16(np.float32([-1, 0, 0.5, 1, 2, 0.5 / 65535, 1.5 / 65535]))
    assert list(u) == [0, 0, 32768, 65535, 65535, 0, 2]
    assert oracle.from_unorm16(np.uint16([65535]))[0] == 1.0


def test_circle_table_matches_reference_literals(oracle, reference_dir):
    src = open(os.path.join(reference_dir, "kernels.cl")).read()
    c = re.search(r"cosValues\[32\]\s*=\s*\{([^}]*)\}", src).group(1)
    s = re.search(r"sinValues\[32\]\s*=\s*\{([^}]*)\}", src).group(1)
    ref_c = np.float32([float(v.strip().rstrip("f")) for v in c.split(",")])
    ref_s = np.float32([float(v.strip().rstrip("f")) for v in s.split(",")])
    oc, os_ = oracle.circle_table()
    assert np.array_equal(oc, ref_c) and np.array_equal(os_, ref_s)


def test_blur_mask(oracle):
    for sigma, m in [(0.5, 1), (1.0, 2), (2.2, 5), (9.0, 5), (0.1, 1)]:
        mm, mask = oracle.blur_mask(sigma)
        assert mm == m
        S = 2 * m + 1
        k = mask.reshape(S, S, S)
        assert abs(float(mask.astype(np.float64).sum()) - 1.0) < 1e-5
        assert np.array_equal(k, k[::-1]) and np.array_equal(k, k.transpose(2, 1, 0))


def test_gvf_constant_field_is_fixed_point(oracle):
    f = np.zeros((6, 7, 8, 4), np.float32)
    f[..., 0], f[..., 1], f[..., 2], f[..., 3] = 0.25, -0.5, 0.125, 1.0
    for storage in ("f32", "f16", "snorm16"):
        v = oracle.gvf(oracle.quantize(f, storage).reshape(f.shape), 0.05, 7, storage)
        assert np.array_equal(v[0], np.full((6, 7, 8), oracle.quantize(np.float32([0.25]), storage)[0]))


def test_gvf_mirror_boundary(oracle, synth):
    """Boundary voxels carry the update computed at index 2 / size-3
    (kernels.cl:1472-1475): after an iteration plane 0 equals plane 2."""
    vol = oracle.blur(synth.vascular_tree((16, 18, 20), seed=1), 0.5)
    v = oracle.gvf(oracle.vector_field(vol, 0.2, 1, "f32"), 0.05, 3, "f32")
    assert np.array_equal(v[:, 0], v[:, 2]) and np.array_equal(v[:, -1], v[:, -3])
    assert np.array_equal(v[:, :, 0], v[:, :, 2]) and np.array_equal(v[:, :, :, -1], v[:, :, :, -3])


def test_gvf_f64_and_f32_agree_when_stable(oracle, synth):
    vol = synth.vascular_tree((24, 24, 24), seed=2)
    f32 = oracle.gvf(oracle.vector_field(oracle.blur(vol, 0.5), 0.2, 1), 0.05, 50)
    f64 = oracle.gvf(oracle.vector_field(oracle.blur(vol, 0.5, f64=True), 0.2, 1, f64=True), 0.05, 50,
                     f64=True)
    assert np.max(np.abs(f32 - f64)) < 1e-5


def test_gvf_unstable_at_mu_0_1(oracle, synth):
    """The explicit scheme needs 12 mu + |f0|^2 <= 2: at mu = 0.1 the
    checkerboard mode, amplified by 1 - 12 mu - |f0|^2 per iteration, grows
    where |f0| = 1; at mu = 0.08 it stays bounded."""
    vol = synth.vascular_tree((32, 32, 32), seed=0)
    f4 = oracle.vector_field(oracle.blur(vol, 0.5, f64=True), 0.2, 1, f64=True)
    assert np.abs(oracle.gvf(f4, 0.1, 150, f64=True)).max() > 10.0
    assert np.abs(oracle.gvf(f4, 0.08, 150, f64=True)).max() <= 1.0


def test_tdf_detects_a_straight_tube(oracle):
    """A bright straight cylinder of radius 3 along z: the TDF peaks on its
    axis with a radius near 3."""
    Z = Y = X = 32
    z, y, x = np.mgrid[:Z, :Y, :X].astype(np.float32)
    vol = ((x - 15.5) ** 2 + (y - 15.5) ** 2 <= 9.0).astype(np.float32)
    f4 = oracle.vector_field(oracle.blur(vol, 1.0), 0.1, 1)
    v = oracle.gvf(f4, 0.05, 100)
    field = oracle.gvf_finish(v)
    T, R = oracle.tdf_circle(field, 2.5, 6.0, 0.5)
    sl = T[16]
    iy, ix = np.unravel_index(np.argmax(sl), sl.shape)
    assert abs(ix - 15.5) <= 1.5 and abs(iy - 15.5) <= 1.5
    assert sl.max() > 0.5 and 2.0 <= R[16, iy, ix] <= 4.5


def test_fmg_reduces_residual(oracle, synth):
    vol = synth.vascular_tree((32, 32, 32), seed=3)
    f4 = oracle.vector_field(oracle.blur(vol, 0.5, f64=True), 0.2, 1, f64=True)
    a = oracle.fmg_gvf(f4, 0.2, 1, f64=True)
    b = oracle.fmg_gvf(f4, 0.2, 3, f64=True)

    def res(o):
        v = np.moveaxis(o[..., :3], -1, 0)
        f = np.moveaxis(f4[..., :3], -1, 0)
        s = (f ** 2).sum(0)
        lap = (np.roll(v, 1, 1) + np.roll(v, -1, 1) + np.roll(v, 1, 2) + np.roll(v, -1, 2) +
               np.roll(v, 1, 3) + np.roll(v, -1, 3) - 6 * v)
        r = 0.2 * lap - s * (v - f)
        return np.abs(r[:, 2:-2, 2:-2, 2:-2]).mean()

    assert res(b) < res(a)


def _hp2d_traverse(img):
    """The reference's 2-D histogram pyramid (constructHPLevel2D,
    scanHPLevel2D, traverseHP2D: kernels.cl:100-142, 229-275) simulated
    directly: returns the (x, y) of every set pixel of img[y, x], in the
    order the traversal enumerates them."""
    S = 2
    while S < max(img.shape):
        S *= 2
    base = np.zeros((S, S), np.int64)
    base[:img.shape[0], :img.shape[1]] = img
    levels = [base]
    while levels[-1].shape[0] > 2:
        l = levels[-1]
        levels.append(l[0::2, 0::2] + l[0::2, 1::2] + l[1::2, 0::2] + l[1::2, 1::2])

    def rd(l, x, y):
        return int(l[y, x]) if 0 <= x < l.shape[1] and 0 <= y < l.shape[0] else 0

    offsets = [(0, 0), (0, 1), (1, 0), (1, 1)]
    out = []
    for t in range(int(base.sum())):
        x = y = acc0 = 0
        for l in reversed(levels):
            n0, n1, n2 = rd(l, x, y), rd(l, x, y + 1), rd(l, x + 1, y)
            acc = acc0 + n0
            c0 = acc <= t
            acc += n1
            c1 = acc <= t
            acc += n2
            c2 = acc <= t
            dx, dy = offsets[c0 + c1 + c2]
            x, y = 2 * (x + dx), 2 * (y + dy)
            acc0 += c0 * n0 + c1 * n1 + c2 * n2
        out.append((x // 2, y // 2))
    return out


@pytest.mark.parametrize("shape", [(8, 8), (13, 21), (40, 33)])
def test_pyramid_2d_order_is_key_sort(shape):
    """The edge list order of the linking stage: a sort by the key that
    interleaves the bits of (x, y) with y as the low bit."""
    rng = np.random.default_rng(5)
    img = (rng.random(shape) < 0.15).astype(np.int64)
    ys, xs = np.nonzero(img)
    key = np.zeros(xs.shape, np.int64)
    for b in range(8):
        key |= (((ys >> b) & 1) | (((xs >> b) & 1) << 1)).astype(np.int64) << (2 * b)
    o = np.argsort(key, kind="stable")
    assert _hp2d_traverse(img) == list(zip(xs[o].tolist(), ys[o].tolist()))


def test_link_chain_known_answer(oracle):
    """Vertices on a line 3 voxels apart inside a bright tube: every inner
    vertex links to both neighbours (angle pi >= 2 rad), one tree.  The end
    vertices have one candidate within the distance and link nothing
    themselves; the tuple (1, 0) is kept as is (no (0, 1)).  Rasterisation
    runs from an edge's first vertex and stops before the second, so x = 2
    (vertex 0, only ever a second vertex) stays unset."""
    T = np.zeros((12, 12, 40), np.float32)
    T[4:8, 4:8, :] = 1.0
    v = np.array([[2 + 3 * i, 6, 6] for i in range(12)], np.int32)
    edges, labels, sizes = oracle.link_centerpoints(v, T, 0.5, 5.0)
    pairs = {tuple(sorted(e)) for e in edges.tolist()}
    assert pairs == {(i, i + 1) for i in range(11)}
    assert edges.tolist()[0] == [1, 0]
    assert (labels == 0).all() and sizes[0] == 12
    cl = oracle.rasterize_trees(v, edges, labels, sizes, 5, T.shape)
    assert cl[6, 6, 3:35].all() and cl.sum() == 32


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
def test_oracle_reproduces_reference_golden(oracle, storage):
    """The oracle against the golden vectors of the reference's own kernel
    text (tests/golden/make_golden.py): every stage bit for bit."""
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_%s.npz" % storage))
    P = dict(zip([str(k) for k in d["param_names"]], d["params"]))
    unorm = storage == "snorm16"

    def st(a):
        return oracle.quantize(a, storage) if storage == "snorm16" else a

    def raw(a):
        return np.rint(a.astype(np.float64) * 32767.0).astype(np.int16) if storage == "snorm16" else a

    vol = d["volume"]
    b = oracle.blur(vol, P["sigma"])
    assert np.array_equal(b, d["blurred"])
    f4 = oracle.vector_field(b, P["fmax"], int(P["vsign"]), storage)
    assert np.array_equal(raw(f4), d["field"])
    fs = oracle.vector_field(vol, P["fmax"], int(P["vsign"]), storage)
    assert np.array_equal(raw(fs), d["field_small"])
    v = oracle.gvf(f4, P["mu"], int(P["iterations"]), storage)
    assert np.array_equal(raw(v), d["gvf"])
    fin = oracle.gvf_finish(v, storage)
    assert np.array_equal(raw(fin), d["gvf_field"])
    Ts, Rs = oracle.tdf_circle(fs, 1.0, 3.0, 0.5)
    Tl, Rl = oracle.tdf_circle(fin, 2.5, 7.0, 0.5)
    conv = oracle.to_unorm16 if unorm else (lambda a: a)
    # combine compares the stored TDF values (unorm16 in the 16-bit mode)
    take = conv(Tl) < conv(Ts)
    T, R = np.where(take, Ts, Tl), np.where(take, Rs, Rl)
    assert np.array_equal(conv(Ts), d["T_small"]) and np.array_equal(Rs, d["R_small"])
    assert np.array_equal(conv(T), d["T"]) and np.array_equal(R, d["R"])
    T_read = oracle.from_unorm16(d["T"]) if unorm else T
    c = oracle.centerpoints(T_read, R, fin, P["tdf_high"], int(P["cube"]))
    assert np.array_equal(c["candidates"], d["candidates"])
    assert np.array_equal(c["mask2"], d["mask2"])
    assert np.array_equal(c["vertices"], d["vertices"])


@pytest.mark.parametrize("kind", [0, 1])
def test_residual_norm_matches_numpy(oracle, synth, kind):
    """The oracle's FP64 residual norms against a float64 numpy evaluation of
    the same residual (mirror rule, spacing 1): agreement to float rounding."""
    vol = oracle.blur(synth.vascular_tree((12, 14, 16), seed=3), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1)
    f0 = np.moveaxis(f4[..., :3], -1, 0).copy()
    v = oracle.gvf(f4, 0.05, 5)
    got = oracle.gvf_residual_norm(f0, v, 0.05, kind)
    m = [np.array([2 if i == 0 else (n - 3 if i >= n - 1 else i) for i in range(n)]) for n in v.shape[1:]]
    V, F = v.astype(np.float64), f0.astype(np.float64)
    sqr = (F ** 2).sum(0)
    r = np.zeros_like(V)
    Vp = np.pad(V, ((0, 0), (1, 1), (1, 1), (1, 1)), mode="edge")
    lap = (Vp[:, 1:-1, 1:-1, 2:] + Vp[:, 1:-1, 1:-1, :-2] + Vp[:, 1:-1, 2:, 1:-1] + Vp[:, 1:-1, :-2, 1:-1] +
           Vp[:, 2:, 1:-1, 1:-1] + Vp[:, :-2, 1:-1, 1:-1] - 6 * V)
    r = 0.05 * lap - (V - F) * sqr if kind == 0 else -sqr * F - (0.05 * lap - sqr * V)
    r = r[:, m[0]][:, :, m[1]][:, :, :, m[2]]
    want = [np.sqrt((r[c] ** 2).sum()) for c in range(3)]
    assert np.allclose(got[:3], want, rtol=1e-5)
    assert np.isclose(got[3], np.sqrt(sum(w ** 2 for w in want)), rtol=1e-5)
    assert np.isclose(got[4], np.abs(r).max(), rtol=1e-5)
