"""Segmentation oracle (no GPU): inverse-gradient region growing and sphere
segmentation (segmentation.cpp:5-307; kernels initGrowing, grow, dilate,
erode, sphereSegmentation, kernels_no_3d_write.cl:1100-1234, 1370-1412).

The C restatement is checked against a second, pure-Python restatement that
follows the kernel text loop by loop on small volumes, against brute-force
known answers, and on a synthetic bright cylinder whose extent it must find."""
import itertools

import numpy as np
import pytest

OFFS = [o for o in itertools.product((-1, 0, 1), repeat=3) if o != (0, 0, 0)]   # (a, b, c) = (x, y, z), x outermost


def _py_segment(cl, F, R):
    """Pure-Python restatement (float32 arithmetic op by op)."""
    Z, Y, X = cl.shape
    f32 = np.float32
    clamp = lambda v, n: min(max(v, 0), n - 1)
    inside = lambda x, y, z: 0 <= x < X and 0 <= y < Y and 0 <= z < Z
    st = cl.copy()
    # initGrowing
    for z, y, x in zip(*np.nonzero(cl == 1)):
        N = min(max(1, int(np.round(f32(R[z, y, x]) / f32(2.0)))), 4)
        for a in range(-N, N + 1):
            for b in range(-N, N + 1):
                for c in range(-N, N + 1):
                    nx, ny, nz = x + a, y + b, z + c
                    if inside(nx, ny, nz) and cl[nz, ny, nx] == 0:
                        st[nz, ny, nx] = 2
    dirs = []
    for a2, b2, c2 in OFFS:
        l = np.sqrt(f32(a2 * a2 + b2 * b2 + c2 * c2), dtype=np.float32)
        dirs.append(((a2, b2, c2), (f32(a2) / l, f32(b2) / l, f32(c2) / l)))
    iters = 0
    while True:
        iters += 1
        acc = np.zeros_like(st)
        mark = np.zeros_like(st)
        any_ = False
        for z, y, x in zip(*np.nonzero(st == 2)):
            wX = F[z, y, x, 3]
            grew = False
            for a, b, c in OFFS:
                yx, yy, yz = x + a, y + b, z + c
                cx, cy, cz = clamp(yx, X), clamp(yy, Y), clamp(yz, Z)
                if st[cz, cy, cx] == 1:
                    continue
                w = F[cz, cy, cx, 3]
                with np.errstate(divide="ignore", invalid="ignore"):
                    fx, fy, fz = (F[cz, cy, cx, k] / w for k in range(3))
                if not w > wX:
                    continue
                best, zpos = f32(-2.0), None
                for (a2, b2, c2), (dx, dy, dz) in dirs:
                    v = (fx * dx + fy * dy) + fz * dz
                    if v > best:
                        best, zpos = v, (yx + a2, yy + b2, yz + c2)
                if zpos == (x, y, z) and inside(yx, yy, yz):
                    mark[yz, yy, yx] = 1
                    grew = True
            if grew:
                acc[z, y, x] = 1
                any_ = True
        st = np.where((st == 1) | (acc == 1), 1, np.where(mark == 1, 2, 0)).astype(np.int8)
        if not any_:
            break
    dil = np.zeros_like(st)
    for z, y, x in zip(*np.nonzero(st == 1)):
        dil[max(z - 1, 0):z + 2, max(y - 1, 0):y + 2, max(x - 1, 0):x + 2] = 1
    pad = np.pad(dil, 1, mode="edge")
    out = np.ones_like(dil)
    for dz, dy, dx in itertools.product(range(3), repeat=3):
        out &= pad[dz:dz + Z, dy:dy + Y, dx:dx + X]
    return out.astype(np.int8), iters


def _spheres_brute(cl, R):
    Z, Y, X = cl.shape
    out = np.zeros(cl.shape, np.int8)
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    for z, y, x in zip(*np.nonzero(cl)):
        r = np.float32(R[z, y, x])
        N = int(np.ceil(r))
        d2 = (xx - x) ** 2 + (yy - y) ** 2 + (zz - z) ** 2
        near = (np.abs(xx - x) <= N) & (np.abs(yy - y) <= N) & (np.abs(zz - z) <= N)
        out[near & (np.sqrt(d2.astype(np.float32)) < r)] = 1
    return out


def _random_case(seed, shape, p_cl=0.03):
    rng = np.random.default_rng(seed)
    cl = (rng.random(shape) < p_cl).astype(np.int8)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    w = rng.random(shape).astype(np.float32)
    n = np.sqrt((v * v).sum(-1))
    F = np.concatenate([v / n[..., None] * w[..., None], w[..., None]], -1).astype(np.float32)
    R = (rng.random(shape) * 7.0).astype(np.float32)
    return cl, F, R


@pytest.mark.parametrize("seed,shape", [(0, (5, 6, 7)), (1, (6, 6, 6)), (2, (4, 9, 5))])
def test_grow_matches_python_restatement(oracle, seed, shape):
    cl, F, R = _random_case(seed, shape)
    seg, it = oracle.segment_inverse_gradient(cl, F, R)
    ref, rit = _py_segment(cl, F, R)
    assert np.array_equal(seg, ref)
    assert it == rit


def test_grow_on_a_radial_field_follows_the_gradient(oracle):
    """A field pointing at the axis with magnitude rising outwards to a peak
    at distance 6: growing fills the inside and stops short of the peak (a
    voxel is accepted only through a neighbour of larger magnitude)."""
    Z, Y, X = 12, 20, 20
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    dy, dx = (yy - 9.5).astype(np.float32), (xx - 9.5).astype(np.float32)
    d = np.sqrt(dx * dx + dy * dy)
    w = np.where(d <= 6.0, d / 6.0, np.maximum(0.0, 1.0 - (d - 6.0))).astype(np.float32)
    F = np.stack([-dx / d * w, -dy / d * w, np.zeros_like(d), w], -1).astype(np.float32)
    cl = np.zeros((Z, Y, X), np.int8)
    cl[:, 9:11, 9:11] = 1
    R = np.full((Z, Y, X), 2.0, np.float32)
    seg, it = oracle.segment_inverse_gradient(cl, F, R)
    ref, rit = _py_segment(cl, F, R)
    assert np.array_equal(seg, ref) and it == rit
    assert it > 3
    assert seg[d <= 4.5].all()                    # the inside grows
    assert not seg[d >= 6.0].any()                # nothing at or beyond the peak


def test_grow_without_centerline(oracle):
    cl = np.zeros((6, 6, 6), np.int8)
    F = np.ones((6, 6, 6, 4), np.float32)
    seg, it = oracle.segment_inverse_gradient(cl, F, np.ones((6, 6, 6), np.float32))
    assert not seg.any() and it == 1


def test_centerline_alone_is_closed(oracle):
    """With no accepting neighbour the checked voxels drop; the closing of a
    centerline line returns the line, except that erosion reads clamp to the
    edge: a line ending one voxel from the border extends to the border."""
    shape = (8, 8, 10)
    F = np.zeros(shape + (4,), np.float32)        # w = 0 everywhere: nothing exceeds it
    R = np.full(shape, 3.0, np.float32)
    cl = np.zeros(shape, np.int8)
    cl[4, 4, 2:8] = 1
    seg, it = oracle.segment_inverse_gradient(cl, F, R)
    assert it == 1 and np.array_equal(seg, cl)
    cl = np.zeros(shape, np.int8)
    cl[4, 4, 1:9] = 1
    seg, it = oracle.segment_inverse_gradient(cl, F, R)
    ref, _ = _py_segment(cl, F, R)
    assert np.array_equal(seg, ref)
    want = np.zeros(shape, np.int8)
    want[4, 4, :] = 1
    assert np.array_equal(seg, want)


@pytest.mark.parametrize("r", [0.5, 1.0, 1.5, 2.0, 2.5, 3.2, 4.0])
def test_spheres_known_answer(oracle, r):
    cl = np.zeros((11, 11, 11), np.int8)
    cl[5, 5, 5] = 1
    cl[0, 10, 0] = 1                              # clipped at the corner
    R = np.full(cl.shape, r, np.float32)
    out = oracle.segment_spheres(cl, R)
    assert np.array_equal(out, _spheres_brute(cl, R))
    counts = {0.5: 1, 1.0: 1, 1.5: 19, 2.0: 27, 2.5: 81}
    if r in counts:
        assert out[2:9, 2:9, 2:9].sum() == counts[r]   # the centre ball alone


def test_spheres_random(oracle):
    rng = np.random.default_rng(5)
    cl = (rng.random((10, 12, 14)) < 0.01).astype(np.int8)
    R = (rng.random(cl.shape) * 5).astype(np.float32)
    assert np.array_equal(oracle.segment_spheres(cl, R), _spheres_brute(cl, R))
