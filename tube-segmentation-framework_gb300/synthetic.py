"""Seeded synthetic volumes for the tube-segmentation workloads.

There is no public dataset behind the benchmark workloads, so volumes are
generated: a random binary tree of tubes, each segment a quadratic Bezier
curve rasterised as a union of balls, plus noise.  Every generator returns the
intensity volume (numpy, indexed [z, y, x]) and the generator-known centerline.

    vascular_tree(shape, seed)          128^3 / 256^3 / 192^3 vessel phantoms:
        31 tubes (5 generations), radius 6 * 0.8^g (floor 1), segments 15-40
        voxels long, intensity 1 on 0, Gaussian noise sigma 0.15, clamp [0,1].
    mra_tree(shape, seed)               512^3 MRA-like phantom: 63 tubes,
        radii 5 -> 0.8, intensity 1 on 0.1, Rician noise sigma 0.08.
    lung_ct(shape, seed)                512x512x400 int16 HU airway phantom.
"""
from __future__ import annotations

import numpy as np


def _unit(v):
    return v / np.linalg.norm(v)


def _rotate_towards(d, rng, angle):
    """Rotate unit vector d by `angle` radians about a random axis orthogonal to d."""
    a = rng.normal(size=3)
    a -= a.dot(d) * d
    a = _unit(a)
    return _unit(np.cos(angle) * d + np.sin(angle) * a)


def _tree_segments(shape, rng, n_generations, r0, r_factor, r_floor, len_range,
                   margin=8.0):
    """Control points (P0, P1, P2) and radius of every segment of a binary tree
    rooted at a random point of a random face, growing inwards."""
    Z, Y, X = shape
    ext = np.array([X, Y, Z], float)
    margin = np.minimum(margin, ext / 4.0)      # thin volumes
    face = rng.integers(6)
    axis, side = face // 2, face % 2
    p0 = rng.uniform(margin, ext - margin)
    p0[axis] = 0.5 if side == 0 else ext[axis] - 1.5
    d0 = np.zeros(3)
    d0[axis] = 1.0 if side == 0 else -1.0
    d0 = _rotate_towards(d0, rng, rng.uniform(0.0, 0.35))
    segs = []
    stack = [(p0, d0, 0)]
    while stack:
        p, d, g = stack.pop()
        if g >= n_generations:
            continue
        r = max(r_floor, r0 * r_factor ** g)
        L = rng.uniform(*len_range)
        # keep the tree inside the volume: bend back towards the centre if needed
        centre = ext / 2
        end = p + L * d
        if np.any(end < margin) or np.any(end > ext - margin):
            d = _unit(0.5 * d + 0.5 * _unit(centre - p))
            end = p + L * d
        mid = 0.5 * (p + end) + rng.normal(scale=0.15 * L, size=3)
        segs.append((p.copy(), mid, end.copy(), r))
        tangent = _unit(end - mid)
        for _ in range(2):
            stack.append((end.copy(), _rotate_towards(tangent, rng, rng.uniform(0.35, 0.9)), g + 1))
    return segs


def _bezier(p0, p1, p2, step=0.25):
    L = np.linalg.norm(p1 - p0) + np.linalg.norm(p2 - p1)
    n = max(2, int(np.ceil(L / step)) + 1)
    t = np.linspace(0.0, 1.0, n)[:, None]
    return (1 - t) ** 2 * p0 + 2 * (1 - t) * t * p1 + t ** 2 * p2


def _paint_balls(vol, pts, r, value=1.0):
    """vol[z,y,x] = value for all voxel centres within distance r of any point."""
    Z, Y, X = vol.shape
    R = int(np.ceil(r))
    off = np.arange(-R - 1, R + 2)
    oz, oy, ox = np.meshgrid(off, off, off, indexing="ij")
    for c in pts:
        ci = np.floor(c).astype(int)
        xs, ys, zs = ci[0] + ox, ci[1] + oy, ci[2] + oz
        d2 = (xs - c[0]) ** 2 + (ys - c[1]) ** 2 + (zs - c[2]) ** 2
        ok = (d2 <= r * r) & (xs >= 0) & (ys >= 0) & (zs >= 0) & (xs < X) & (ys < Y) & (zs < Z)
        vol[zs[ok], ys[ok], xs[ok]] = value


def _rasterise(shape, segs):
    vol = np.zeros(shape, np.float32)
    cl = np.zeros(shape, np.int8)
    Z, Y, X = shape
    pts_all = []
    for p0, p1, p2, r in segs:
        pts = _bezier(p0, p1, p2)
        _paint_balls(vol, pts, r)
        idx = np.round(pts).astype(int)
        ok = np.all((idx >= 0) & (idx < np.array([X, Y, Z])), axis=1)
        idx = idx[ok]
        cl[idx[:, 2], idx[:, 1], idx[:, 0]] = 1
        pts_all.append(pts)
    return vol, cl, np.concatenate(pts_all) if pts_all else np.zeros((0, 3))


def centerline_gaussian(shape, pts, sigma=1.0):
    """exp(-d^2 / (2 sigma^2)) with d the distance to the nearest centerline
    sample (evaluated within 3 sigma)."""
    out = np.zeros(shape, np.float32)
    Z, Y, X = shape
    R = int(np.ceil(3 * sigma))
    off = np.arange(-R - 1, R + 2)
    oz, oy, ox = np.meshgrid(off, off, off, indexing="ij")
    for c in pts:
        ci = np.floor(c).astype(int)
        xs, ys, zs = ci[0] + ox, ci[1] + oy, ci[2] + oz
        ok = (xs >= 0) & (ys >= 0) & (zs >= 0) & (xs < X) & (ys < Y) & (zs < Z)
        xs, ys, zs = xs[ok], ys[ok], zs[ok]
        d2 = (xs - c[0]) ** 2 + (ys - c[1]) ** 2 + (zs - c[2]) ** 2
        g = np.exp(-d2 / (2 * sigma * sigma)).astype(np.float32)
        np.maximum.at(out, (zs, ys, xs), g)
    return out


def vascular_tree(shape=(128, 128, 128), seed=0, n_tubes=31, noise=0.15, with_truth=False):
    """The 128^3 / 256^3 / 192^3 vessel phantom (float32 in [0,1])."""
    rng = np.random.default_rng(seed)
    n_gen = int(round(np.log2(n_tubes + 1)))
    segs = _tree_segments(shape, rng, n_gen, 6.0, 0.8, 1.0, (15.0, 40.0))
    vol, cl, pts = _rasterise(shape, segs)
    vol += rng.normal(scale=noise, size=shape).astype(np.float32)
    np.clip(vol, 0.0, 1.0, out=vol)
    if with_truth:
        return vol, {"centerline": cl, "points": pts, "segments": segs}
    return vol


def mra_tree(shape=(512, 512, 512), seed=0, n_tubes=63, sigma=0.08, with_truth=False):
    """MRA-like phantom: bright tubes (radii 5 -> 0.8) on 0.1, Rician noise."""
    rng = np.random.default_rng(seed)
    n_gen = int(round(np.log2(n_tubes + 1)))
    q = (0.8 / 5.0) ** (1.0 / max(1, n_gen - 1))
    segs = _tree_segments(shape, rng, n_gen, 5.0, q, 0.8, (15.0, 40.0))
    vol, cl, pts = _rasterise(shape, segs)
    vol = 0.1 + 0.9 * vol
    n1 = rng.normal(scale=sigma, size=shape).astype(np.float32)
    n2 = rng.normal(scale=sigma, size=shape).astype(np.float32)
    vol = np.sqrt((vol + n1) ** 2 + n2 ** 2).astype(np.float32)
    np.clip(vol, 0.0, 1.0, out=vol)
    if with_truth:
        return vol, {"centerline": cl, "points": pts, "segments": segs}
    return vol


def lung_ct(shape=(400, 512, 512), seed=0, with_truth=False):
    """Lung-airway-like CT in HU (int16), indexed [z, y, x].

    Parenchyma -850 +- 30 HU inside a lung ellipsoid, body +40 HU outside it,
    a 6-generation airway tree (trachea radius 9 halving every 2 generations
    to 1, segments 20-60 voxels) with lumen -1000 HU and a wall of thickness
    0.25 r at -100 HU, additive Gaussian noise sigma 25 HU."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    zz, yy, xx = np.ogrid[:Z, :Y, :X]
    inside = (((xx - X / 2) / (0.45 * X)) ** 2 + ((yy - Y / 2) / (0.42 * Y)) ** 2 +
              ((zz - Z / 2) / (0.48 * Z)) ** 2) <= 1.0
    vol = np.where(inside, np.float32(-850.0), np.float32(40.0)).astype(np.float32)
    vol += np.where(inside, rng.normal(scale=30.0, size=shape).astype(np.float32), 0)
    # airway tree from the top (z = 0 side) downwards
    segs = []
    p0 = np.array([X / 2, Y / 2, 1.0])
    stack = [(p0, np.array([0.0, 0.0, 1.0]), 0)]
    while stack:
        p, d, g = stack.pop()
        if g >= 6:
            continue
        r = max(1.0, 9.0 * 0.5 ** (g // 2))
        L = rng.uniform(20.0, 60.0)
        end = p + L * d
        mid = 0.5 * (p + end) + rng.normal(scale=0.1 * L, size=3)
        segs.append((p.copy(), mid, end.copy(), r))
        t = _unit(end - mid)
        for _ in range(2):
            stack.append((end.copy(), _rotate_towards(t, rng, rng.uniform(0.4, 0.8)), g + 1))
    wall = np.zeros(shape, np.float32)
    lumen = np.zeros(shape, np.float32)
    pts_all = []
    for p0_, p1_, p2_, r in segs:
        pts = _bezier(p0_, p1_, p2_)
        _paint_balls(wall, pts, r * 1.25)
        _paint_balls(lumen, pts, r)
        pts_all.append(pts)
    vol = np.where(wall > 0, np.float32(-100.0), vol)
    vol = np.where(lumen > 0, np.float32(-1000.0), vol)
    vol += rng.normal(scale=25.0, size=shape).astype(np.float32)
    hu = np.clip(np.round(vol), -32768, 32767).astype(np.int16)
    if with_truth:
        return hu, {"points": np.concatenate(pts_all), "segments": segs}
    return hu


def window_to_unit(hu, lo=-1100.0, hi=-600.0):
    """toFloat semantics (kernels.cl:989-1015): clamp to [lo, hi], map to [0,1]."""
    v = np.clip(hu.astype(np.float32), lo, hi)
    return ((v - np.float32(lo)) / np.float32(hi - lo)).astype(np.float32)
