"""Cropping, CPU side (no GPU): the oracle's scan-line counts
(cropDatasetThreshold / cropDatasetLung, kernels.cl:813-946) on known
answers, and the host crop box of the C ABI (tsf_crop_bounds,
tsf_crop_box_fixed; tube-segmentation.cpp:1611-1772) against a Python
restatement of the reference's host code on random counts."""
import numpy as np
import pytest


def py_crop_bounds(cx, cy, cz, min_lines, middle):
    """tube-segmentation.cpp:1611-1719, restated."""
    X, Y, Z = len(cx), len(cy), len(cz)
    x1, x2, y1, y2, z1, z2 = 0, X, 0, Y, 0, Z
    start, a = (Z // 2, -1) if middle else (0, 1)
    for s in range(X):
        if cx[s] > min_lines:
            x1 = s
            break
    for s in range(X - 1, 0, -1):
        if cx[s] > min_lines:
            x2 = s
            break
    for s in range(Y):
        if cy[s] > min_lines:
            y1 = s
            break
    for s in range(Y - 1, 0, -1):
        if cy[s] > min_lines:
            y2 = s
            break
    for s in range(start, Z):
        if a * int(cz[s]) > a * min_lines:
            z2 = s
            break
    for s in range(Z - start - 1, 0, -1):
        if a * int(cz[s]) > a * min_lines:
            z1 = s
            break
    if not middle:
        z1, z2 = z2, z1
    S = [x2 - x1, y2 - y1, z2 - z1]
    if min(S) <= 0:
        return None
    lo, hi, full = [x1, y1, z1], [x2, y2, z2], [X, Y, Z]
    lower = False
    for k in range(3):
        while S[k] % 4 != 0 and S[k] < full[k]:
            if lower and lo[k] > 0:
                lo[k] -= 1
            elif hi[k] < full[k]:
                hi[k] += 1
            lower = not lower
            S[k] = hi[k] - lo[k]
        while S[k] % 4 != 0:
            S[k] -= 1
    if min(S) <= 0:
        return None
    return (lo[0], lo[1], lo[2], S[0], S[1], S[2])


def test_threshold_counts_known_answer(oracle):
    v = np.zeros((8, 9, 10), np.int16)
    v[2:5, 3:6, 1:4] = 100
    cx, cy, cz = oracle.crop_scan_lines(v, 0, 50.0)
    assert cx.tolist() == [0, 3, 3, 3] + [0] * 6
    assert cy.tolist() == [0, 0, 0, 3, 3, 3, 0, 0, 0]
    assert cz.tolist() == [0, 0, 3, 3, 3, 0, 0, 0]
    assert not any(a.any() for a in oracle.crop_scan_lines(v, 0, 100.0))   # strictly above


def test_lung_counts_known_answer(oracle):
    """A z-column white 40, black 40, white 40 (HU limit -150): two white
    areas and one black -> inside; white 40, black 40 only -> not."""
    Z = 120
    v = np.full((Z, 4, 5), -1000, np.int16)
    col = np.r_[np.full(40, 0), np.full(40, -1000), np.full(40, 0)].astype(np.int16)
    v[:, 1, 2] = col
    v[:80, 2, 3] = col[:80]
    cx, cy, cz = oracle.crop_scan_lines(v, 1)
    assert cx.tolist() == [0, 0, 1, 0, 0] and cy.tolist() == [0, 1, 0, 0]
    # unsigned data: limit -150 + 1024
    cxu, cyu, _ = oracle.crop_scan_lines((v.astype(np.int32) + 1024).astype(np.uint16), 1)
    assert cxu.tolist() == cx.tolist() and cyu.tolist() == cy.tolist()


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("middle", [False, True])
def test_crop_bounds_match_restatement(tsf, seed, middle):
    rng = np.random.default_rng(seed)
    X, Y, Z = (int(n) for n in rng.integers(9, 70, 3))
    lo, hi = sorted(rng.integers(0, 40, 2))
    cx, cy, cz = (rng.integers(0, 60, n).astype(np.int16) for n in (X, Y, Z))
    mn = int(rng.integers(lo, hi + 1))
    want = py_crop_bounds(cx, cy, cz, mn, middle)
    if want is None:
        with pytest.raises(tsf.TSFError):
            tsf.crop_bounds(cx, cy, cz, mn, middle)
    else:
        assert tsf.crop_bounds(cx, cy, cz, mn, middle) == want


def test_crop_bounds_known_answer(tsf):
    X, Y, Z = 40, 30, 50
    cx, cy, cz = np.zeros(X, np.int16), np.zeros(Y, np.int16), np.zeros(Z, np.int16)
    cx[7:31] = 20            # x: 7..30, 23 wide -> x2 + 1 (24)
    cy[5:25] = 20            # y: 5..24, 19 -> y1 - 1 (the alternation carries over)
    cz[10:40] = 20           # z: 10..39, 29 -> z2 + 1, z1 - 1, z2 + 1 (32)
    box = tsf.crop_bounds(cx, cy, cz, 10, False)
    assert box == py_crop_bounds(cx, cy, cz, 10, False)
    assert box == (7, 4, 9, 24, 20, 32)


def test_crop_bounds_empty_is_an_error(tsf):
    """"middle" with an odd Z: both z searches start at slice Z // 2, so a
    column of empty slices gives z1 = z2 and an empty box."""
    cx = cy = np.full(8, 50, np.int16)
    cz = np.zeros(13, np.int16)
    assert py_crop_bounds(cx, cy, cz, 10, True) is None
    with pytest.raises(tsf.TSFError, match="Invalid cropping"):
        tsf.crop_bounds(cx, cy, cz, 10, True)


@pytest.mark.parametrize("shape", [(100, 512, 512), (37, 101, 99), (8, 10, 12)])
def test_crop_box_fixed(tsf, shape):
    Z, Y, X = shape
    box = tsf.crop_box_fixed(shape, 0.15)
    ox, oy = (int(np.floor(np.float32(n) * np.float32(0.15) + 0.5)) for n in (X, Y))   # round half away
    assert box[:3] == (ox, oy, 0)
    assert box[3] == (X - 2 * ox) // 4 * 4 and box[4] == (Y - 2 * oy) // 4 * 4 and box[5] == Z // 4 * 4
