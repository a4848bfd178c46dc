"""The reference's system-test gates (tests/tubeSegmentationTests.cpp:41-99,
metrics of tests/tubeValidation.cpp:17-143) on its own synthetic dataset_1
(100^3 u8, preset Synthetic-Vascusynth, centerline-method gpu), run through
the oracle: toFloat, the small-radius and the GVF-based large-radius TDF, the
combination, the candidate stage, linking, the host loop removal (this
library's host code), and inverse-gradient segmentation.  Every GPU stage is
tested bit for bit against these oracle stages, so the gates pin the product
end to end.  Skipped where the reference's source tree (with its test data)
is absent."""
import os

import numpy as np
import pytest


def _volume(path):
    return np.fromfile(path, np.uint8).reshape(100, 100, 100)


def _pipeline(oracle, tsf, vol_u8, sixteen_bit):
    """run() with the Synthetic-Vascusynth preset: minimum 0, maximum 75,
    small-blur 1, large-blur 1, fmax 0.1, radius 0.5..4 (step 1; small pass
    0.5..3 step 0.5), 250 GVF iterations at mu 0.05, tdf-high 0.35, cube-size 3,
    min-mean-tdf 0.3, max-distance 10, min-tree-length 3, loop removal."""
    v = np.clip(vol_u8.astype(np.float32), np.float32(0), np.float32(75)) / np.float32(75)
    st = "snorm16" if sixteen_bit else "f32"
    fs = oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st)
    Ts, Rs = oracle.tdf_circle(fs, 0.5, 3.0, 0.5)
    field = oracle.gvf_finish(oracle.gvf(oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st), 0.05, 250, st), st)
    Tl, Rl = oracle.tdf_circle(field, 2.5, 4.0, 1.0)
    if sixteen_bit:                                        # unorm16 TDF buffers, combined as integers
        us, ul = oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)
        m = ul < us
        T = oracle.from_unorm16(np.where(m, us, ul))
    else:
        m = Tl < Ts
        T = np.where(m, Ts, Tl).astype(np.float32)
    R = np.where(m, Rs, Rl).astype(np.float32)
    verts = oracle.centerpoints(T, R, field, 0.35, 3)["vertices"]
    e, l, s = oracle.link_centerpoints(verts, T, 0.3, 10.0)
    cl, rad, _, _ = tsf.centerline_graph(verts, e, l, s, 3, R)
    seg, _ = oracle.segment_inverse_gradient(cl, field, rad)
    return cl, seg


def _validation(cl, seg, real, original):
    """getValidationMeasures (tubeValidation.cpp:17-143): for every extracted
    centerline voxel the real centerline voxels within distance < 4 are
    detected and the nearest one's distance averaged; recall and precision of
    the segmentation against the original tubes."""
    Z, Y, X = cl.shape
    pts = np.argwhere(cl == 1)                             # (z, y, x)
    best = np.full(len(pts), np.inf)
    detected = np.zeros_like(real, dtype=bool)
    for a in range(-4, 5):
        for b in range(-4, 5):
            for c in range(-4, 5):
                d = np.sqrt(float(a * a + b * b + c * c))
                if not d < 4:
                    continue
                nz, ny, nx = pts[:, 0] + c, pts[:, 1] + b, pts[:, 2] + a
                ok = (nx >= 0) & (ny >= 0) & (nz >= 0) & (nx < X) & (ny < Y) & (nz < Z)
                hit = np.zeros(len(pts), bool)
                hit[ok] = real[nz[ok], ny[ok], nx[ok]] == 1
                detected[nz[hit], ny[hit], nx[hit]] = True
                best[hit] = np.minimum(best[hit], d)
    found = np.isfinite(best)
    det = int(detected.sum())
    und = int(((real == 1) & ~detected).sum())
    truth, test = original == 1, seg == 1
    tp, fp, fn = int((truth & test).sum()), int((~truth & test).sum()), int((truth & ~test).sum())
    return {"average_distance": float(best[found].mean()), "percentage_extracted": 100.0 * det / (det + und),
            "recall": tp / (tp + fn), "precision": tp / (tp + fp), "incorrect": int((~found).sum())}


@pytest.mark.parametrize("sixteen_bit", [True, False], ids=["16bit", "32bit"])
def test_synthetic_dataset_quality_gates(oracle, tsf, reference_dir, sixteen_bit):
    d = os.path.join(reference_dir, "tests", "data", "synthetic", "dataset_1")
    if not os.path.exists(os.path.join(d, "noisy0.raw")):
        pytest.skip("the reference's synthetic test data is not present")
    cl, seg = _pipeline(oracle, tsf, _volume(os.path.join(d, "noisy0.raw")), sixteen_bit)
    r = _validation(cl, seg, _volume(os.path.join(d, "real_centerline.raw")), _volume(os.path.join(d, "original.raw")))
    # the reference's thresholds (tubeSegmentationTests.cpp:61-64 and the 32-bit variants)
    assert r["average_distance"] < 1.5, r
    assert r["percentage_extracted"] > 75.0, r
    assert r["precision"] > 0.7, r
    assert r["recall"] > 0.7, r
