"""Parity at the benchmark workloads' full sizes.

The other GPU parity tests use small shapes and few iterations.  These run
the whole hot path -- blur, vector field, small-radius TDF on the un-diffused
field, GVF, finish, large-radius TDF, combine and the candidate stage up to
the vertex list -- at the sizes the benchmark measures:

* the 128^3 vessel tree with 250 GVF iterations, FP32 and FP16 storage;
* the 256^3 vessel tree with 500 GVF iterations, FP16 storage (the
  benchmark's headline workload);

through the C ABI, and compare with the float oracle on the same volume:
stored GVF field, TDF response, radius and vertex list must be identical bit
for bit (tolerance 0).  mu is 0.05, the benchmark's value: at mu = 0.1 the
explicit scheme diverges on these volumes (tests/test_oracle_pins.py).

A third test states the accuracy of the GPU path against the FP64 oracle
run of the same method on the 128^3 workload -- the figures the benchmark
description asks for -- and asserts them: TDF mean absolute error <= 1e-3 in
every format; FP32: the FP64 vertex list exactly and Dice 1 for the linked
centerline and the segmentation; 16-bit: segmentation Dice >= 0.995.
The reference gates its own results only end to end
(tests/tubeSegmentationTests.cpp:41-99: centerline distance, precision,
recall); these are the stage-level counterparts.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P = dict(large_blur=0.5, fmax=0.2, vsign=1, rmin=1.0, rmax=7.0, rstep=0.5, tdf_high=0.5, cube_size=4)
MU = 0.05


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _oracle_path(O, vol, storage, iters, f64=False):
    """The float (or FP64) oracle run of the hot path: field4, planar v,
    combined T and R, vertex list."""
    b = O.blur(vol, P["large_blur"], f64=f64)
    f4 = O.vector_field(b, P["fmax"], P["vsign"], storage, f64=f64)
    v = O.gvf(f4, MU, iters, storage, f64=f64)
    field = O.gvf_finish(v, storage, f64=f64)
    src = vol.astype(np.float64) if f64 else vol
    fs = O.vector_field(src, P["fmax"], P["vsign"], storage, f64=f64)
    Ts, Rs = O.tdf_circle(fs, P["rmin"], 3.0, 0.5, f64=f64)
    Tl, Rl = O.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"], f64=f64)
    T, R = O.combine(Ts, Rs, Tl, Rl, f64=f64)
    verts = O.centerpoints(T, R, field, P["tdf_high"], P["cube_size"], f64=f64)["vertices"]
    return field, v, T, R, verts


def _gpu_path(torch, tsf, vol, storage, iters):
    """The same path on the GPU through the C ABI (paired texels for the
    16-bit TDF, as the benchmark runs it)."""
    Z, Y, X = vol.shape
    g = torch.from_numpy(vol).cuda()
    b = tsf.blur(g, P["large_blur"])
    _, fs = tsf.vector_field(g, P["fmax"], P["vsign"], storage, planar=False, field4=True)
    ws = tsf.workspace(tsf.load().tsf_tdf_workspace_size(X, Y, Z, tsf.STORAGE[storage]))
    Ts, Rs = tsf.tdf_circle(fs, P["rmin"], 3.0, 0.5, storage=storage, ws=ws)
    f0, _ = tsf.vector_field(b, P["fmax"], P["vsign"], storage)
    tsf.gvf_device_error()
    v = tsf.gvf(f0, MU, iters, storage)
    field = tsf.gvf_finish(v, storage)
    Tl, Rl = tsf.tdf_circle(field, max(2.5, P["rmin"]), P["rmax"], P["rstep"], storage=storage, ws=ws)
    tsf.tdf_combine(Ts, Rs, Tl, Rl)
    out = tsf.candidates(Tl, Rl, field, storage, P["tdf_high"], P["cube_size"], raise_on_range=False)
    torch.cuda.synchronize()
    assert tsf.gvf_device_error() == 0
    assert out["status"] == 0
    return field, v, Tl, Rl, out["vertices"].cpu().numpy()


def _stored(t, storage):
    a = t.detach().cpu()
    if storage == "snorm16":
        s = a.numpy().astype(np.float32)
        return np.maximum(np.float32(-1.0), s / np.float32(32767.0)).astype(np.float32)
    return a.float().numpy()


def _assert_same(torch, tsf, oracle, synth, n, iters, storage):
    vol = synth.vascular_tree((n, n, n), seed=0)
    field, v, T, R, verts = _gpu_path(torch, tsf, vol, storage, iters)
    ofield, ov, oT, oR, overts = _oracle_path(oracle, vol, storage, iters)
    assert np.array_equal(_stored(v, storage), ov), "GVF field differs from the oracle"
    assert np.array_equal(_stored(field, storage), ofield), "finished field differs from the oracle"
    assert np.array_equal(T.cpu().numpy(), oT), "TDF differs from the oracle"
    assert np.array_equal(R.cpu().numpy(), oR), "TDF radius differs from the oracle"
    assert len(overts) >= 8
    assert np.array_equal(verts, overts), "vertex list differs from the oracle"


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_vessel_tree_128_250_iterations(torch_dev, tsf, oracle, synth, storage):
    _assert_same(torch_dev, tsf, oracle, synth, 128, 250, storage)


def test_vessel_tree_256_500_iterations_f16(torch_dev, tsf, oracle, synth):
    _assert_same(torch_dev, tsf, oracle, synth, 256, 500, "f16")


def _dice(a, b):
    return 2.0 * float(np.logical_and(a, b).sum()) / max(1.0, float(a.sum() + b.sum()))


def test_accuracy_against_fp64_128(torch_dev, tsf, oracle, synth):
    """GPU path vs the FP64 oracle run of the same method (128^3, 250
    iterations).  Linking (Synthetic-Vascusynth: min-mean-tdf 0.3,
    max-distance 10, min-tree-length 3) and the inverse-gradient
    segmentation follow on each side."""
    torch = torch_dev
    n, iters = 128, 250
    shape = (n, n, n)
    vol = synth.vascular_tree(shape, seed=0)
    field64, _, T64, R64, V64 = _oracle_path(oracle, vol, "f32", iters, f64=True)
    e64, l64, s64 = oracle.link_centerpoints(V64, T64.astype(np.float32), 0.3, 10.0)
    cl64 = oracle.rasterize_trees(V64, e64, l64, s64, 3, shape) != 0
    seg64, _ = oracle.segment_inverse_gradient(cl64.astype(np.int8), field64.astype(np.float32),
                                               R64.astype(np.float32))
    seg64 = seg64 != 0
    report = {}
    for storage in ("f32", "f16", "snorm16"):
        field, _, T, R, verts = _gpu_path(torch, tsf, vol, storage, iters)
        dT = np.abs(T.cpu().numpy().astype(np.float64) - T64)
        dv = torch.from_numpy(verts).cuda().contiguous()
        edges, labels, sizes = tsf.link_centerpoints(dv, T, 0.3, 10.0)
        cl = tsf.rasterize_trees(dv, edges, labels, sizes, 3, shape)
        seg, _ = tsf.segment_inverse_gradient(cl, field, R, storage=storage)
        cl, seg = cl.cpu().numpy() != 0, seg.cpu().numpy() != 0
        report[storage] = dict(tdf_mean=float(dT.mean()), tdf_p999=float(np.quantile(dT, 0.999)),
                               same_vertices=bool(np.array_equal(verts, V64)), vertices=len(verts),
                               fp64_vertices=len(V64), centerline_dice=_dice(cl, cl64),
                               segmentation_dice=_dice(seg, seg64))
    print("accuracy vs FP64 (128^3, 250 iterations):", report)
    for st, r in report.items():
        assert r["tdf_mean"] <= 1e-3, (st, r)
        assert r["segmentation_dice"] >= 0.995, (st, r)
    assert report["f32"]["same_vertices"], report["f32"]
    assert report["f32"]["centerline_dice"] == 1.0 and report["f32"]["segmentation_dice"] == 1.0
