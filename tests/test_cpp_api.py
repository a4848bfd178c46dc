"""The drop-in C++ API (run / runSegmentation, TSFOutput, paramList).

CPU: the C++ driver's parameter, TSFOutput and I/O-error checks, mirroring the
reference's tests/parameterTests.cpp, tests/TSFOutputTests.cpp and
tests/tubeSegmentationTests.cpp:4-7.

GPU: run() on an .mhd/.raw volume with the Synthetic-Vascusynth preset (the
preset of the reference's system test), compared with the oracle running the
same stages in the same order: toFloat, small-blur field and small-radius TDF,
large-blur field, GVF (snorm16 storage, the reference's 16-bit mode), the
large-radius TDF, combine, the unorm16 TDF read back as u / 65535, and the
candidate stage.
"""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def api_tests(tsf):
    import build as tsf_build
    return tsf_build.API_TESTS


def test_cpp_api_cpu_checks(api_tests):
    out = subprocess.run([api_tests, "cpu"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert " 0 failures" in out.stdout


def _write_mhd(path, vol_u8):
    Z, Y, X = vol_u8.shape
    with open(path + ".mhd", "w") as f:
        f.write("ObjectType = Image\nNDims = 3\nDimSize = %d %d %d\nElementType = MET_UCHAR\n"
                "ElementDataFile = %s.raw\n" % (X, Y, Z, os.path.basename(path)))
    vol_u8.tofile(path + ".raw")


def _oracle_run(oracle, vol_u8, iters):
    """run() with the Synthetic-Vascusynth preset, restated with the oracle."""
    v = np.clip(vol_u8.astype(np.float32), np.float32(0), np.float32(75)) / np.float32(75)   # toFloat
    st = "snorm16"
    f_small = oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st)                          # small-blur 1.0
    Ts, Rs = oracle.tdf_circle(f_small, 0.5, 3.0, 0.5)
    f4 = oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st)                               # large-blur 1.0
    vv = oracle.gvf(f4, 0.05, iters - iters % 2, st)
    field = oracle.gvf_finish(vv, st)
    Tl, Rl = oracle.tdf_circle(field, 2.5, 4.0, 1.0)
    us, ul = oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)
    m = ul < us
    T16 = np.where(m, us, ul)
    R = np.where(m, Rs, Rl).astype(np.float32)
    return oracle.from_unorm16(T16), R, field


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tdf-only", "centerpoints-only", "vertices"])
def test_run_matches_oracle(api_tests, oracle, synth, tmp_path, mode):
    pytest.importorskip("torch")
    vol = synth.vascular_tree((44, 52, 60), seed=11)
    vol_u8 = np.round(vol * 90.0).astype(np.uint8)          # some voxels above the preset maximum 75
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21                                              # odd: the reference runs 20
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters)]
    if mode != "vertices":
        args += ["--" + mode]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    X, Y, Z = map(int, open(tmp_path / "size.txt").read().split())
    assert (X, Y, Z) == (60, 52, 44)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(Z, Y, X)
    T, R, field = _oracle_run(oracle, vol_u8, iters)
    assert np.array_equal(tdf, T)
    if mode == "tdf-only":
        return
    ref = oracle.centerpoints(T, R, field, tdf_high=0.35, cube_size=3)
    cl = np.fromfile(tmp_path / "centerline.raw", np.int8).reshape(Z, Y, X)
    if mode == "centerpoints-only":
        assert np.array_equal(cl, ref["mask2"])
    else:
        got = np.loadtxt(tmp_path / "vertices.txt", dtype=np.int32).reshape(-1, 3)
        assert np.array_equal(got, ref["vertices"])
        assert cl.sum() == len(ref["vertices"])
