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


def _write_mhd(path, vol_u8, element="MET_UCHAR"):
    Z, Y, X = vol_u8.shape
    with open(path + ".mhd", "w") as f:
        f.write("ObjectType = Image\nNDims = 3\nDimSize = %d %d %d\nElementType = %s\n"
                "ElementDataFile = %s.raw\n" % (X, Y, Z, element, os.path.basename(path)))
    vol_u8.tofile(path + ".raw")


def _oracle_run(oracle, vol_u8, iters, spline=False, sixteen_bit=True, window=(0.0, 75.0), storage=None):
    """run() with the Synthetic-Vascusynth preset, restated with the oracle
    (spline: the large-radius TDF is the spline TDF from max(1.5, radius-min);
    sixteen_bit False: the 32-bit mode, FP32 fields and a float TDF; window:
    the toFloat limits, the preset's 0 and 75 unless given; storage: the
    fields' format when gvf-storage names one)."""
    lo, hi = np.float32(window[0]), np.float32(window[1])
    v = (np.clip(vol_u8.astype(np.float32), lo, hi) - lo) / (hi - lo)                       # toFloat
    st = storage or ("snorm16" if sixteen_bit else "f32")
    f_small = oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st)                          # small-blur 1.0
    Ts, Rs = oracle.tdf_circle(f_small, 0.5, 3.0, 0.5)
    f4 = oracle.vector_field(oracle.blur(v, 1.0), 0.1, 1, st)                               # large-blur 1.0
    vv = oracle.gvf(f4, 0.05, iters - iters % 2, st)
    field = oracle.gvf_finish(vv, st)
    Tl, Rl = oracle.tdf_spline(field, 1.5, 4.0, 1.0) if spline else oracle.tdf_circle(field, 2.5, 4.0, 1.0)
    if not sixteen_bit:
        m = Tl < Ts
        return np.where(m, Ts, Tl).astype(np.float32), np.where(m, Rs, Rl).astype(np.float32), field
    us, ul = oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)
    m = ul < us
    T16 = np.where(m, us, ul)
    R = np.where(m, Rs, Rl).astype(np.float32)
    return oracle.from_unorm16(T16), R, field


def _read_vtk(path):
    lines = open(path).read().split("\n")
    npts = int(lines[4].split()[1])
    pts = np.array([list(map(int, l.split())) for l in lines[5:5 + npts]], np.int32).reshape(-1, 3)
    k = lines.index("", 5 + npts)
    nl = int(lines[k + 1].split()[1])
    edges = np.array([list(map(int, l.split()))[1:] for l in lines[k + 2:k + 2 + nl]], np.int32).reshape(-1, 2)
    return pts, edges


@pytest.mark.gpu
def test_run_32bit_vectors(api_tests, oracle, synth, tmp_path):
    """run() in the 32-bit mode (32bit-vectors: FP32 fields, a float TDF):
    the TDF and the vertex list equal the oracle's."""
    pytest.importorskip("torch")
    vol_u8 = np.round(synth.vascular_tree((44, 52, 60), seed=11) * 90.0).astype(np.uint8)
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters), "--32bit-vectors", "true",
            "--16bit-vectors", "false", "--no-segmentation", "true"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    T, R, field = _oracle_run(oracle, vol_u8, iters, sixteen_bit=False)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(T.shape)
    assert np.array_equal(tdf, T)
    ref = oracle.centerpoints(T, R, field, tdf_high=0.35, cube_size=3)
    got = np.loadtxt(tmp_path / "vertices.txt", dtype=np.int32).reshape(-1, 3)
    assert len(got) > 20 and np.array_equal(got, ref["vertices"])


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_run_gvf_storage(api_tests, oracle, synth, tmp_path, storage):
    """The gvf-storage parameter (no counterpart in the reference): run() with
    the fields stored in FP16 or BF16 and the 16-bit mode's unorm16 TDF gives
    the oracle's TDF and vertices for that storage."""
    pytest.importorskip("torch")
    vol_u8 = np.round(synth.vascular_tree((44, 52, 60), seed=11) * 90.0).astype(np.uint8)
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters), "--gvf-storage", storage,
            "--no-segmentation", "true"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    T, R, field = _oracle_run(oracle, vol_u8, iters, storage=storage)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(T.shape)
    assert np.array_equal(tdf, T)
    ref = oracle.centerpoints(T, R, field, tdf_high=0.35, cube_size=3)
    got = np.loadtxt(tmp_path / "vertices.txt", dtype=np.int32).reshape(-1, 3)
    assert len(got) > 20 and np.array_equal(got, ref["vertices"])


@pytest.mark.gpu
def test_run_limits_from_the_data(api_tests, oracle, synth, tmp_path):
    """minimum and maximum off: toFloat takes the volume's own limits
    (getLimits, tube-segmentation.cpp:1380-1396), which run() folds over
    several threads' slices of the raw file (a 10 MB MET_FLOAT volume with
    negative values); the TDF equals the oracle's with numpy's min and max."""
    pytest.importorskip("torch")
    vol = synth.vascular_tree((160, 128, 128), seed=13)
    rng = np.random.default_rng(6)
    data = (vol * 90.0 - 20.0 + rng.normal(scale=0.5, size=vol.shape)).astype(np.float32)
    base = str(tmp_path / "vol")
    _write_mhd(base, data, "MET_FLOAT")
    iters = 20
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters), "--minimum", "off", "--maximum", "off",
            "--tdf-only"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    T, _, _ = _oracle_run(oracle, data, iters, window=(float(data.min()), float(data.max())))
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(T.shape)
    assert np.array_equal(tdf, T)
    assert (tdf > 0).any()


@pytest.mark.gpu
def test_run_aaa_preset(api_tests, oracle, synth, tmp_path):
    """run() with the AAA-Vessels-CT preset on an int16 volume (no cropping
    option): the preset's fixed in-plane crop (15 % of x and y per side, then
    multiples of 4; the shift vector stays zero as in the reference), toFloat
    with minimum 50 / maximum 150, blur 2, the vector field (fmax 0.3), the
    multigrid GVF (10 cycles, mu 0.2) and the spline TDF from max(1.5, 3.5) to
    90 in steps of 1, in the 16-bit mode -- the TDF equals the oracle's."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    vol = synth.vascular_tree((40, 64, 72), seed=12)
    hu = np.round(vol * 180.0 + rng.normal(scale=8.0, size=vol.shape)).astype(np.int16)
    base = str(tmp_path / "ct")
    _write_mhd(base, hu, "MET_SHORT")
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "AAA-Vessels-CT",
            "--centerline-method", "gpu", "--tdf-only"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    ox, oy = int(np.floor(72 * np.float32(0.15) + 0.5)), int(np.floor(64 * np.float32(0.15) + 0.5))
    SX, SY, SZ = (72 - 2 * ox) // 4 * 4, (64 - 2 * oy) // 4 * 4, 40
    assert tuple(map(int, open(tmp_path / "size.txt").read().split())) == (SX, SY, SZ)
    assert tuple(map(int, open(tmp_path / "shift.txt").read().split())) == (0, 0, 0)
    crop = np.ascontiguousarray(hu[:SZ, oy:oy + SY, ox:ox + SX])
    v = (np.clip(crop.astype(np.float32), np.float32(50), np.float32(150)) - np.float32(50)) / np.float32(100)
    f4 = oracle.vector_field(oracle.blur(v, 2.0), 0.3, 1, "snorm16")
    field = oracle.fmg_gvf(f4, 0.2, 10, "snorm16")
    T, _ = oracle.tdf_spline(field, 3.5, 90.0, 1.0)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(SZ, SY, SX)
    assert np.array_equal(tdf, oracle.from_unorm16(oracle.to_unorm16(T)))
    assert (tdf > 0).any()


@pytest.mark.gpu
def test_run_lung_preset(api_tests, oracle, tmp_path):
    """run() with the Lung-Airways-CT preset (lung cropping with the "middle"
    z search and 128 minimum scan lines, dark tubes, HU window -1024..-400,
    small blur 0.5, large blur 1, fmax 0.3, 250 GVF iterations) on a chest
    phantom in int16 HU: the crop box and shift vector follow the oracle's
    scan-line counts and the reference's host rule, and the TDF of the cropped
    volume equals the oracle's."""
    pytest.importorskip("torch")
    import test_crop
    import test_gpu_crop
    hu = np.round(test_gpu_crop.chest((200, 200, 360), 2)).astype(np.int16)
    base = str(tmp_path / "chest")
    _write_mhd(base, hu, "MET_SHORT")
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Lung-Airways-CT",
            "--centerline-method", "gpu", "--tdf-only"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    cx, cy, cz = oracle.crop_scan_lines(hu, 1)
    x1, y1, z1, SX, SY, SZ = test_crop.py_crop_bounds(cx, cy, cz, 128, True)
    assert SX < 360 and SY < 200 and SZ < 200
    assert tuple(map(int, open(tmp_path / "size.txt").read().split())) == (SX, SY, SZ)
    assert tuple(map(int, open(tmp_path / "shift.txt").read().split())) == (x1, y1, z1)
    crop = np.ascontiguousarray(hu[z1:z1 + SZ, y1:y1 + SY, x1:x1 + SX])
    v = (np.clip(crop.astype(np.float32), np.float32(-1024), np.float32(-400)) - np.float32(-1024)) / np.float32(624)
    st = "snorm16"
    Ts, Rs = oracle.tdf_circle(oracle.vector_field(oracle.blur(v, 0.5), 0.3, -1, st), 0.5, 3.0, 0.5)
    f4 = oracle.vector_field(oracle.blur(v, 1.0), 0.3, -1, st)
    field = oracle.gvf_finish(oracle.gvf(f4, 0.05, 250, st), st)
    Tl, _ = oracle.tdf_circle(field, 2.5, 15.0, 1.0)
    us, ul = oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)
    T = oracle.from_unorm16(np.where(ul < us, us, ul))
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(SZ, SY, SX)
    assert np.array_equal(tdf, T)


@pytest.mark.gpu
def test_run_spline_tdf(api_tests, oracle, synth, tmp_path):
    """run() with use-spline-tdf: the combined TDF (small-radius circle fit,
    large-radius spline TDF) matches the oracle's, and the pipeline links and
    segments on it."""
    pytest.importorskip("torch")
    vol_u8 = np.round(synth.vascular_tree((44, 52, 60), seed=11) * 90.0).astype(np.uint8)
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters), "--use-spline-tdf", "true"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    T, R, field = _oracle_run(oracle, vol_u8, iters, spline=True)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(T.shape)
    assert np.array_equal(tdf, T)
    ref = oracle.centerpoints(T, R, field, tdf_high=0.35, cube_size=3)
    got = np.loadtxt(tmp_path / "vertices.txt", dtype=np.int32).reshape(-1, 3)
    assert len(got) > 20 and np.array_equal(got, ref["vertices"])
    assert (tmp_path / "segmentation.raw").exists()


@pytest.mark.gpu
def test_run_threshold_cropping(api_tests, oracle, synth, tmp_path):
    """run() with threshold cropping (cropping-start-z end): the vessel tree
    embedded in a dim, larger volume is cropped to the box the oracle's
    scan-line counts and the reference's host rule give, the shift vector is
    the box corner, and the TDF of the cropped volume matches the oracle's."""
    import test_crop
    pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    vol_u8 = (rng.random((60, 70, 84)) * 30).astype(np.uint8)
    vol_u8[7:51, 11:63, 13:73] = np.round(synth.vascular_tree((44, 52, 60), seed=11) * 90.0).astype(np.uint8)
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters), "--tdf-only",
            "--cropping", "threshold", "--cropping-threshold", "60", "--min-scan-lines-threshold", "3"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    cx, cy, cz = oracle.crop_scan_lines(vol_u8, 0, 60.0)
    x1, y1, z1, SX, SY, SZ = test_crop.py_crop_bounds(cx, cy, cz, 3, False)
    assert (SX, SY, SZ) != (84, 70, 60)
    assert tuple(map(int, open(tmp_path / "size.txt").read().split())) == (SX, SY, SZ)
    assert tuple(map(int, open(tmp_path / "shift.txt").read().split())) == (x1, y1, z1)
    cropped = np.ascontiguousarray(vol_u8[z1:z1 + SZ, y1:y1 + SY, x1:x1 + SX])
    T, _, _ = _oracle_run(oracle, cropped, iters)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(SZ, SY, SX)
    assert np.array_equal(tdf, T)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tdf-only", "centerpoints-only", "no-loop-removal", "default", "vtk",
                                  "sphere", "no-segmentation", "timing"])
def test_run_matches_oracle(api_tests, oracle, synth, tmp_path, mode):
    """run() of the Synthetic-Vascusynth preset on an .mhd volume: the TDF,
    the centerpoints and vertices bit for bit against the oracle; without loop
    removal the linked and rasterised trees bit for bit; by default (loop
    removal) the centerlines of the host graph stage applied to the oracle's
    linked graph; with a VTK file, the file's graph rasterises to the
    centerline volume (split vertices may land on existing positions, which
    the reference's position-keyed loop removal merges).  The segmentation
    (inverse gradient, or spheres) of those centerlines bit for bit against
    the oracle, with the radius averaged along the edges after loop removal.
    With the timing parameter: the same results, and one "RUNTIME <stage>:
    <ms> ms" line per stage (the reference's stage names)."""
    pytest.importorskip("torch")
    vol = synth.vascular_tree((44, 52, 60), seed=11)
    vol_u8 = np.round(vol * 90.0).astype(np.uint8)          # some voxels above the preset maximum 75
    base = str(tmp_path / "vol")
    _write_mhd(base, vol_u8)
    iters = 21                                              # odd: the reference runs 20
    args = [api_tests, "run", base + ".mhd", str(tmp_path), "--parameters", "Synthetic-Vascusynth",
            "--centerline-method", "gpu", "--gvf-iterations", str(iters)]
    vtk = str(tmp_path / "centerline.vtk")
    if mode in ("tdf-only", "centerpoints-only"):
        args += ["--" + mode]
    elif mode == "no-loop-removal":
        args += ["--loop-removal", "false"]
    elif mode == "sphere":
        args += ["--loop-removal", "false", "--sphere-segmentation", "true"]
    elif mode == "no-segmentation":
        args += ["--no-segmentation", "true"]
    elif mode == "vtk":
        args += ["--centerline-vtk-file", vtk]
    elif mode == "timing":
        args += ["--timing", "true"]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    runtime = [l for l in out.stdout.splitlines() if l.startswith("RUNTIME ")]
    if mode != "timing":
        assert not runtime
    else:
        stages = [l[len("RUNTIME "):l.rindex(":")] for l in runtime]
        assert stages == ["of reading the dataset", "of data transfer to device", "of cropping",
                          "of to float conversion", "of Create vector field", "of TDF small", "blurring",
                          "Create vector field", "of GVF", "of TDF large", "of combine", "centerpoint extraction",
                          "linking", "of loop removal and centerline voxels (host)", "of removing small trees",
                          "of segmentation"], stages
        for l in runtime:
            assert l.endswith(" ms") and float(l[l.rindex(":") + 1:-3]) >= 0.0
    X, Y, Z = map(int, open(tmp_path / "size.txt").read().split())
    assert (X, Y, Z) == (60, 52, 44)
    tdf = np.fromfile(tmp_path / "tdf.raw", np.float32).reshape(Z, Y, X)
    T, R, field = _oracle_run(oracle, vol_u8, iters)
    assert np.array_equal(tdf, T)
    if mode == "tdf-only":
        assert not (tmp_path / "segmentation.raw").exists()
        return
    ref = oracle.centerpoints(T, R, field, tdf_high=0.35, cube_size=3)
    cl = np.fromfile(tmp_path / "centerline.raw", np.int8).reshape(Z, Y, X)
    if mode == "centerpoints-only":
        assert np.array_equal(cl, ref["mask2"])
        assert not (tmp_path / "segmentation.raw").exists()
        return
    seg_file = tmp_path / "segmentation.raw"
    assert seg_file.exists() == (mode != "no-segmentation")
    seg = np.fromfile(seg_file, np.int8).reshape(Z, Y, X) if seg_file.exists() else None
    got = np.loadtxt(tmp_path / "vertices.txt", dtype=np.int32).reshape(-1, 3)
    assert np.array_equal(got, ref["vertices"])
    # linking, Synthetic-Vascusynth: min-mean-tdf 0.3, max-distance 10, min-tree-length 3
    edges, labels, sizes = oracle.link_centerpoints(ref["vertices"], T, 0.3, 10.0)
    if mode in ("no-loop-removal", "sphere"):
        assert np.array_equal(cl, oracle.rasterize_trees(ref["vertices"], edges, labels, sizes, 3, T.shape))
        if mode == "sphere":
            assert np.array_equal(seg, oracle.segment_spheres(cl, R))
        else:
            ref_seg, _ = oracle.segment_inverse_gradient(cl, field, R)
            assert ref_seg.sum() > cl.sum()
            assert np.array_equal(seg, ref_seg)
        return
    import tsf_gb300 as tsf
    if mode in ("default", "no-segmentation", "timing"):
        ref_cl, rad, _, _ = tsf.centerline_graph(ref["vertices"], edges, labels, sizes, 3, R)
        assert np.array_equal(cl, ref_cl)
        if mode in ("default", "timing"):
            assert np.array_equal(seg, oracle.segment_inverse_gradient(ref_cl, field, rad)[0])
        return
    pts, ve = _read_vtk(vtk)
    assert len(ve) > 0
    import test_centerline_graph as G
    ref_cl, _ = G._raster(pts, ve, np.zeros(T.shape, np.float32))
    assert np.array_equal(cl, ref_cl)
