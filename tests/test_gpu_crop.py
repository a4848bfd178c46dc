"""GPU tests of the cropping stage against the oracle, bit for bit: the
per-slice scan-line counts of tsf_crop_scan_lines (cropDatasetThreshold,
cropDatasetLung; kernels.cl:813-946) for every raw type, extents that are not
multiples of the kernels' tiles, and the crop copy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RAW = {"u8": (np.uint8, 0), "i8": (np.int8, 1), "u16": (np.uint16, 2), "i16": (np.int16, 3), "f32": (np.float32, 4)}


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def chest(shape, seed, noise=25.0):
    """Slabs of air (-1000 HU), body (+40) and two lungs (-850), noise 25 HU.
    At the nominal extents (Z 200, X 360) the z-columns through a lung read
    air 35, body 35, lung 70, body 40, air 20 and the x-rows through both
    lungs air 40, wall 40, lung 70, mediastinum 60, lung 70, wall 40, air 40:
    runs longer than the 30-voxel limit, so the lung scan lines count.  The
    lungs span the middle two thirds of y."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    zf = np.arange(Z)[:, None, None] / Z * 200.0
    yf = np.arange(Y)[None, :, None] / Y
    xf = np.arange(X)[None, None, :] / X * 360.0
    body = (zf >= 35) & (zf < 180) & (xf >= 40) & (xf < 320)
    lung = (zf >= 70) & (zf < 140) & (yf >= 1 / 6) & (yf < 5 / 6) & (((xf >= 80) & (xf < 150)) |
                                                                    ((xf >= 210) & (xf < 280)))
    hu = np.where(body, np.where(lung, -850.0, 40.0), -1000.0) + rng.normal(scale=noise, size=shape)
    return hu.astype(np.float32)


def _as_raw(hu, kind):
    dt, _ = RAW[kind]
    if kind == "u16":
        return np.clip(hu + 1024, 0, 65535).astype(np.uint16)
    if kind == "u8":
        return np.clip((hu + 1024) / 8, 0, 255).astype(np.uint8)
    if kind == "i8":
        return np.clip(hu / 8, -128, 127).astype(np.int8)
    if kind == "i16":
        return np.clip(hu, -32768, 32767).astype(np.int16)
    return hu.astype(np.float32)


def _device(torch, a, kind):
    if kind == "u16":
        return torch.from_numpy(a.view(np.int16)).cuda()
    return torch.from_numpy(a).cuda()


@pytest.mark.parametrize("kind", list(RAW))
@pytest.mark.parametrize("shape", [(200, 48, 360), (70, 33, 161), (5, 7, 3)])
def test_scan_lines_bitexact(torch_dev, tsf, oracle, kind, shape):
    torch = torch_dev
    raw = _as_raw(chest(shape, sum(shape)), kind)
    d = _device(torch, raw, kind)
    thr = {"u8": 100.0, "i8": -60.0, "u16": 900.0, "i16": -200.0, "f32": -200.5}[kind]
    methods = [0] if kind == "f32" else [0, 1]
    for m in methods:
        got = tsf.crop_scan_lines(d, m, thr, raw_type=RAW[kind][1])
        want = oracle.crop_scan_lines(raw, m, thr)
        for g, w in zip(got, want):
            assert np.array_equal(g.cpu().numpy(), w)
    if shape == (200, 48, 360) and kind in ("i16", "u16"):
        cx, cy, cz = oracle.crop_scan_lines(raw, 1)
        assert cx.max() > 0 and cz.max() > 0          # the lung state machine fires


def test_lung_rejects_float(torch_dev, tsf):
    torch = torch_dev
    v = torch.zeros((8, 8, 8), dtype=torch.float32, device="cuda")
    with pytest.raises(tsf.TSFError, match="lung cropping"):
        tsf.crop_scan_lines(v, 1)


@pytest.mark.parametrize("kind", list(RAW))
def test_crop_copy(torch_dev, tsf, kind):
    torch = torch_dev
    raw = _as_raw(chest((37, 45, 67), 3), kind)
    d = _device(torch, raw, kind)
    for box in [(3, 5, 7, 40, 28, 20), (0, 0, 0, 67, 45, 37), (66, 44, 36, 1, 1, 1)]:
        x1, y1, z1, SX, SY, SZ = box
        out = tsf.crop_copy(d, box, raw_type=RAW[kind][1]).cpu().numpy()
        if kind == "u16":
            out = out.view(np.uint16)
        assert np.array_equal(out, raw[z1:z1 + SZ, y1:y1 + SY, x1:x1 + SX])
    with pytest.raises(tsf.TSFError):
        tsf.crop_copy(d, (60, 0, 0, 8, 4, 4), raw_type=RAW[kind][1])


def test_crop_pipeline_box(torch_dev, tsf, oracle):
    """Counts on the GPU, box on the host: the lung cropping of the chest
    phantom keeps the lungs (all but their last y row: the reference's end
    slice is exclusive) and drops the air."""
    torch = torch_dev
    shape = (200, 48, 360)
    raw = _as_raw(chest(shape, 9), "i16")
    d = _device(torch, raw, "i16")
    cx, cy, cz = (c.cpu().numpy() for c in tsf.crop_scan_lines(d, 1))
    box = tsf.crop_bounds(cx, cy, cz, 5, True)
    x1, y1, z1, SX, SY, SZ = box
    assert all(s % 4 == 0 for s in box[3:])
    assert SX < shape[2] and SY < shape[1]
    zz, yy, xx = np.nonzero(chest(shape, 9, noise=0.0) == -850.0)
    inside = (xx >= x1) & (xx < x1 + SX) & (yy >= y1) & (yy < y1 + SY) & (zz >= z1) & (zz < z1 + SZ)
    assert inside.mean() > 0.95
    assert SX * SY * SZ < 0.5 * raw.size
