"""GPU tests of the spline TDF (tsf_tdf_spline) against the oracle, bit for
bit: T (float and unorm16) and R, in every storage format, on a vessel
phantom, a straight tube, odd extents, the presets' radius ranges and an empty
range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STORAGES = ["f32", "f16", "bf16", "snorm16"]


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _to_device_field4(torch, field4, storage):
    if storage == "f32":
        return torch.from_numpy(field4.astype(np.float32)).cuda()
    if storage == "f16":
        return torch.from_numpy(field4.astype(np.float16)).cuda()
    if storage == "bf16":
        return torch.from_numpy(field4.astype(np.float32)).to(torch.bfloat16).cuda()
    s = np.rint(field4.astype(np.float32) * np.float32(32767.0)).clip(-32768, 32767).astype(np.int16)
    return torch.from_numpy(s).cuda()


def _field(oracle, synth, shape, seed, storage, blur=1.0, iters=30):
    vol = oracle.blur(synth.vascular_tree(shape, seed=seed), blur)
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    return oracle.gvf_finish(oracle.gvf(f4, 0.1, iters, storage), storage)


def _check(torch, tsf, oracle, F, storage, rmin, rmax, rstep, unorm):
    d = _to_device_field4(torch, F, storage)
    T, R = tsf.tdf_spline(d, rmin, rmax, rstep, storage=storage, unorm16=unorm)
    Tr, Rr = oracle.tdf_spline(F, rmin, rmax, rstep)
    if unorm:
        assert np.array_equal(T.cpu().numpy().view(np.uint16), oracle.to_unorm16(Tr))
    else:
        assert np.array_equal(T.cpu().numpy(), Tr)
    assert np.array_equal(R.cpu().numpy(), Rr)
    return Tr


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("rng_", [(1.5, 15.0, 0.5), (3.5, 30.0, 1.0)])
def test_spline_bitexact(torch_dev, tsf, oracle, synth, storage, rng_):
    F = _field(oracle, synth, (40, 44, 48), 5, storage)
    for unorm in (False, True):
        Tr = _check(torch_dev, tsf, oracle, F, storage, *rng_, unorm)
    assert (Tr > 0).sum() > 50


@pytest.mark.parametrize("shape", [(37, 29, 45), (4, 5, 6), (20, 24, 33)])
def test_spline_odd_extents(torch_dev, tsf, oracle, synth, shape):
    F = _field(oracle, synth, shape, 7, "f32", blur=0.5, iters=10)
    _check(torch_dev, tsf, oracle, F, "f32", 1.0, 8.0, 0.5, False)


def test_spline_tube_and_empty_range(torch_dev, tsf, oracle):
    Z, Y, X = 24, 40, 40
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    vol = (np.sqrt((xx - 19.5) ** 2 + (yy - 20.0) ** 2) <= 5).astype(np.float32)
    F = oracle.gvf_finish(oracle.gvf(oracle.vector_field(oracle.blur(vol, 1.0), 0.2, 1, "f32"), 0.1, 80, "f32"),
                          "f32")
    Tr = _check(torch_dev, tsf, oracle, F, "f32", 1.5, 15.0, 0.5, False)
    assert Tr.max() > 0.9
    Tr = _check(torch_dev, tsf, oracle, F, "f32", 9.0, 4.0, 0.5, False)       # rmin > rmax
    assert not Tr.any()
    _check(torch_dev, tsf, oracle, F, "f32", 0.5, 60.0, 0.5, False)           # margins beyond the volume
