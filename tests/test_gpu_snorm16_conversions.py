"""The device's CL_SNORM_INT16 read and write (kernels_no_3d_write.cl:9-21,
OpenCL 1.1 section 8.3) checked exhaustively through tsf_convert_field:
every one of the 65,536 stored values read as max(-1, s / 32767) with the
division correctly rounded, and FP32 values written as
convert_short_sat_rte(v * 32767) -- round half to even, saturate, NaN -> 0 --
at the rounding boundaries, their neighbours and the special values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_every_stored_value_reads_as_the_rounded_quotient(torch_dev, tsf):
    torch = torch_dev
    s = np.arange(-32768, 32768, dtype=np.int64)
    got = tsf.convert_field(torch.from_numpy(s.astype(np.int16)).cuda(), "snorm16", "f32").cpu().numpy()
    want = np.maximum(np.float32(-1.0), s.astype(np.float32) / np.float32(32767.0))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _write_rule(v):
    f = (v.astype(np.float32) * np.float32(32767.0)).astype(np.float32)
    out = np.zeros(v.shape, np.int64)
    ok = ~np.isnan(f)
    out[ok] = np.clip(np.rint(f[ok].astype(np.float64)), -32768, 32767).astype(np.int64)
    return out.astype(np.int16)


def test_writes_round_half_even_saturate_and_zero_nan(torch_dev, tsf):
    torch = torch_dev
    k = np.arange(-33000, 33000, dtype=np.float64)
    ties = ((k + 0.5) / 32767.0).astype(np.float32)          # near v * 32767 = k + 1/2
    exact = (k / 32767.0).astype(np.float32)
    v = np.concatenate([ties, np.nextafter(ties, np.float32(np.inf)), np.nextafter(ties, np.float32(-np.inf)),
                        exact, np.float32([0.0, -0.0, 1.0, -1.0, 1.0000153, -1.0000153, 1.5, -1.5, 3e38, -3e38,
                                           np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1e-38])]).astype(np.float32)
    got = tsf.convert_field(torch.from_numpy(v).cuda(), "f32", "snorm16").cpu().numpy()
    assert np.array_equal(got, _write_rule(v))
