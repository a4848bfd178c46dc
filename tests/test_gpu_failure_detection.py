"""Failure detection of the streaming GVF kernel, without a GPU fault.

Every barrier wait of gvf_zs_kernel is bounded: a shared-memory copy that
has not landed within the limit is treated as lost -- the kernel records it
in a device error word, stops and returns, instead of spinning.  Here the
wait is made to run out on purpose (tsf_gvf_wait_selftest: one launch with
every copy suppressed and a 1 ms limit, so the barriers are never armed) and
the test checks that the error bit is reported, that it is cleared by the
read, and that the device is still usable: a normal GVF run right after it
gives the oracle's bits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.mark.parametrize("storage", ["f16", "f32", "snorm16"])
def test_bounded_wait_reports_and_recovers(torch_dev, tsf, oracle, synth, storage):
    torch = torch_dev
    shape = (40, 16, 64)
    vol = oracle.blur(synth.vascular_tree(shape, seed=9), 0.5)
    f0, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    v = f0.clone()
    L = tsf.load()
    ws = tsf.workspace(L.tsf_gvf_workspace_size(64, 16, 40, tsf.STORAGE[storage]))
    assert tsf.gvf_device_error() == 0
    word = L.tsf_gvf_wait_selftest(tsf._ptr(f0), tsf._ptr(v), 64, 16, 40, tsf.STORAGE[storage], 2_000_000,
                                   tsf._ptr(ws), ws.numel(), tsf._stream())
    assert word >= 0, L.tsf_last_error_string()
    assert word & 1, "the timed-out waits were not reported"
    assert tsf.gvf_device_error() == 0                       # the self-test read cleared it
    # the context is intact: a normal run matches the oracle
    got = tsf.gvf(f0, 0.05, 7, storage)
    want = oracle.gvf(oracle.vector_field(vol, 0.2, 1, storage), 0.05, 7, storage)
    a = got.cpu()
    a = np.maximum(np.float32(-1), a.numpy().astype(np.float32) / np.float32(32767)) if storage == "snorm16" \
        else a.float().numpy()
    assert np.array_equal(a, want)
    assert tsf.gvf_device_error() == 0


def test_selftest_rejects_what_the_kernel_cannot_run(torch_dev, tsf):
    torch = torch_dev
    L = tsf.load()
    f0 = torch.zeros((3, 8, 8, 33), dtype=torch.float16, device="cuda")     # 66-byte rows
    v = f0.clone()
    ws = tsf.workspace(3 * 8 * 8 * 33 * 2)
    r = L.tsf_gvf_wait_selftest(tsf._ptr(f0), tsf._ptr(v), 33, 8, 8, tsf.STORAGE["f16"], 1000, tsf._ptr(ws),
                                ws.numel(), tsf._stream())
    assert r == -1 and b"cannot run" in L.tsf_last_error_string()
