"""tsf_gvf_static: the GVF entry point for callers that cannot allocate.

Some hosts can neither call cudaMalloc nor hand the library a workspace (a
plug-in host that owns the device allocator, a real-time pipeline that
forbids device allocation once running).  tsf_gvf_static keeps its scratch in
a fixed array inside the library.  These tests call it through the C ABI and
check that it returns exactly what tsf_gvf returns (the same tolerance as the
other GVF parity tests: bit-identical), on two calls in a row with different
inputs, so state left by the first call cannot leak into the second.  The
file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _field(torch, tsf, synth, shape, seed, storage):
    vol = synth.vascular_tree(shape, seed=seed)
    g = tsf.blur(torch.from_numpy(vol).cuda(), 0.5)
    f0, _ = tsf.vector_field(g, 0.2, 1, storage)
    return f0


def _static(torch, tsf, f0, mu, iters, storage):
    _, Z, Y, X = f0.shape
    v = f0.clone()
    code = tsf.load().tsf_gvf_static(tsf._ptr(f0), tsf._ptr(v), X, Y, Z, C.c_float(mu), iters,
                                     tsf.STORAGE[storage], tsf._stream())
    tsf._check(code)
    return v


@pytest.mark.parametrize("storage,shapes", [
    ("f16", [(64, 64, 64), (40, 52, 36)]),
    ("f32", [(48, 40, 36), (33, 21, 26)]),
])
def test_static_scratch_matches_workspace_gvf(torch_dev, tsf, synth, storage, shapes):
    torch = torch_dev
    for k, shape in enumerate(shapes):            # two calls in a row
        f0 = _field(torch, tsf, synth, shape, 20 + k, storage)
        tsf.load().tsf_gvf_device_error(1)
        got = _static(torch, tsf, f0, 0.05, 13, storage)
        torch.cuda.synchronize()
        # a copy that timed out in the streaming kernel shows here, not only as a mismatch
        assert tsf.load().tsf_gvf_device_error(1) == 0
        ref = tsf.gvf(f0, 0.05, 13, storage)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)


def test_static_scratch_rejects_oversize(torch_dev, tsf):
    L = tsf.load()
    code = L.tsf_gvf_static(None, None, 257, 256, 256, C.c_float(0.05), 3, tsf.STORAGE["f16"], None)
    assert code == 6
    assert b"too large" in L.tsf_last_error_string()
