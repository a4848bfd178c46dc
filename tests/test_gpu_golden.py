"""GPU path against golden vectors of the reference's own kernel text.

tests/golden/reference_{f32,snorm16}.npz hold the outputs of kernels.cl
(smistad/Tube-Segmentation-Framework) compiled for the CPU under an OpenCL C
shim and driven in the order of the reference's host code
(tests/golden/make_golden.py).  Here the same volume runs through
libtsf_gb300's C ABI -- blur, both vector fields, 20 GVF iterations, finish,
both TDF passes, combine, the candidate stage -- and every stage must equal
the reference's bits (tolerance 0), in the reference's two field formats
(CL_FLOAT with a float TDF, CL_SNORM_INT16 with the unorm16 TDF of its 16-bit
mode).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _np(t):
    a = t.detach().cpu().numpy()
    return a


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
def test_gpu_matches_reference_golden(torch_dev, tsf, storage):
    torch = torch_dev
    d = np.load(os.path.join(GOLDEN, "reference_%s.npz" % storage))
    P = dict(zip([str(k) for k in d["param_names"]], d["params"]))
    unorm = storage == "snorm16"
    vol = torch.from_numpy(d["volume"]).cuda()
    b = tsf.blur(vol, P["sigma"])
    assert np.array_equal(_np(b), d["blurred"])
    p, f4 = tsf.vector_field(b, P["fmax"], int(P["vsign"]), storage, planar=True, field4=True)
    assert np.array_equal(_np(f4), d["field"])
    _, fs = tsf.vector_field(vol, P["fmax"], int(P["vsign"]), storage, planar=False, field4=True)
    assert np.array_equal(_np(fs), d["field_small"])
    v = tsf.gvf(p, P["mu"], int(P["iterations"]), storage)
    assert np.array_equal(_np(v), d["gvf"])
    fin = tsf.gvf_finish(v, storage)
    assert np.array_equal(_np(fin), d["gvf_field"])
    Ts, Rs = tsf.tdf_circle(fs, 1.0, 3.0, 0.5, storage=storage, unorm16=unorm)
    Tl, Rl = tsf.tdf_circle(fin, 2.5, 7.0, 0.5, storage=storage, unorm16=unorm)
    Tt = (lambda t: _np(t).view(np.uint16)) if unorm else _np
    assert np.array_equal(Tt(Ts), d["T_small"]) and np.array_equal(_np(Rs), d["R_small"])
    tsf.tdf_combine(Ts, Rs, Tl, Rl, unorm16=unorm)
    assert np.array_equal(Tt(Tl), d["T"]) and np.array_equal(_np(Rl), d["R"])
    out = tsf.candidates(Tl, Rl, fin, storage, P["tdf_high"], int(P["cube"]), unorm16=unorm,
                         want_centerpoints=True, want_candidates=True, raise_on_range=False)
    assert np.array_equal(_np(out["candidates"]), d["candidates"])
    assert np.array_equal(_np(out["centerpoints"]), d["mask2"])
    assert np.array_equal(_np(out["vertices"]), d["vertices"])
