"""FP64 GVF residual norms and the GVF that stops on them, against the oracle.

tsf_gvf_residual_norm evaluates, at every voxel's mirrored position, the
per-voxel residual of the reference's kernels in FP32 (kind 0: the Jacobi
update of GVF3DIteration, kernels.cl:1486-1490; kind 1: fmgResidual on the
finest level, kernels.cl:2008-2053) and sums the squares in FP64.  The
per-voxel values are the oracle's bit for bit, so the norms agree up to the
order of the FP64 sums: relative 1e-12 (the max |r| exactly).  The device
sums in a fixed order, so repeated calls give identical bits.
"""
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


def _stored(t, storage):
    a = t.detach().cpu()
    if storage == "snorm16":
        s = a.numpy().astype(np.float32)
        return np.maximum(np.float32(-1.0), s / np.float32(32767.0)).astype(np.float32)
    return a.float().numpy()


def _close(got, want):
    assert np.allclose(got[:4], want[:4], rtol=1e-12, atol=0), (got, want)
    assert got[4] == want[4], (got, want)


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("shape", [(20, 26, 33), (9, 40, 128)])
def test_residual_norm_matches_oracle(torch_dev, tsf, oracle, synth, storage, kind, shape):
    torch = torch_dev
    vol = oracle.blur(synth.vascular_tree(shape, seed=4), 0.5)
    f0, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    v = tsf.gvf(f0, 0.05, 9, storage)
    got = tsf.gvf_residual_norm(f0, v, 0.05, storage, kind)
    want = oracle.gvf_residual_norm(_stored(f0, storage), _stored(v, storage), 0.05, kind)
    _close(got, want)
    again = tsf.gvf_residual_norm(f0, v, 0.05, storage, kind)
    assert np.array_equal(got, again)                       # fixed summation order


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
def test_residual_norm_field4_of_multigrid(torch_dev, tsf, oracle, synth, storage):
    """Field4 layout: the multigrid GVF's input and output images."""
    torch = torch_dev
    vol = oracle.blur(synth.vascular_tree((28, 32, 36), seed=5), 0.5)
    _, f4 = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage, planar=False, field4=True)
    out1 = tsf.gvf_fmg(f4, 0.2, 1, storage)
    out3 = tsf.gvf_fmg(f4, 0.2, 3, storage)
    r1 = tsf.gvf_residual_norm(f4, out1, 0.2, storage, 1, field4=True)
    r3 = tsf.gvf_residual_norm(f4, out3, 0.2, storage, 1, field4=True)
    pl = lambda t: np.moveaxis(_stored(t, storage)[..., :3], -1, 0)
    _close(r3, oracle.gvf_residual_norm(pl(f4), pl(out3), 0.2, 1))
    assert r3[3] < r1[3]                                     # more cycles, smaller residual


def test_jacobi_residual_is_the_update(torch_dev, tsf, synth, oracle):
    """Kind 0 is the next Jacobi update: with FP32 storage its norm equals the
    FP64 norm of v_{k+1} - v_k up to the rounding of v_{k+1}."""
    torch = torch_dev
    vol = oracle.blur(synth.vascular_tree((24, 24, 40), seed=6), 0.5)
    f0, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, "f32")
    v = tsf.gvf(f0, 0.05, 15, "f32")
    w = tsf.gvf(f0, 0.05, 1, "f32", v=v.clone())
    r = tsf.gvf_residual_norm(f0, v, 0.05, "f32", 0)
    d = (w.double() - v.double()).cpu().numpy()
    assert abs(r[3] - np.sqrt((d ** 2).sum())) <= 1e-6 * r[3]


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_converge_stops_on_the_residual(torch_dev, tsf, oracle, synth, storage):
    torch = torch_dev
    vol = oracle.blur(synth.vascular_tree((24, 28, 32), seed=7), 0.5)
    f0, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    n3 = 3 * f0[0].numel()
    r0 = tsf.gvf_residual_norm(f0, f0, 0.05, storage)[3] / np.sqrt(n3)
    tol = r0 / 20
    v, it, rms, code = tsf.gvf_converge(f0, 0.05, 400, 10, tol, storage)
    assert code == 0 and 0 < it <= 400 and it % 10 == 0 and rms <= tol
    # the same iterate as a plain run of that many iterations, and the check
    # before it had not converged
    assert torch.equal(v, tsf.gvf(f0, 0.05, it, storage))
    prev = tsf.gvf_residual_norm(f0, tsf.gvf(f0, 0.05, it - 10, storage), 0.05, storage)[3] / np.sqrt(n3)
    assert prev > tol
    assert abs(rms - tsf.gvf_residual_norm(f0, v, 0.05, storage)[3] / np.sqrt(n3)) == 0.0
    # cap reached: TSF_ERR_NOT_CONVERGED with the last iterate
    v2, it2, rms2, code2 = tsf.gvf_converge(f0, 0.05, 25, 10, 0.0, storage, raise_not_converged=False)
    assert code2 == 5 and it2 == 25 and rms2 > 0
    assert torch.equal(v2, tsf.gvf(f0, 0.05, 25, storage))
