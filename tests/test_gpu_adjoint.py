"""GPU tests of the hand-written GVF adjoint (tsf_gvf_adjoint).

Checked against (1) autograd of a plain FP64 torch GVF with the same mirror
boundary rule, wrapped in a torch.autograd.Function around the C ABI, and (2)
FP64 central finite differences (h = 1e-4) of the FP64 oracle, on the data
term f0 (random voxels) and on mu.  The adjoint computes in FP32 from FP32
forward states; the tolerance is 1e-4 relative to the largest gradient entry.
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


def _mirror_index(n, torch):
    i = torch.arange(n)
    i = torch.where(i == 0, torch.full_like(i, 2), i)
    return torch.where(i >= n - 1, torch.full_like(i, n - 3), i)


def torch_gvf(f0, mu, K, rounding=None):
    """Plain FP64 torch GVF (kernels.cl:1464-1493 semantics), differentiable.
    rounding: optional storage rounding applied to every iteration's result
    with a straight-through gradient (the adjoint's model of stored states)."""
    import torch
    _, Z, Y, X = f0.shape
    mz, my, mx = (_mirror_index(n, torch).to(f0.device) for n in (Z, Y, X))
    s = (f0 * f0).sum(0)
    v = f0
    for _ in range(K):
        pad = torch.nn.functional.pad(v[None], (1, 1, 1, 1, 1, 1), mode="replicate")[0]
        lap = (pad[:, 1:-1, 1:-1, 2:] + pad[:, 1:-1, 1:-1, :-2] + pad[:, 1:-1, 2:, 1:-1] +
               pad[:, 1:-1, :-2, 1:-1] + pad[:, 2:, 1:-1, 1:-1] + pad[:, :-2, 1:-1, 1:-1] - 6 * v)
        u = v + mu * lap - (v - f0) * s
        v = u[:, mz][:, :, my][:, :, :, mx]
        if rounding is not None:
            v = v + (rounding(v) - v).detach()
    return v


def _rounding(storage):
    import torch
    if storage == "f16":
        return lambda v: v.half().double()
    if storage == "bf16":
        return lambda v: v.to(torch.bfloat16).double()
    return lambda v: torch.clamp(torch.clamp(torch.round(v * 32767.0), -32768, 32767) / 32767.0, min=-1.0)


class GVFFunction:
    """torch.autograd.Function over the C ABI (forward tsf_gvf, backward tsf_gvf_adjoint)."""

    @staticmethod
    def make(tsf):
        import torch

        class _F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, f0, mu, K):
                v = tsf.gvf(f0.contiguous(), float(mu), int(K), "f32")
                ctx.save_for_backward(f0)
                ctx.mu, ctx.K = float(mu), int(K)
                return v

            @staticmethod
            def backward(ctx, gv):
                (f0,) = ctx.saved_tensors
                gf, dmu = tsf.gvf_adjoint(f0, ctx.mu, ctx.K, gv.contiguous().float(), "f32")
                return gf, torch.tensor(dmu, dtype=torch.float64), None

        return _F


def _field(tsf, synth, shape, seed):
    import torch
    vol = synth.vascular_tree(shape, seed=seed)
    b = tsf.blur(torch.from_numpy(vol).cuda(), 0.5)
    f0, _ = tsf.vector_field(b, 0.2, 1, "f32")
    return f0


@pytest.mark.parametrize("shape,K,C", [((16, 18, 20), 12, 0), ((13, 9, 24), 10, 3), ((8, 8, 8), 7, 7),
                                       ((12, 10, 16), 9, 1), ((12, 10, 16), 1, 0), ((12, 10, 16), 8, 20)])
def test_adjoint_matches_fp64_autograd(torch_dev, tsf, synth, shape, K, C):
    """C = 0: sqrt(K) checkpoints; C = 1: every state kept; C = 3: a short
    last segment; C >= K: one segment, all states from the forward pass."""
    torch = torch_dev
    f0 = _field(tsf, synth, shape, 3)
    gv = torch.randn(f0.shape, generator=torch.Generator().manual_seed(1)).float().cuda()
    gf, dmu = tsf.gvf_adjoint(f0, 0.05, K, gv, "f32", checkpoint_every=C)
    # the same through a checkpointed forward whose states the adjoint reuses
    ws = tsf.gvf_adjoint_workspace(f0, K, "f32", C)
    vK = tsf.gvf_checkpointed(f0, 0.05, K, ws, "f32", C)
    assert torch.equal(vK, tsf.gvf(f0, 0.05, K, "f32"))
    gf2, dmu2 = tsf.gvf_adjoint(f0, 0.05, K, gv, "f32", C, ws=ws, checkpoints_stored=True)
    assert torch.equal(gf, gf2) and dmu == dmu2
    assert tsf.gvf_device_error() == 0
    f64 = f0.double().cpu().requires_grad_(True)
    mu64 = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    v = torch_gvf(f64, mu64, K)
    (v * gv.double().cpu()).sum().backward()
    ref = f64.grad.numpy()
    got = gf.cpu().numpy()
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-4 * scale
    assert abs(dmu - mu64.grad.item()) <= 1e-4 * max(1.0, abs(mu64.grad.item()))


@pytest.mark.parametrize("storage", ["f16", "bf16", "snorm16"])
@pytest.mark.parametrize("shape", [(12, 10, 16), (9, 11, 20)])
def test_adjoint_16bit_storage(torch_dev, tsf, synth, storage, shape):
    """16-bit forward states (X = 16: the streaming adjoint kernel; X = 20: the
    vector kernel).  The adjoint treats the storage rounding as the identity;
    the FP64 reference rounds each state to the storage format with a
    straight-through gradient, the same model."""
    torch = torch_dev
    vol = synth.vascular_tree(shape, seed=7)
    b = tsf.blur(torch.from_numpy(vol).cuda(), 0.5)
    f16, _ = tsf.vector_field(b, 0.2, 1, storage)
    K = 9
    gv = torch.randn((3,) + shape, generator=torch.Generator().manual_seed(2)).float().cuda()
    gf, dmu = tsf.gvf_adjoint(f16, 0.05, K, gv, storage, checkpoint_every=3)
    assert tsf.gvf_device_error() == 0
    a = f16.detach().cpu()
    if storage == "snorm16":
        a = torch.clamp(a.float() / 32767.0, min=-1.0)
    f64 = a.double().requires_grad_(True)
    mu64 = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    (torch_gvf(f64, mu64, K, _rounding(storage)) * gv.double().cpu()).sum().backward()
    ref = f64.grad.numpy()
    tol = 1e-3
    assert np.abs(gf.cpu().numpy() - ref).max() <= tol * np.abs(ref).max()
    assert abs(dmu - mu64.grad.item()) <= tol * max(1.0, abs(mu64.grad.item()))


def test_adjoint_matches_fp64_finite_differences(torch_dev, tsf, oracle, synth):
    torch = torch_dev
    shape, K, mu = (12, 14, 16), 9, 0.05
    f0 = _field(tsf, synth, shape, 5)
    rng = np.random.default_rng(2)
    gv = rng.normal(size=(3,) + shape).astype(np.float32)
    gf, dmu = tsf.gvf_adjoint(f0, mu, K, torch.from_numpy(gv).cuda(), "f32")
    gf = gf.cpu().numpy()
    f = f0.cpu().numpy().astype(np.float64)

    def loss(ff, m):
        return float((oracle.gvf_planar(ff, ff, m, K, f64=True) * gv).sum())

    h = 1e-4
    scale = np.abs(gf).max()
    for _ in range(12):
        c, z, y, x = (rng.integers(3), rng.integers(shape[0]), rng.integers(shape[1]), rng.integers(shape[2]))
        fp, fm = f.copy(), f.copy()
        fp[c, z, y, x] += h
        fm[c, z, y, x] -= h
        fd = (loss(fp, mu) - loss(fm, mu)) / (2 * h)
        assert abs(fd - gf[c, z, y, x]) <= 1e-4 * scale
    # mu: the oracle takes mu as a float, so difference between float-representable values
    mp, mm = float(np.float32(mu + 2.0 ** -14)), float(np.float32(mu - 2.0 ** -14))
    fd_mu = (loss(f, mp) - loss(f, mm)) / (mp - mm)
    assert abs(fd_mu - dmu) <= 2e-4 * max(1.0, abs(fd_mu))


def test_autograd_function_wrapper(torch_dev, tsf, synth):
    """The torch.autograd.Function wrapper (test harness only) drives a tiny
    gradient step on mu through the C ABI."""
    torch = torch_dev
    F = GVFFunction.make(tsf)
    f0 = _field(tsf, synth, (10, 12, 14), 7).requires_grad_(True)
    mu = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    v = F.apply(f0, mu, 6)
    loss = (v.double() ** 2).mean()
    loss.backward()
    assert f0.grad is not None and torch.isfinite(f0.grad).all()
    assert mu.grad is not None and np.isfinite(mu.grad.item())
