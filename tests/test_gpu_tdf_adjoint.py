"""GPU tests of the TDF, vector-field and blur adjoints and of the whole
gradient chain (calibration.py), against FP64 central finite differences of
the FP64 oracle.

The TDF is piecewise smooth (the sweep's arg-max and stopping radius change
at ties), so derivatives are checked along random directions with a small
step, where crossing a tie is improbable, and the agreement bar is a relative
error of the directional derivative.  The adjoints compute in FP32.
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


def _gvf_field(oracle, synth, shape, seed, iters=20):
    vol = synth.vascular_tree(shape, seed=seed)
    f4 = oracle.vector_field(oracle.blur(vol, 0.5), 0.2, 1, "f32")
    v = oracle.gvf(f4, 0.05, iters, "f32")
    return oracle.gvf_finish(v, "f32")


def _with_norm_w(field4):
    """FP64 field whose w is exactly |v| (1 where 0), the model of the adjoint."""
    f = field4.astype(np.float64).copy()
    l = np.sqrt((f[..., :3] ** 2).sum(-1))
    f[..., 3] = np.where(l > 0, l, 1.0)
    return f


@pytest.mark.parametrize("rng_", [(2.5, 7.0, 0.5), (1.0, 3.0, 0.5)])
def test_tdf_backward_directional(torch_dev, tsf, oracle, synth, rng_):
    torch = torch_dev
    field = _gvf_field(oracle, synth, (20, 22, 24), 3)
    if rng_[1] < 4:                          # small pass: un-normalised Hessian, w = 1
        field[..., 3] = 1.0
    f64 = _with_norm_w(field) if rng_[1] >= 4 else field.astype(np.float64)
    T0, _ = oracle.tdf_circle(f64, *rng_, f64=True)
    rng = np.random.default_rng(4)
    gT = (rng.normal(size=T0.shape) * (T0 > 0)).astype(np.float32)
    d4 = torch.from_numpy(f64.astype(np.float32)).cuda()
    g = tsf.tdf_backward(d4, *rng_, torch.from_numpy(gT).cuda()).cpu().numpy().astype(np.float64)
    rels = []
    for trial in range(3):
        D = rng.normal(size=(3,) + T0.shape)
        h = 1e-6

        def L(sign):
            f = f64.copy()
            f[..., :3] += sign * h * np.moveaxis(D, 0, -1)
            if rng_[1] >= 4:
                f = _with_norm_w(f)
            T, _ = oracle.tdf_circle(f, *rng_, f64=True)
            return float((T * gT).sum())

        fd = (L(1) - L(-1)) / (2 * h)
        an = float((g * D).sum())
        rels.append(abs(fd - an) / max(abs(fd), 1e-12))
    assert sorted(rels)[1] < 2e-3, rels          # median of three directions


def test_vector_field_backward_directional(torch_dev, tsf, oracle, synth):
    torch = torch_dev
    vol = oracle.blur(synth.vascular_tree((18, 20, 22), seed=5), 1.0).astype(np.float64)
    rng = np.random.default_rng(5)
    gf = rng.normal(size=(3,) + vol.shape).astype(np.float32)
    gin = tsf.vector_field_backward(torch.from_numpy(vol.astype(np.float32)).cuda(),
                                    torch.from_numpy(gf).cuda(), 0.2, -1).cpu().numpy()
    D = rng.normal(size=vol.shape)
    h = 1e-6

    def L(sign):
        f = oracle.vector_field(vol + sign * h * D, 0.2, -1, "f32", f64=True)
        return float((np.moveaxis(f[..., :3], -1, 0) * gf).sum())

    fd = (L(1) - L(-1)) / (2 * h)
    an = float((gin.astype(np.float64) * D).sum())
    assert abs(fd - an) <= 1e-4 * abs(fd)


@pytest.mark.parametrize("sigma", [0.5, 1.3])
def test_blur_backward_directional(torch_dev, tsf, oracle, synth, sigma):
    torch = torch_dev
    vol = synth.vascular_tree((14, 16, 18), seed=6).astype(np.float32)
    rng = np.random.default_rng(6)
    gb = rng.normal(size=vol.shape).astype(np.float32)
    gin, dsig = tsf.blur_backward(torch.from_numpy(vol).cuda(), torch.from_numpy(gb).cuda(), sigma)
    gin = gin.cpu().numpy().astype(np.float64)
    # the blur is linear in I: exact transposition check
    D = rng.normal(size=vol.shape).astype(np.float32)
    lhs = float((oracle.blur(D, sigma, f64=True) * gb).sum())
    assert abs(lhs - float((gin * D).sum())) <= 1e-4 * max(1.0, abs(lhs))
    # sigma: analytic mask derivative vs a central difference of the FP64 mask
    h = 1e-3

    def L(s):
        m, mask = oracle.blur_mask(s)
        S = 2 * m + 1
        return float((_blur64(vol, mask.astype(np.float64).reshape(S, S, S), m) * gb).sum())

    fd = (L(sigma + h) - L(sigma - h)) / (2 * h)
    assert abs(fd - dsig) <= 2e-3 * max(1.0, abs(fd))


def _blur64(vol, k, m):
    Z, Y, X = vol.shape
    p = np.pad(vol.astype(np.float64), m, mode="edge")
    out = np.zeros(vol.shape)
    for c in range(2 * m + 1):
        for b in range(2 * m + 1):
            for a in range(2 * m + 1):
                out += k[c, b, a] * p[c:c + Z, b:b + Y, a:a + X]
    return out


def _oracle_pipeline_T(oracle, vol, mu, sigma, iters):
    """FP64 oracle of calibration.forward."""
    vol = vol.astype(np.float64)
    fs = oracle.vector_field(vol, 0.2, 1, "f32", f64=True)
    Ts, _ = oracle.tdf_circle(fs, 1.0, 3.0, 0.5, f64=True)
    b = oracle.blur(vol.astype(np.float32), sigma, f64=True)
    f4 = oracle.vector_field(b, 0.2, 1, "f32", f64=True)
    v = oracle.gvf(f4, mu, iters, f64=True)
    F = oracle.gvf_finish(v, f64=True)
    Tl, _ = oracle.tdf_circle(F, 2.5, 7.0, 0.5, f64=True)
    return np.where(Tl < Ts, Ts, Tl)


def test_pipeline_gradient_mu(torch_dev, tsf, oracle, synth):
    """dL/dmu of the whole chain against an FP64 central difference."""
    torch = torch_dev
    import calibration as CAL
    shape = (20, 20, 24)
    vol, truth = synth.vascular_tree(shape, seed=8, with_truth=True)
    G = synth.centerline_gaussian(shape, truth["points"], 1.0)
    p = CAL.Params(mu=0.05, sigma=0.5, iterations=16)
    L, gI, dmu, dsig = CAL.loss_and_grad(torch.from_numpy(vol).cuda(), torch.from_numpy(G).cuda(), p)
    hm = 2.0 ** -12

    def Lo(mu):
        T = _oracle_pipeline_T(oracle, vol, mu, 0.5, 16)
        return float(((T - G) ** 2).mean())

    mp, mm = float(np.float32(0.05 + hm)), float(np.float32(0.05 - hm))
    fd = (Lo(mp) - Lo(mm)) / (mp - mm)
    assert abs(fd - dmu) <= 0.02 * abs(fd) + 1e-9, (fd, dmu)
    assert np.isfinite(gI.cpu().numpy()).all()


def test_calibration_reduces_loss(torch_dev, tsf, synth):
    """A few Adam steps on (mu, sigma) lower the centerline loss."""
    torch = torch_dev
    import calibration as CAL
    shape = (32, 32, 32)
    vol, truth = synth.vascular_tree(shape, seed=9, with_truth=True)
    G = synth.centerline_gaussian(shape, truth["points"], 1.0)
    p = CAL.Params(mu=0.02, sigma=1.5, iterations=30)
    p, hist = CAL.calibrate(torch.from_numpy(vol).cuda(), torch.from_numpy(G).cuda(), p, steps=6)
    assert hist[-1]["loss"] < hist[0]["loss"]
