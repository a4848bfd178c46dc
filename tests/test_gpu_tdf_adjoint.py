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


def _smooth_fd(f, h):
    """Central difference of the scalar function f at 0, or None where f is not
    smooth on [-2h, 2h] (a stopping decision or an eigenvector sign of the
    reference's procedure changes there).  Smooth means the slopes and the
    curvatures measured at steps h and 2h agree; a jump or a kink inside the
    interval breaks one of them by O(jump / h) or O(kink)."""
    f0, fp, fm, fp2, fm2 = f(0.0), f(h), f(-h), f(2 * h), f(-2 * h)
    d1 = (fp - fm) / (2 * h)
    d2 = (fp2 - fm2) / (4 * h)
    c1 = (fp + fm - 2 * f0) / (h * h)
    c2 = (fp2 + fm2 - 2 * f0) / (4 * h * h)
    noise = 1e-13 * max(1.0, abs(f0)) / (h * h)          # FP64 rounding of the five values
    if abs(d1 - d2) > 1e-4 * max(abs(d1), 1e-6):
        return None
    if abs(c1 - c2) > 0.05 * max(abs(c1), abs(c2)) + noise:
        return None
    return d1


@pytest.mark.parametrize("rng_", [(2.5, 7.0, 0.5), (1.0, 3.0, 0.5)])
def test_tdf_backward_directional(torch_dev, tsf, oracle, synth, rng_):
    """dT(x)/d(field) along random directions, one voxel at a time.  Voxels
    next to a face are skipped: there the mirror rule makes a Hessian row
    exactly zero and the reference's eigenvector signs jump."""
    torch = torch_dev
    field = _gvf_field(oracle, synth, (20, 22, 24), 3)
    if rng_[1] < 4:                          # small pass: un-normalised Hessian, w = 1
        field[..., 3] = 1.0
    f64 = _with_norm_w(field) if rng_[1] >= 4 else field.astype(np.float64)
    T0, _ = oracle.tdf_circle(f64, *rng_, f64=True)
    d4 = torch.from_numpy(f64.astype(np.float32)).cuda()
    rng = np.random.default_rng(4)
    inner = np.zeros(T0.shape, bool)
    inner[2:-2, 2:-2, 2:-2] = True
    cand = np.argwhere((T0 > 0.05) & inner)
    checked, bad = 0, []
    for t in range(16):
        z, y, x = cand[rng.integers(len(cand))]
        gT = np.zeros(T0.shape, np.float32)
        gT[z, y, x] = 1.0
        gT_d = torch.from_numpy(gT).cuda()
        g = tsf.tdf_backward(d4, *rng_, gT_d).cpu().numpy()
        # the same at the forward's arg-max radius, without repeating the sweep
        Tf, Rf = tsf.tdf_circle(d4, *rng_, storage="f32")
        g2 = tsf.tdf_backward(d4, *rng_, gT_d, T=Tf, R=Rf).cpu().numpy()
        assert np.allclose(g, g2, rtol=1e-5, atol=1e-7 * np.abs(g).max())
        g = np.moveaxis(g, 0, -1).astype(np.float64)
        D = rng.normal(size=f64.shape[:3] + (3,))

        def T_at(h):
            f = f64.copy()
            f[..., :3] += h * D
            if rng_[1] >= 4:
                f = _with_norm_w(f)
            return float(oracle.tdf_circle(f, *rng_, f64=True)[0][z, y, x])

        fd = _smooth_fd(T_at, 1e-6)
        if fd is None:
            continue
        checked += 1
        an = float((g * D).sum())
        if abs(fd - an) > 2e-3 * max(abs(fd), 1e-3):
            bad.append(((z, y, x), fd, an))
    assert checked >= 6, checked
    assert not bad, bad


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


@pytest.mark.parametrize("sigma", [0.7, 1.3])
def test_blur_backward_directional(torch_dev, tsf, oracle, synth, sigma):
    """The mask width m = ceil(sigma / 0.5) jumps at multiples of 0.5, so sigma
    is checked inside a constant-width interval."""
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
    """dL/dmu of the whole chain (both TDF passes, GVF, vector field, blur)
    against an FP64 central difference, for a loss on interior voxels whose
    response is smooth in mu."""
    torch = torch_dev
    import calibration as CAL
    shape = (20, 20, 24)
    vol, truth = synth.vascular_tree(shape, seed=8, with_truth=True)
    G = synth.centerline_gaussian(shape, truth["points"], 1.0)
    p = CAL.Params(mu=0.05, sigma=0.7, iterations=16)
    Tc, state = CAL.forward(torch.from_numpy(vol).cuda(), p)
    T = Tc.cpu().numpy()
    inner = np.zeros(shape, bool)
    inner[2:-2, 2:-2, 2:-2] = True
    rng = np.random.default_rng(3)
    cand = np.argwhere((T > 0.1) & inner)
    sel = cand[rng.choice(len(cand), size=min(12, len(cand)), replace=False)]
    mask = np.zeros(shape, bool)
    mask[tuple(sel.T)] = True
    gT = np.where(mask, 2.0 * (T - G), 0.0).astype(np.float32)
    _, dmu, _ = CAL.backward(state, torch.from_numpy(gT).cuda(), p)

    def Lo(dm):
        mu = float(np.float32(0.05 + dm))
        To = _oracle_pipeline_T(oracle, vol, mu, 0.7, 16)
        return float(((To - G) ** 2)[mask].sum())

    for e in (16, 18, 20):                  # the largest step with no decision change inside
        fd = _smooth_fd(Lo, 2.0 ** -e)
        if fd is not None:
            break
    assert fd is not None
    assert abs(fd - dmu) <= 0.01 * abs(fd) + 1e-7, (fd, dmu)


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
