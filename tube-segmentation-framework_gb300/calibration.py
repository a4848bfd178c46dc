"""Gradient of a TDF loss through the whole hot path, and calibration of a
preset's GVF mu and blur sigma with it.

Forward (the `gpu` method's TDF, reference runCircleFittingMethod,
tube-segmentation.cpp:212-939):
    small pass: f_s = VF(I)              T_s = TDF(f_s; rmin..3, step 0.5)
    large pass: b = blur(I, sigma), f0 = VF(b), v = GVF^K(f0; mu), F = finish(v)
                T_l = TDF(F; max(2.5, rmin)..rmax, rstep)
    T = combine(T_s, T_l)                (the larger response per voxel)
Loss: L = mean((T - G)^2) for a target map G (e.g. a Gaussian centerline map).
Backward: the library's adjoints (tsf_tdf_circle_backward at the forward's
arg-max radii, tsf_gvf_adjoint with memory-budgeted checkpointing,
tsf_vector_field_backward, tsf_blur_backward) give
dL/dI, dL/dmu and dL/dsigma; torch is only the glue (elementwise products and
the combine mask).  FP32 arithmetic; the fields are stored in FP32 or, with
Params.storage, a 16-bit format (the adjoints then treat the rounding as the
identity, straight through).
"""
from __future__ import annotations

import math

import tsf_gb300 as T


class Params:
    """checkpoint_every: GVF adjoint checkpoint interval; 0 = the smallest
    interval whose workspace fits in 60 % of the free device memory (1, no
    recomputation, whenever all states fit), else sqrt(K).  storage: the
    fields' storage format ("f32", "f16", "bf16", "snorm16")."""

    def __init__(self, mu=0.05, sigma=0.5, iterations=300, fmax=0.2, vsign=1, rmin=1.0, rmax=7.0, rstep=0.5,
                 checkpoint_every=0, storage="f32"):
        self.mu, self.sigma, self.iterations = mu, sigma, iterations
        self.fmax, self.vsign = fmax, vsign
        self.rmin, self.rmax, self.rstep = rmin, rmax, rstep
        self.checkpoint_every = checkpoint_every
        self.storage = storage


def forward(vol, p: Params, reuse=None):
    """vol: float32 CUDA tensor [Z, Y, X].  Returns (T, state).  reuse: a
    previous state whose GVF adjoint workspace (possibly ~100 GB) is taken
    over when the size matches, so repeated calls do not allocate."""
    import torch
    st = p.storage
    s = {}
    _, f_s = T.vector_field(vol, p.fmax, p.vsign, st, planar=False, field4=True)
    Ts, Rs = T.tdf_circle(f_s, p.rmin, 3.0, 0.5, st)
    b = T.blur(vol, p.sigma)
    f0, _ = T.vector_field(b, p.fmax, p.vsign, st, planar=True, field4=False)
    ws = None
    if reuse is not None and reuse.get("gvf_ws") is not None and (
            p.checkpoint_every <= 0 or p.checkpoint_every == reuse["checkpoint_every"]):
        C = reuse["checkpoint_every"]
        need = T.load().tsf_gvf_adjoint_workspace_size(*reversed(f0.shape[1:]), T.STORAGE[st], p.iterations, C)
        if reuse["gvf_ws"].numel() >= need:
            ws = reuse.pop("gvf_ws")
    if ws is None:
        C = p.checkpoint_every if p.checkpoint_every > 0 else T.gvf_adjoint_interval(f0, p.iterations, st)
        ws = T.gvf_adjoint_workspace(f0, p.iterations, st, C)
    v = T.gvf_checkpointed(f0, p.mu, p.iterations, ws, st, C)
    F = T.gvf_finish(v, st)
    Tl, Rl = T.tdf_circle(F, max(2.5, p.rmin), p.rmax, p.rstep, st)
    small = Ts > Tl                       # combine (kernels.cl:561-572): T_l < T_s -> take T_s
    Tc = torch.where(small, Ts, Tl)
    s.update(vol=vol, f_s=f_s, b=b, f0=f0, F=F, small=small, gvf_ws=ws, checkpoint_every=C, Ts=Ts, Rs=Rs, Tl=Tl,
             Rl=Rl)
    return Tc, s


def backward(state, gT, p: Params, mark=None):
    """dL/dI (tensor), dL/dmu, dL/dsigma for dL/dT = gT.  mark(name), if
    given, is called after each stage (timing)."""
    import torch
    st = p.storage
    mark = mark or (lambda name: None)
    vol = state["vol"]
    small = state["small"]
    gTs = torch.where(small, gT, torch.zeros_like(gT)).contiguous()
    gTl = torch.where(small, torch.zeros_like(gT), gT).contiguous()
    # small pass -> the un-diffused field of I
    g_fs = T.tdf_backward(state["f_s"], p.rmin, 3.0, 0.5, gTs, st, T=state["Ts"], R=state["Rs"])
    mark("tdf_small_backward")
    gI = T.vector_field_backward(vol, g_fs, p.fmax, p.vsign)
    # large pass -> GVF -> vector field -> blur
    g_v = T.tdf_backward(state["F"], max(2.5, p.rmin), p.rmax, p.rstep, gTl, st, T=state["Tl"], R=state["Rl"])
    mark("tdf_large_backward")
    g_f0, dmu = T.gvf_adjoint(state["f0"], p.mu, p.iterations, g_v, st, state["checkpoint_every"],
                              ws=state["gvf_ws"], checkpoints_stored=True)
    mark("gvf_adjoint")
    g_b = T.vector_field_backward(state["b"], g_f0, p.fmax, p.vsign)
    gI, dsigma = T.blur_backward(vol, g_b, p.sigma, gin=gI)
    mark("vector_field_and_blur_backward")
    return gI, dmu, dsigma


def loss_and_grad(vol, G, p: Params, reuse=None):
    Tc, state = forward(vol, p, reuse)
    n = Tc.numel()
    diff = Tc - G
    L = float((diff.double() ** 2).sum() / n)
    gT = (2.0 / n) * diff
    gI, dmu, dsigma = backward(state, gT.float().contiguous(), p)
    return L, gI, dmu, dsigma, state


def calibrate(vol, G, p: Params, steps=20, lr_mu=0.005, lr_sigma=0.05, log=None):
    """Adam on (mu, sigma) for the loss mean((TDF - G)^2).  mu is kept in the
    stable range (0, 1/12) of the explicit scheme and sigma in [0.25, 5]."""
    b1, b2, eps = 0.9, 0.999, 1e-8
    m = [0.0, 0.0]
    v2 = [0.0, 0.0]
    hist = []
    state = None
    for t in range(1, steps + 1):
        L, _, dmu, dsig, state = loss_and_grad(vol, G, p, state)
        hist.append({"step": t - 1, "loss": L, "mu": p.mu, "sigma": p.sigma, "dmu": dmu, "dsigma": dsig})
        if log:
            log(hist[-1])
        for k, g in enumerate((dmu, dsig)):
            m[k] = b1 * m[k] + (1 - b1) * g
            v2[k] = b2 * v2[k] + (1 - b2) * g * g
        mh = [m[k] / (1 - b1 ** t) for k in range(2)]
        vh = [v2[k] / (1 - b2 ** t) for k in range(2)]
        p.mu = min(max(p.mu - lr_mu * mh[0] / (math.sqrt(vh[0]) + eps), 1e-3), 1.0 / 12 - 1e-3)
        p.sigma = min(max(p.sigma - lr_sigma * mh[1] / (math.sqrt(vh[1]) + eps), 0.25), 5.0)
    L, _, _, _, _ = loss_and_grad(vol, G, p, state)
    hist.append({"step": steps, "loss": L, "mu": p.mu, "sigma": p.sigma})
    return p, hist
