"""Python binding of libtsf_gb300 (ctypes over include/tsf/tsf_c.h).

Test and benchmark harness: torch supplies device memory and streams; every
computation runs in the library's CUDA kernels.  There is no CPU fallback --
loading fails loudly when the library is missing or no GPU is present.

Arrays follow the library's layout: volumes are torch tensors indexed
[z, y, x] (x fastest in memory); planar fields are [3, z, y, x]; field4 images
are [z, y, x, 4]; storage dtypes are float32, float16, bfloat16 or int16
(snorm16).
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", "libtsf_gb300.so")
HEADER = os.path.join(ROOT, "include", "tsf", "tsf_c.h")

TSF_OK = 0
ERRORS = {1: "TSF_ERR_INVALID_ARG", 2: "TSF_ERR_CUDA", 3: "TSF_ERR_WORKSPACE",
          4: "TSF_ERR_COUNT_RANGE", 5: "TSF_ERR_NOT_CONVERGED", 6: "TSF_ERR_CAPACITY"}
STORAGE = {"f32": 0, "f16": 1, "bf16": 2, "snorm16": 3}


class TSFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (no GPU needed to load it)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"libtsf_gb300 not built: {path} missing (run __graft_entry__.build())")
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def declared_symbols(header: str = HEADER):
    """Function names declared in the C header."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tsf_[a-z0-9_]+)\s*\(", txt)))


_p, _i, _i64, _f, _sz = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_size_t


def _declare(L):
    sig = {
        "tsf_abi_version": (_i, []),
        "tsf_last_error_string": (C.c_char_p, []),
        "tsf_storage_bytes": (_sz, [_i]),
        "tsf_kernel_launches": (C.c_ulonglong, []),
        "tsf_blur_mask": (_i, [_f, _p, _p]),
        "tsf_to_float": (_i, [_p, _i, _i64, _f, _f, _p, _p]),
        "tsf_blur": (_i, [_p, _p, _i, _i, _i, _f, _p]),
        "tsf_vector_field": (_i, [_p, _i, _i, _i, _f, _i, _i, _p, _p, _p]),
        "tsf_gvf_workspace_size": (_sz, [_i, _i, _i, _i]),
        "tsf_gvf": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _p, _sz, _p]),
        "tsf_gvf_mode": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _p, _sz, _i, _p]),
        "tsf_gvf_device_error": (_i, [_i]),
        "tsf_link_workspace_size": (_sz, [_i]),
        "tsf_link_centerpoints": (_i, [_p, _i, _p, _i, _i, _i, _i, _f, _f, _p, _p, _p, _p, _p, _sz, _p]),
        "tsf_rasterize_trees": (_i, [_p, _p, _i, _p, _p, _i, _p, _i, _i, _i, _p]),
        "tsf_crop_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_crop_scan_lines": (_i, [_p, _i, _i, _i, _i, _i, _f, _p, _p, _sz, _p]),
        "tsf_crop_bounds": (_i, [_p, _i, _i, _i, _i, _i, _p]),
        "tsf_crop_box_fixed": (_i, [_i, _i, _i, _f, _p]),
        "tsf_crop_copy": (_i, [_p, _i, _i, _i, _i, _p, _p, _p]),
        "tsf_segment_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_segment_inverse_gradient": (_i, [_p, _p, _i, _p, _i, _i, _i, _p, _p, _p, _sz, _p]),
        "tsf_segment_spheres": (_i, [_p, _p, _i, _i, _i, _p, _p]),
        "tsf_remove_loops": (_i, [_p, _i, _p, _i, _i, _i, _i, _p, _p, _i, _p, _p]),
        "tsf_centerline_graph": (_i, [_p, _i, _p, _i, _p, _p, _i, _i, _i, _i, _i, _p, _p, _p, _p, _i, _p, _p]),
        "tsf_write_centerline_vtk": (_i, [C.c_char_p, _p, _i, _p, _i]),
        "tsf_centerline_graph_cells": (_i, [_p, _i, _p, _i, _p, _p, _i, _i, _i, _i, _i, _p, _p, _i, _p, _p, _p, _p,
                                            _i64, _p]),
        "tsf_centerline_smooth_radius": (_i, [_p, _p, _i, _p, _p, _p, _p]),
        "tsf_gather_cells": (_i, [_p, _i, _i, _i, _p, _i64, _p, _p]),
        "tsf_centerline_apply": (_i, [_p, _p, _i, _i, _i, _p, _p, _i64, _p]),
        "tsf_gvf_adjoint_checkpoint_interval": (_i, [_i, _i, _i, _i, _i, _sz]),
        "tsf_gvf_finish": (_i, [_p, _p, _i, _i, _i, _i, _p]),
        "tsf_gvf_static": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _p]),
        "tsf_gvf_adjoint_workspace_size": (_sz, [_i, _i, _i, _i, _i, _i]),
        "tsf_gvf_adjoint": (_i, [_p, _i, _i, _i, _f, _i, _i, _p, _p, _p, _i, _i, _p, _sz, _p]),
        "tsf_gvf_checkpointed": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _i, _p, _sz, _p]),
        "tsf_tdf_backward_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_tdf_circle_backward": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _p, _p, _p, _p, _sz, _p]),
        "tsf_vector_field_backward": (_i, [_p, _p, _i, _i, _i, _f, _i, _p, _p]),
        "tsf_blur_backward_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_blur_backward": (_i, [_p, _p, _i, _i, _i, _f, _p, _p, _p, _sz, _p]),
        "tsf_tdf_circle": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _i, _p, _p]),
        "tsf_tdf_workspace_size": (_sz, [_i, _i, _i, _i]),
        "tsf_tdf_circle_ws": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _i, _p, _p, _sz, _p]),
        "tsf_tdf_spline": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _i, _p, _p]),
        "tsf_tdf_combine": (_i, [_p, _p, _p, _p, _i64, _i, _p]),
        "tsf_tdf_circle_mode": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _i, _p, _i, _p]),
        "tsf_candidates_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_candidates": (_i, [_p, _i, _p, _p, _i, _i, _i, _i, _f, _i, _p, _i64, _p, _p, _i64,
                                _p, _p, _p, _sz, _p]),
        "tsf_compact_workspace_size": (_sz, [_i, _i, _i]),
        "tsf_compact_mask": (_i, [_p, _i, _i, _i, _p, _i64, _p, _p, _sz, _p]),
        "tsf_gvf_fmg_workspace_size": (_sz, [_i, _i, _i, _i]),
        "tsf_gvf_one_component_workspace_size": (_sz, [_i, _i, _i, _i]),
        "tsf_gvf_one_component": (_i, [_p, _i, _i, _i, _f, _i, _i, _p, _p, _sz, _p]),
        "tsf_gvf_fmg": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _p, _sz, _p]),
        "tsf_gvf_wait_selftest": (_i, [_p, _p, _i, _i, _i, _i, C.c_longlong, _p, _sz, _p]),
        "tsf_tdf_circle_ex": (_i, [_p, _i, _i, _i, _i, _f, _f, _f, _p, _p, _i, _p, _p, _sz, _p]),
        "tsf_convert_field": (_i, [_p, _i, _p, _i, _i64, _p]),
        "tsf_gvf_residual_workspace_size": (_sz, []),
        "tsf_gvf_residual_norm": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, _i, _p, _p, _sz, _p]),
        "tsf_gvf_converge_workspace_size": (_sz, [_i, _i, _i, _i]),
        "tsf_gvf_converge": (_i, [_p, _p, _i, _i, _i, _f, _i, _i, C.c_double, _i, _p, _p, _p, _sz, _p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args


def kernel_launches() -> int:
    return int(load().tsf_kernel_launches())


def gvf_device_error(clear: bool = True) -> int:
    """The streaming GVF kernel's device error word (0 = none); raises if it
    cannot be read."""
    v = int(load().tsf_gvf_device_error(int(clear)))
    if v < 0:
        raise TSFError(2, load().tsf_last_error_string().decode())
    return v


def _check(code):
    if code != TSF_OK:
        raise TSFError(code, load().tsf_last_error_string().decode())


# ---------------------------------------------------------------------------
# torch helpers (imported lazily so that loading the library needs no torch)
# ---------------------------------------------------------------------------

def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("libtsf_gb300 computes on the GPU only; no CUDA device is available")
    return torch


def storage_dtype(storage: str):
    import torch
    return {"f32": torch.float32, "f16": torch.float16, "bf16": torch.bfloat16,
            "snorm16": torch.int16}[storage]


def _ptr(t):
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "device tensors must be contiguous CUDA tensors"
    return C.c_void_p(t.data_ptr())


def _stream(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dims(vol):
    Z, Y, X = vol.shape[:3]
    return int(X), int(Y), int(Z)


def workspace(nbytes: int):
    torch = _torch()
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")


# ---------------------------------------------------------------------------
# stage wrappers
# ---------------------------------------------------------------------------

def blur_mask(sigma: float):
    import numpy as np
    buf = np.zeros(11 ** 3, np.float32)
    m = C.c_int(0)
    _check(load().tsf_blur_mask(float(sigma), buf.ctypes.data_as(C.c_void_p), C.byref(m)))
    return m.value, buf[: (2 * m.value + 1) ** 3].copy()


def blur(vol, sigma: float, out=None, stream=None):
    torch = _torch()
    out = torch.empty_like(vol) if out is None else out
    X, Y, Z = _dims(vol)
    _check(load().tsf_blur(_ptr(vol), _ptr(out), X, Y, Z, float(sigma), _stream(stream)))
    return out


def vector_field(vol, fmax: float, vsign: int = 1, storage: str = "f32", planar=True, field4=False,
                 stream=None):
    torch = _torch()
    X, Y, Z = _dims(vol)
    dt = storage_dtype(storage)
    p = torch.empty((3, Z, Y, X), dtype=dt, device=vol.device) if planar else None
    f4 = torch.empty((Z, Y, X, 4), dtype=dt, device=vol.device) if field4 else None
    _check(load().tsf_vector_field(_ptr(vol), X, Y, Z, float(fmax), int(vsign), STORAGE[storage],
                                   _ptr(p), _ptr(f4), _stream(stream)))
    return p, f4


def gvf(f0, mu: float, iterations: int, storage: str = "f32", v=None, ws=None, mode: int = 0,
        stream=None):
    """Runs `iterations` Jacobi iterations; v (planar) defaults to a copy of f0."""
    _, Z, Y, X = f0.shape
    L = load()
    v = f0.clone() if v is None else v
    need = L.tsf_gvf_workspace_size(X, Y, Z, STORAGE[storage])
    ws = workspace(need) if ws is None else ws
    _check(L.tsf_gvf_mode(_ptr(f0), _ptr(v), X, Y, Z, float(mu), int(iterations), STORAGE[storage],
                          _ptr(ws), ws.numel(), int(mode), _stream(stream)))
    return v


def gvf_residual_norm(f0, v, mu: float, storage: str = "f32", kind: int = 0, field4: bool = False, stream=None):
    """FP64 residual norms (tsf_gvf_residual_norm): [|r_x|, |r_y|, |r_z|, |r|,
    max |r|].  f0, v planar (3, Z, Y, X), or field4 (Z, Y, X, 4) when field4;
    kind 0 = the Jacobi update, 1 = the multigrid residual."""
    import numpy as np
    layout = 1 if field4 else 0
    Z, Y, X = (v.shape[:3] if layout else v.shape[1:])
    L = load()
    ws = workspace(L.tsf_gvf_residual_workspace_size())
    out = np.zeros(5, np.float64)
    _check(L.tsf_gvf_residual_norm(_ptr(f0), _ptr(v), X, Y, Z, float(mu), STORAGE[storage], int(kind), layout,
                                   out.ctypes.data_as(C.c_void_p), _ptr(ws), ws.numel(), _stream(stream)))
    return out


def gvf_converge(f0, mu: float, max_iterations: int, check_every: int, tolerance: float, storage: str = "f32",
                 v=None, stream=None, raise_not_converged=True):
    """tsf_gvf_converge: Jacobi iterations until the RMS of the next update is
    <= tolerance (checked every check_every iterations).  Returns (v,
    iterations run, last RMS, status)."""
    _, Z, Y, X = f0.shape
    L = load()
    v = f0.clone() if v is None else v
    ws = workspace(L.tsf_gvf_converge_workspace_size(X, Y, Z, STORAGE[storage]))
    it, rms = C.c_int(0), C.c_double(0.0)
    code = L.tsf_gvf_converge(_ptr(f0), _ptr(v), X, Y, Z, float(mu), int(max_iterations), int(check_every),
                              float(tolerance), STORAGE[storage], C.byref(it), C.byref(rms), _ptr(ws), ws.numel(),
                              _stream(stream))
    if code != TSF_OK and (raise_not_converged or code != 5):
        _check(code)
    return v, it.value, rms.value, code


def gvf_adjoint_interval(f0, iterations: int, storage: str = "f32", budget_bytes: int = None) -> int:
    """Smallest checkpoint interval whose adjoint workspace fits budget_bytes
    (default: 60 % of the device memory free now); 0 means the default
    sqrt(K) interval."""
    if budget_bytes is None:
        free, _ = _torch().cuda.mem_get_info(f0.device)
        budget_bytes = int(0.6 * free)
    _, Z, Y, X = f0.shape
    return int(load().tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, STORAGE[storage], int(iterations),
                                                          int(budget_bytes)))


def gvf_adjoint_workspace(f0, iterations: int, storage: str = "f32", checkpoint_every: int = 0):
    _, Z, Y, X = f0.shape
    return workspace(load().tsf_gvf_adjoint_workspace_size(X, Y, Z, STORAGE[storage], int(iterations),
                                                           int(checkpoint_every)))


def gvf_checkpointed(f0, mu: float, iterations: int, ws, storage: str = "f32", checkpoint_every: int = 0,
                     stream=None):
    """Forward GVF (result returned) keeping the adjoint's checkpoints in ws."""
    _, Z, Y, X = f0.shape
    v = f0.clone()
    _check(load().tsf_gvf_checkpointed(_ptr(f0), _ptr(v), X, Y, Z, float(mu), int(iterations), STORAGE[storage],
                                       int(checkpoint_every), _ptr(ws), ws.numel(), _stream(stream)))
    return v


def gvf_adjoint(f0, mu: float, iterations: int, gv, storage: str = "f32", checkpoint_every: int = 0,
                ws=None, checkpoints_stored: bool = False, stream=None):
    """dL/df0 (planar float32) and dL/dmu for L with dL/dv_K = gv."""
    torch = _torch()
    _, Z, Y, X = f0.shape
    L = load()
    ws = gvf_adjoint_workspace(f0, iterations, storage, checkpoint_every) if ws is None else ws
    gf = torch.empty((3, Z, Y, X), dtype=torch.float32, device=f0.device)
    dmu = C.c_double(0.0)
    _check(L.tsf_gvf_adjoint(_ptr(f0), X, Y, Z, float(mu), int(iterations), STORAGE[storage], _ptr(gv), _ptr(gf),
                             C.byref(dmu), int(checkpoint_every), 1 if checkpoints_stored else 0, _ptr(ws),
                             ws.numel(), _stream(stream)))
    return gf, dmu.value


def tdf_backward(field4, rmin, rmax, rstep, gT, storage: str = "f32", gfield=None, T=None, R=None, stream=None):
    """Adds dL/d(field xyz) (planar float32) for dL/dT = gT; returns gfield.
    T, R: the forward's float response and radius (the sweep is then not
    repeated)."""
    torch = _torch()
    Z, Y, X = field4.shape[:3]
    L = load()
    gfield = torch.zeros((3, Z, Y, X), dtype=torch.float32, device=field4.device) if gfield is None else gfield
    ws = workspace(L.tsf_tdf_backward_workspace_size(X, Y, Z))
    _check(L.tsf_tdf_circle_backward(_ptr(field4), X, Y, Z, STORAGE[storage], float(rmin), float(rmax), float(rstep),
                                     _ptr(gT), _ptr(T), _ptr(R), _ptr(gfield), _ptr(ws), ws.numel(),
                                     _stream(stream)))
    return gfield


def vector_field_backward(vol, gf, fmax, vsign=1, gin=None, stream=None):
    torch = _torch()
    X, Y, Z = _dims(vol)
    gin = torch.zeros_like(vol) if gin is None else gin
    _check(load().tsf_vector_field_backward(_ptr(vol), _ptr(gf), X, Y, Z, float(fmax), int(vsign), _ptr(gin),
                                            _stream(stream)))
    return gin


def blur_backward(vol, gout, sigma, gin=None, stream=None):
    torch = _torch()
    X, Y, Z = _dims(vol)
    L = load()
    gin = torch.zeros_like(vol) if gin is None else gin
    ws = workspace(L.tsf_blur_backward_workspace_size(X, Y, Z))
    ds = C.c_double(0.0)
    _check(L.tsf_blur_backward(_ptr(vol), _ptr(gout), X, Y, Z, float(sigma), _ptr(gin), C.byref(ds), _ptr(ws),
                               ws.numel(), _stream(stream)))
    return gin, ds.value


def gvf_finish(v, storage: str = "f32", out=None, stream=None):
    torch = _torch()
    _, Z, Y, X = v.shape
    out = torch.empty((Z, Y, X, 4), dtype=v.dtype, device=v.device) if out is None else out
    _check(load().tsf_gvf_finish(_ptr(v), _ptr(out), X, Y, Z, STORAGE[storage], _stream(stream)))
    return out


class TdfOptions(C.Structure):
    """tsf_tdf_options (include/tsf/tsf_c.h)."""
    _fields_ = [("samples", C.c_int), ("stride", C.c_int), ("eigen", C.c_int), ("kernel", C.c_int)]


def tdf_circle(field4, rmin, rmax, rstep, storage: str = "f32", unorm16: bool = False, mode: int = 0,
               stream=None, ws=None, samples: int = None, stride: int = 1, eigen: int = None):
    """Circle-fitting TDF.  ws: a workspace of tsf_tdf_workspace_size bytes
    (tsf_tdf_circle_ws: paired texels for 16-bit storage); mode forces the
    kernel (tsf_tdf_circle_mode) when ws is None.  samples / stride / eigen
    given: tsf_tdf_circle_ex with those options (mode as its kernel)."""
    torch = _torch()
    Z, Y, X = field4.shape[:3]
    T = torch.empty((Z, Y, X), dtype=torch.int16 if unorm16 else torch.float32, device=field4.device)
    R = torch.empty((Z, Y, X), dtype=torch.float32, device=field4.device)
    if samples is not None or eigen is not None:
        opt = TdfOptions(32 if samples is None else int(samples), int(stride), 0 if eigen is None else int(eigen),
                         int(mode))
        _check(load().tsf_tdf_circle_ex(_ptr(field4), X, Y, Z, STORAGE[storage], float(rmin), float(rmax),
                                        float(rstep), C.byref(opt), _ptr(T), int(unorm16), _ptr(R),
                                        _ptr(ws) if ws is not None else None, ws.numel() if ws is not None else 0,
                                        _stream(stream)))
        return T, R
    if ws is not None:
        _check(load().tsf_tdf_circle_ws(_ptr(field4), X, Y, Z, STORAGE[storage], float(rmin), float(rmax),
                                        float(rstep), _ptr(T), int(unorm16), _ptr(R), _ptr(ws), ws.numel(),
                                        _stream(stream)))
        return T, R
    _check(load().tsf_tdf_circle_mode(_ptr(field4), X, Y, Z, STORAGE[storage], float(rmin), float(rmax),
                                      float(rstep), _ptr(T), int(unorm16), _ptr(R), int(mode), _stream(stream)))
    return T, R


def tdf_spline(field4, rmin, rmax, rstep, storage: str = "f32", unorm16: bool = False, stream=None):
    """splineTDF with runSplineTDF's constants: (T, R) on the device."""
    torch = _torch()
    Z, Y, X = field4.shape[:3]
    T = torch.empty((Z, Y, X), dtype=torch.int16 if unorm16 else torch.float32, device=field4.device)
    R = torch.empty((Z, Y, X), dtype=torch.float32, device=field4.device)
    _check(load().tsf_tdf_spline(_ptr(field4), X, Y, Z, STORAGE[storage], float(rmin), float(rmax), float(rstep),
                                 _ptr(T), int(unorm16), _ptr(R), _stream(stream)))
    return T, R


def link_centerpoints(vertices, T, min_mean_tdf: float, max_distance: float, unorm16: bool = False, stream=None):
    """vertices: (n, 3) int32 CUDA tensor (x, y, z); T: the TDF (float32, or
    int16-typed unorm16 bits).  Returns (edges (m, 2) int32 in the 2-D pyramid
    order, labels (n,), tree sizes (n,))."""
    torch = _torch()
    L = load()
    n = vertices.shape[0]
    Z, Y, X = T.shape
    edges = torch.zeros((2 * n, 2), dtype=torch.int32, device=T.device)
    labels = torch.empty(n, dtype=torch.int32, device=T.device)
    sizes = torch.empty(n, dtype=torch.int32, device=T.device)
    ws = workspace(L.tsf_link_workspace_size(n))
    ne = C.c_int(0)
    _check(L.tsf_link_centerpoints(_ptr(vertices), n, _ptr(T), int(unorm16), X, Y, Z, float(min_mean_tdf),
                                   float(max_distance), _ptr(edges), C.byref(ne), _ptr(labels), _ptr(sizes),
                                   _ptr(ws), ws.numel(), _stream(stream)))
    return edges[:ne.value], labels, sizes


def rasterize_trees(vertices, edges, labels, sizes, min_tree_length: int, shape, stream=None):
    torch = _torch()
    Z, Y, X = shape
    out = torch.zeros(shape, dtype=torch.int8, device=vertices.device)
    e = edges.contiguous()
    _check(load().tsf_rasterize_trees(_ptr(vertices), _ptr(e) if e.numel() else None, e.shape[0], _ptr(labels),
                                      _ptr(sizes), int(min_tree_length), _ptr(out), X, Y, Z, _stream(stream)))
    return out


def _raw_type(t):
    torch = _torch()
    return {torch.uint8: 0, torch.int8: 1, torch.int16: 3, torch.float32: 4}[t.dtype]


def crop_scan_lines(vol, method: int, threshold: float = 0.0, raw_type: int = None, stream=None):
    """cropDatasetThreshold (method 0) / cropDatasetLung (method 1) on a raw
    CUDA volume (Z, Y, X): (counts_x, counts_y, counts_z) int16.  raw_type
    overrides the type taken from the dtype (2 = uint16 data held in an int16
    tensor)."""
    torch = _torch()
    L = load()
    Z, Y, X = vol.shape
    rt = _raw_type(vol) if raw_type is None else raw_type
    counts = torch.empty(X + Y + Z, dtype=torch.int16, device=vol.device)
    ws = workspace(L.tsf_crop_workspace_size(X, Y, Z))
    _check(L.tsf_crop_scan_lines(_ptr(vol), rt, X, Y, Z, int(method), float(threshold), _ptr(counts), _ptr(ws),
                                 ws.numel(), _stream(stream)))
    return counts[:X], counts[X:X + Y], counts[X + Y:]


def crop_bounds(cx, cy, cz, min_scan_lines: int, start_z_middle: bool):
    """Host crop box (x1, y1, z1, SX, SY, SZ) from numpy int16 counts."""
    import numpy as np
    c = np.ascontiguousarray(np.concatenate([cx, cy, cz]), dtype=np.int16)
    box = (C.c_int * 6)()
    _check(load().tsf_crop_bounds(_np_ptr(c), len(cx), len(cy), len(cz), int(min_scan_lines), int(start_z_middle),
                                  box))
    return tuple(box)


def crop_box_fixed(shape, fraction: float):
    Z, Y, X = shape
    box = (C.c_int * 6)()
    _check(load().tsf_crop_box_fixed(X, Y, Z, float(fraction), box))
    return tuple(box)


def crop_copy(vol, box, raw_type: int = None, stream=None):
    torch = _torch()
    Z, Y, X = vol.shape
    x1, y1, z1, SX, SY, SZ = box
    out = torch.empty((SZ, SY, SX), dtype=vol.dtype, device=vol.device)
    b = (C.c_int * 6)(*box)
    _check(load().tsf_crop_copy(_ptr(vol), _raw_type(vol) if raw_type is None else raw_type, X, Y, Z, b, _ptr(out),
                                _stream(stream)))
    return out


def segment_inverse_gradient(centerlines, field4, radius, storage: str = "f32", stream=None):
    """runInverseGradientSegmentation: centerlines (Z, Y, X) int8, field4
    (Z, Y, X, 4) in `storage`'s dtype, radius (Z, Y, X) float32, all CUDA.
    Returns (segmentation int8, grow iterations)."""
    torch = _torch()
    L = load()
    Z, Y, X = centerlines.shape
    out = torch.empty((Z, Y, X), dtype=torch.int8, device=centerlines.device)
    ws = workspace(L.tsf_segment_workspace_size(X, Y, Z))
    it = C.c_int(0)
    _check(L.tsf_segment_inverse_gradient(_ptr(centerlines), _ptr(field4), STORAGE[storage], _ptr(radius), X, Y, Z,
                                          _ptr(out), C.byref(it), _ptr(ws), ws.numel(), _stream(stream)))
    return out, it.value


def segment_spheres(centerlines, radius, stream=None):
    """runSphereSegmentation: 1 within distance < radius of every centerline voxel."""
    torch = _torch()
    Z, Y, X = centerlines.shape
    out = torch.empty((Z, Y, X), dtype=torch.int8, device=centerlines.device)
    _check(load().tsf_segment_spheres(_ptr(centerlines), _ptr(radius), X, Y, Z, _ptr(out), _stream(stream)))
    return out


def _np_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def remove_loops(vertices, edges, shape):
    """Host removeLoops (parallelCenterlineExtraction.cpp:129-285) on numpy
    arrays: vertices (n, 3) int (x, y, z), edges (m, 2).  Returns (vertices,
    edges) of the loop-free graph."""
    import numpy as np
    v = np.ascontiguousarray(vertices, dtype=np.int32)
    e = np.ascontiguousarray(edges, dtype=np.int32)
    Z, Y, X = shape
    cap = max(16, 2 * (len(v) + len(e)))
    ov, oe = np.zeros((cap, 3), np.int32), np.zeros((cap, 2), np.int32)
    nv, ne = C.c_int(0), C.c_int(0)
    _check(load().tsf_remove_loops(_np_ptr(v), len(v), _np_ptr(e), len(e), X, Y, Z, _np_ptr(ov), _np_ptr(oe), cap,
                                   C.byref(nv), C.byref(ne)))
    return ov[:nv.value].copy(), oe[:ne.value].copy()


def centerline_graph(vertices, edges, labels, sizes, min_tree_length, radius, max_edge_distance=0):
    """Host centerline graph stage (parallelCenterlineExtraction.cpp:1168-1247)
    on numpy arrays; returns (centerlines int8 volume, radius (updated copy),
    vertices, edges)."""
    import numpy as np
    v = np.ascontiguousarray(vertices, dtype=np.int32)
    e = np.ascontiguousarray(edges, dtype=np.int32)
    rad = np.ascontiguousarray(radius, dtype=np.float32).copy()
    Z, Y, X = rad.shape
    cl = np.zeros(rad.shape, np.int8)
    cap = 4 * (len(v) + len(e)) + 1024
    while True:
        ov, oe = np.zeros((cap, 3), np.int32), np.zeros((cap, 2), np.int32)
        nv, ne = C.c_int(0), C.c_int(0)
        r2 = rad.copy()
        cl[...] = 0
        code = load().tsf_centerline_graph(_np_ptr(v), len(v), _np_ptr(e), len(e),
                                           _np_ptr(np.ascontiguousarray(labels, dtype=np.int32)),
                                           _np_ptr(np.ascontiguousarray(sizes, dtype=np.int32)), int(min_tree_length),
                                           int(max_edge_distance), X, Y, Z, _np_ptr(r2), _np_ptr(cl), _np_ptr(ov),
                                           _np_ptr(oe), cap, C.byref(nv), C.byref(ne))
        if code != 6:
            break
        cap = 2 * max(nv.value, ne.value)
    _check(code)
    return cl, r2, ov[:nv.value].copy(), oe[:ne.value].copy()


def tdf_combine(Ts, Rs, Tl, Rl, unorm16: bool = False, stream=None):
    _check(load().tsf_tdf_combine(_ptr(Ts), _ptr(Rs), _ptr(Tl), _ptr(Rl), Tl.numel(), int(unorm16),
                                  _stream(stream)))
    return Tl, Rl


def candidates(T, R, field4, storage: str, tdf_high: float, cube_size: int, unorm16: bool = False,
               max_vertices: int = 1 << 16, want_centerpoints=False, want_candidates=False, ws=None,
               stream=None, raise_on_range=True):
    """Returns dict(vertices [n,3] int32 (x,y,z), n_candidates, n_vertices,
    centerpoints int8 volume or None, candidates [n,3] or None, status)."""
    torch = _torch()
    Z, Y, X = T.shape
    L = load()
    need = L.tsf_candidates_workspace_size(X, Y, Z)
    ws = workspace(need) if ws is None else ws
    verts = torch.zeros((max_vertices, 3), dtype=torch.int32, device=T.device)
    cp = torch.zeros((Z, Y, X), dtype=torch.int8, device=T.device) if want_centerpoints else None
    ncap = X * Y * Z // 2 + 1
    cand = torch.zeros((ncap, 3), dtype=torch.int32, device=T.device) if want_candidates else None
    nc, nv = C.c_int64(0), C.c_int64(0)
    code = L.tsf_candidates(_ptr(T), int(unorm16), _ptr(R), _ptr(field4), STORAGE[storage], X, Y, Z,
                            float(tdf_high), int(cube_size), _ptr(verts), max_vertices, _ptr(cp),
                            _ptr(cand), ncap if want_candidates else 0, C.byref(nc), C.byref(nv),
                            _ptr(ws), ws.numel(), _stream(stream))
    if code != TSF_OK and (raise_on_range or code != 4):
        _check(code)
    nvv = min(nv.value, max_vertices)
    return {"vertices": verts[:nvv], "n_candidates": nc.value, "n_vertices": nv.value,
            "centerpoints": cp, "candidates": cand[: nc.value] if cand is not None else None,
            "status": code}


def compact_mask(mask, cap=None, stream=None):
    torch = _torch()
    Z, Y, X = mask.shape
    L = load()
    ws = workspace(L.tsf_compact_workspace_size(X, Y, Z))
    cap = int(mask.numel()) if cap is None else cap
    pos = torch.zeros((max(cap, 1), 3), dtype=torch.int32, device=mask.device)
    cnt = C.c_int64(0)
    _check(L.tsf_compact_mask(_ptr(mask), X, Y, Z, _ptr(pos), cap, C.byref(cnt), _ptr(ws), ws.numel(),
                              _stream(stream)))
    return pos[: cnt.value]


def gvf_fmg(field4, mu: float, iterations: int, storage: str = "f32", ws=None, stream=None):
    torch = _torch()
    Z, Y, X = field4.shape[:3]
    L = load()
    need = L.tsf_gvf_fmg_workspace_size(X, Y, Z, STORAGE[storage])
    ws = workspace(need) if ws is None else ws
    out = torch.empty_like(field4)
    _check(L.tsf_gvf_fmg(_ptr(field4), _ptr(out), X, Y, Z, float(mu), int(iterations), STORAGE[storage],
                         _ptr(ws), ws.numel(), _stream(stream)))
    return out


def gvf_one_component(field4, mu: float, iterations: int, storage: str = "f32", ws=None, stream=None):
    """The low-memory GVF (tsf_gvf_one_component): field4 in, field4 (w = |v|) out."""
    torch = _torch()
    Z, Y, X = field4.shape[:3]
    L = load()
    need = L.tsf_gvf_one_component_workspace_size(X, Y, Z, STORAGE[storage])
    ws = workspace(need) if ws is None else ws
    out = torch.empty_like(field4)
    _check(L.tsf_gvf_one_component(_ptr(field4), X, Y, Z, float(mu), int(iterations), STORAGE[storage],
                                   _ptr(out), _ptr(ws), ws.numel(), _stream(stream)))
    return out


def convert_field(t, storage: str, to: str, stream=None):
    """tsf_convert_field: a new tensor holding t's values in storage `to`."""
    torch = _torch()
    out = torch.empty(t.shape, dtype=storage_dtype(to), device=t.device)
    _check(load().tsf_convert_field(_ptr(t), STORAGE[storage], _ptr(out), STORAGE[to], t.numel(), _stream(stream)))
    return out


def to_float(t, storage: str):
    """Stored values -> float32 (snorm16: max(-1, s/32767))."""
    torch = _torch()
    if storage == "snorm16":
        return torch.clamp_min(t.to(torch.float32) / 32767.0, -1.0)
    return t.to(torch.float32)
