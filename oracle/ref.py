"""ctypes binding of oracle/_ref/libtsf_ref.so: the reference's own kernel
source (kernels.cl of smistad/Tube-Segmentation-Framework) compiled for the
CPU under an OpenCL C shim (oracle/clshim/), driven in the order the
reference's host code enqueues its kernels.

TEST INFRASTRUCTURE ONLY: used by tests/ to pin the oracle (oracle.py) to the
reference's text, and by tests/golden/make_golden.py to write the golden
vectors the GPU tests compare with.  It needs the reference source tree
($TSF_REFERENCE_DIR, default /root/reference); available() is False without
it.  Only the reference's two field formats exist here: CL_FLOAT ("f32") and
CL_SNORM_INT16 ("snorm16").
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "clshim"))
import make_ref  # noqa: E402

_lib = None
_p, _i, _i64, _f = C.c_void_p, C.c_int, C.c_int64, C.c_float


def available() -> bool:
    return os.path.exists(os.path.join(make_ref.reference_dir(), "kernels.cl"))


def build(force: bool = False) -> str:
    return make_ref.build(force=force)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        for s in ("_f", "_u"):
            getattr(_lib, "ref_blur" + s).argtypes = [_p, _i, _i, _i, _i, _p, _p]
            getattr(_lib, "ref_vector_field" + s).argtypes = [_p, _i, _i, _i, _f, _i, _i, _p]
            getattr(_lib, "ref_gvf" + s).argtypes = [_p, _i, _i, _i, _f, _i, _i, _p, _p]
            getattr(_lib, "ref_tdf_circle" + s).argtypes = [_p, _i, _i, _i, _i, _f, _f, _f, _p, _p]
            getattr(_lib, "ref_combine" + s).argtypes = [_p, _p, _p, _p, _i64]
            getattr(_lib, "ref_candidates" + s).argtypes = [_p, _p, _p, _i, _i, _i, _i, _f, _i, _p, _i64, _p, _p,
                                                             _p, _i64, _p]
            getattr(_lib, "ref_candidates" + s).restype = _i
            getattr(_lib, "ref_eigen" + s).argtypes = [_p, _i64, _p, _p]
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _xyz(a):
    Z, Y, X = a.shape[:3]
    return X, Y, Z


def _sn(storage):
    if storage not in ("f32", "snorm16"):
        raise ValueError("the reference's field formats are f32 and snorm16")
    return 1 if storage == "snorm16" else 0


def blur(vol, mask_size: int, mask) -> np.ndarray:
    """blurVolumeWithGaussian (kernels.cl:1017-1040) with a given mask."""
    v = np.ascontiguousarray(vol, np.float32)
    m = np.ascontiguousarray(mask, np.float32)
    out = np.empty_like(v)
    lib().ref_blur_f(_ptr(v), *_xyz(v), int(mask_size), _ptr(m), _ptr(out))
    return out


def vector_field(vol, fmax: float, vsign: int, storage: str = "f32") -> np.ndarray:
    """createVectorField (kernels.cl:1042-1063) -> field4 [Z,Y,X,4] as stored."""
    v = np.ascontiguousarray(vol, np.float32)
    out = np.empty(v.shape + (4,), np.float32)
    lib().ref_vector_field_f(_ptr(v), *_xyz(v), float(fmax), int(vsign), _sn(storage), _ptr(out))
    return out


def gvf(field4, mu: float, iterations: int, storage: str = "f32"):
    """runFastGVF (gradientVectorFlow.cpp:1105-1170): GVF3DInit, the
    GVF3DIteration ping-pong, GVF3DFinish.  Returns (v field4 [Z,Y,X,4] as
    the finish reads it -- after `iterations` iterations when that is even,
    iterations - 1 when odd -- with w = f0z, finished field4 with w = |v|)."""
    f = np.ascontiguousarray(field4, np.float32)
    v = np.empty_like(f)
    fin = np.empty_like(f)
    lib().ref_gvf_f(_ptr(f), *_xyz(f), float(mu), int(iterations), _sn(storage), _ptr(v), _ptr(fin))
    return v, fin


def tdf_circle(field4, rmin, rmax, rstep, storage: str = "f32", unorm16: bool = False):
    """circleFittingTDF (kernels.cl:1071-1157): (T, R); T is uint16 (unorm16,
    the VECTORS_16BIT build) when unorm16, else float32."""
    f = np.ascontiguousarray(field4, np.float32)
    shape = f.shape[:3]
    T = np.zeros(shape, np.uint16 if unorm16 else np.float32)
    R = np.zeros(shape, np.float32)
    getattr(lib(), "ref_tdf_circle" + ("_u" if unorm16 else "_f"))(
        _ptr(f), *_xyz(f), _sn(storage), float(rmin), float(rmax), float(rstep), _ptr(T), _ptr(R))
    return T, R


def combine(Ts, Rs, Tl, Rl):
    """combine (kernels.cl:561-572) -> new (T, R)."""
    unorm = Ts.dtype == np.uint16
    Tl2, Rl2 = np.ascontiguousarray(Tl).copy(), np.ascontiguousarray(Rl, np.float32).copy()
    Ts_, Rs_ = np.ascontiguousarray(Ts), np.ascontiguousarray(Rs, np.float32)
    getattr(lib(), "ref_combine" + ("_u" if unorm else "_f"))(_ptr(Ts_), _ptr(Rs_), _ptr(Tl2), _ptr(Rl2), Tl2.size)
    return Tl2, Rl2


def candidates(T, R, field4, storage: str, tdf_high: float, cube_size: int):
    """The candidate stage (parallelCenterlineExtraction.cpp:806-899): dict
    with the candidate list (pyramid order), the filtered candidate mask and
    the vertex list.  T: float32, or uint16 (unorm16 TDF image)."""
    unorm = T.dtype == np.uint16
    T_ = np.ascontiguousarray(T)
    R_ = np.ascontiguousarray(R, np.float32)
    f = np.ascontiguousarray(field4, np.float32)
    X, Y, Z = _xyz(f)
    n = X * Y * Z
    cand = np.zeros((n // 2 + 1, 3), np.int32)
    verts = np.zeros((16384 + 8, 3), np.int32)
    mask2 = np.zeros(f.shape[:3], np.int8)
    nc, nv = C.c_int64(0), C.c_int64(0)
    r = getattr(lib(), "ref_candidates" + ("_u" if unorm else "_f"))(
        _ptr(T_), _ptr(R_), _ptr(f), _sn(storage), X, Y, Z, float(tdf_high), int(cube_size), _ptr(cand),
        cand.shape[0], C.byref(nc), _ptr(mask2), _ptr(verts), verts.shape[0], C.byref(nv))
    if r != 0:
        raise RuntimeError("capacity exceeded")
    return {"candidates": cand[:nc.value].copy(), "mask2": mask2, "vertices": verts[:nv.value].copy()}


def eigen(A):
    """eigen_decomposition (kernels.cl:1519-1773) of symmetric 3x3 matrices
    [n, 3, 3] -> (V [n, 3, 3] with eigenvectors as columns, d [n, 3])."""
    A_ = np.ascontiguousarray(A, np.float32).reshape(-1, 9)
    V = np.empty_like(A_)
    d = np.empty((A_.shape[0], 3), np.float32)
    lib().ref_eigen_f(_ptr(A_), A_.shape[0], _ptr(V), _ptr(d))
    return V.reshape(-1, 3, 3), d
