"""ctypes binding of the CPU oracle (liboracle_tsf.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
the cpu_baseline / reference legs of bench.py, always as the checker or the
timed CPU baseline, never as part of the product path.

Parity against the reference's own outputs is unpinned (the reference is
OpenCL 1.1 and cannot run here; it has no golden vectors).  Each wrapper names
the reference kernel it restates (file:line in smistad/Tube-Segmentation-Framework).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_tsf.so")

F32, F16, BF16, SNORM16 = 0, 1, 2, 3
STORAGE = {"f32": F32, "f16": F16, "bf16": BF16, "snorm16": SNORM16}

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t
               for f in ("tsf_oracle.c", "tsf_oracle_impl.h", "tsf_oracle.h", "tsf_oracle_eigc.h"))


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_p = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_f = C.c_float


def _declare(L):
    L.orc_quantize.restype = _f
    L.orc_quantize.argtypes = [_f, _i]
    L.orc_quantize_array.argtypes = [_p, _i64, _i]
    L.orc_to_unorm16_array.argtypes = [_p, _p, _i64]
    L.orc_from_unorm16_array.argtypes = [_p, _p, _i64]
    L.orc_circle_table.argtypes = [_p, _p]
    L.orc_blur_mask.restype = _i
    L.orc_blur_mask.argtypes = [_f, _p]
    L.orc_hp_compact.restype = _i64
    L.orc_hp_compact.argtypes = [_p, _i, _i, _i, _p, _i64]
    L.orc_link_centerpoints.restype = _i
    L.orc_link_centerpoints.argtypes = [_p, _i, _p, _i, _i, _i, _f, _f, _p, _p, _p]
    L.orc_rasterize_trees.restype = None
    L.orc_rasterize_trees.argtypes = [_p, _p, _i, _p, _p, _i, _p, _i, _i, _i]
    L.orc_segment_inverse_gradient.restype = _i
    L.orc_segment_inverse_gradient.argtypes = [_p, _p, _p, _i, _i, _i, _p]
    L.orc_crop_scan_lines.restype = None
    L.orc_crop_scan_lines.argtypes = [_p, _i, _i, _i, _i, _i, _f, _p]
    L.orc_segment_spheres.restype = None
    L.orc_segment_spheres.argtypes = [_p, _p, _i, _i, _i, _p]
    L.orc_threshold_f32.argtypes = [_p, _i64, _f, _p]
    L.orc_eig3_closed_f32.argtypes = [_p, _p, _p]
    L.orc_gvf_residual_norm.argtypes = [_p, _p, _i, _i, _i, _f, _i, _p]
    L.orc_set_threads.argtypes = [_i]
    L.orc_get_threads.restype = _i
    for s in ("_f32", "_f64"):
        getattr(L, "orc_blur" + s).argtypes = [_p, _i, _i, _i, _i, _p, _p]
        getattr(L, "orc_vector_field" + s).argtypes = [_p, _i, _i, _i, _f, _i, _i, _p]
        getattr(L, "orc_gvf_init" + s).argtypes = [_p, _i64, _p, _p]
        getattr(L, "orc_gvf" + s).argtypes = [_p, _p, _i, _i, _i, _f, _i, _i]
        getattr(L, "orc_gvf_finish" + s).argtypes = [_p, _i64, _i, _p]
        getattr(L, "orc_gvf_one_component" + s).argtypes = [_p, _i, _i, _i, _f, _i, _i, _p]
        getattr(L, "orc_eig3" + s).argtypes = [_p, _p, _p]
        getattr(L, "orc_tdf_circle" + s).argtypes = [_p, _i, _i, _i, _f, _f, _f, _p, _p]
        getattr(L, "orc_tdf_circle_ex" + s).argtypes = [_p, _i, _i, _i, _f, _f, _f, _i, _i, _i, _p, _p]
        getattr(L, "orc_tdf_spline" + s).argtypes = [_p, _i, _i, _i, _f, _f, _f, _p, _p]
        getattr(L, "orc_combine" + s).argtypes = [_p, _p, _p, _p, _i64]
        getattr(L, "orc_candidates2" + s).argtypes = [_p, _p, _i, _i, _i, _p, _i64, _p]
        getattr(L, "orc_dd" + s).argtypes = [_p, _p, _i, _i, _i, _i, _p]
        getattr(L, "orc_fmg_gvf" + s).argtypes = [_p, _i, _i, _i, _f, _i, _i, _p]


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


def _real(f64: bool):
    return (np.float64, "_f64") if f64 else (np.float32, "_f32")


def _dims(vol: np.ndarray):
    """numpy volumes are indexed [z, y, x]; returns (X, Y, Z)."""
    Z, Y, X = vol.shape[:3]
    return X, Y, Z


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


# ---- conversions ----------------------------------------------------------

def quantize(a: np.ndarray, storage: str) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=np.float32).copy()
    lib().orc_quantize_array(_ptr(out), out.size, STORAGE[storage])
    return out


def to_unorm16(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty(a.shape, np.uint16)
    lib().orc_to_unorm16_array(_ptr(a), _ptr(out), a.size)
    return out


def from_unorm16(u: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.uint16)
    out = np.empty(u.shape, np.float32)
    lib().orc_from_unorm16_array(_ptr(u), _ptr(out), u.size)
    return out


def circle_table():
    c = np.zeros(32, np.float32)
    s = np.zeros(32, np.float32)
    lib().orc_circle_table(_ptr(c), _ptr(s))
    return c, s


def blur_mask(sigma: float):
    """createBlurMask, tube-segmentation.cpp:188-211 -> (m, mask[(2m+1)^3])."""
    buf = np.zeros(11 ** 3, np.float32)
    m = lib().orc_blur_mask(float(sigma), _ptr(buf))
    return m, buf[: (2 * m + 1) ** 3].copy()


# ---- kernels ----------------------------------------------------------------

def blur(vol: np.ndarray, sigma: float, f64: bool = False) -> np.ndarray:
    """blurVolumeWithGaussian, kernels.cl:1017-1040."""
    dt, s = _real(f64)
    vol = np.ascontiguousarray(vol, dtype=np.float32)
    X, Y, Z = _dims(vol)
    m, mask = blur_mask(sigma)
    out = np.empty(vol.shape, dt)
    getattr(lib(), "orc_blur" + s)(_ptr(vol), X, Y, Z, m, _ptr(mask), _ptr(out))
    return out


def vector_field(vol: np.ndarray, fmax: float, vsign: int = 1, storage: str = "f32",
                 f64: bool = False) -> np.ndarray:
    """createVectorField, kernels.cl:1042-1063 -> field4 [Z,Y,X,4]."""
    dt, s = _real(f64)
    vol = np.ascontiguousarray(vol, dtype=dt)
    X, Y, Z = _dims(vol)
    out = np.empty(vol.shape + (4,), dt)
    getattr(lib(), "orc_vector_field" + s)(_ptr(vol), X, Y, Z, float(fmax), int(vsign),
                                           STORAGE[storage], _ptr(out))
    return out


def gvf(field4: np.ndarray, mu: float, iterations: int, storage: str = "f32",
        f64: bool = False) -> np.ndarray:
    """GVF3DInit + iterations x GVF3DIteration (kernels.cl:1464-1503).
    Returns planar v [3, Z, Y, X]."""
    dt, s = _real(f64)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    Z, Y, X = field4.shape[:3]
    n = X * Y * Z
    v = np.empty((3, Z, Y, X), dt)
    f = np.empty((3, Z, Y, X), dt)
    L = lib()
    getattr(L, "orc_gvf_init" + s)(_ptr(field4), n, _ptr(v), _ptr(f))
    getattr(L, "orc_gvf" + s)(_ptr(f), _ptr(v), X, Y, Z, float(mu), int(iterations),
                              STORAGE[storage])
    return v


def gvf_planar(f: np.ndarray, v0: np.ndarray, mu: float, iterations: int,
               storage: str = "f32", f64: bool = False) -> np.ndarray:
    """GVF iterations from explicit planar f0 and v0 ([3,Z,Y,X])."""
    dt, s = _real(f64)
    f = np.ascontiguousarray(f, dtype=dt)
    v = np.ascontiguousarray(v0, dtype=dt).copy()
    _, Z, Y, X = f.shape
    getattr(lib(), "orc_gvf" + s)(_ptr(f), _ptr(v), X, Y, Z, float(mu), int(iterations),
                                  STORAGE[storage])
    return v


def gvf_residual_norm(f0: np.ndarray, v: np.ndarray, mu: float, kind: int = 0) -> np.ndarray:
    """FP64 norms of the GVF residual at every voxel's mirrored position
    (kind 0: GVF3DIteration's update, kernels.cl:1486-1490; kind 1:
    fmgResidual, kernels.cl:2008-2053, spacing 1); f0, v planar [3,Z,Y,X]
    stored values.  Returns [|r_x|, |r_y|, |r_z|, |r|, max |r|]."""
    f = np.ascontiguousarray(f0, dtype=np.float32)
    vv = np.ascontiguousarray(v, dtype=np.float32)
    _, Z, Y, X = f.shape
    out = np.zeros(5, np.float64)
    lib().orc_gvf_residual_norm(_ptr(f), _ptr(vv), X, Y, Z, float(mu), int(kind), _ptr(out))
    return out


def gvf_finish(v: np.ndarray, storage: str = "f32", f64: bool = False) -> np.ndarray:
    """GVF3DFinish, kernels.cl:1506-1515 -> field4 [Z,Y,X,4]."""
    dt, s = _real(f64)
    v = np.ascontiguousarray(v, dtype=dt)
    _, Z, Y, X = v.shape
    out = np.empty((Z, Y, X, 4), dt)
    getattr(lib(), "orc_gvf_finish" + s)(_ptr(v), X * Y * Z, STORAGE[storage], _ptr(out))
    return out


def gvf_one_component(field4: np.ndarray, mu: float, iterations: int, storage: str = "f32",
                      f64: bool = False) -> np.ndarray:
    """runLowMemoryGVF (gradientVectorFlow.cpp:1172-1300, kernels
    kernels_no_3d_write.cl:1669-1741): one component at a time with |f0|^2
    stored, then the finish pass -> field4 [Z,Y,X,4]."""
    dt, s = _real(f64)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    Z, Y, X = field4.shape[:3]
    out = np.empty((Z, Y, X, 4), dt)
    getattr(lib(), "orc_gvf_one_component" + s)(_ptr(field4), X, Y, Z, float(mu), int(iterations),
                                                STORAGE[storage], _ptr(out))
    return out


def eig3(A: np.ndarray, f64: bool = False):
    """eigen_decomposition (tred2 + tql2), kernels.cl:1519-1773."""
    dt, s = _real(f64)
    A = np.ascontiguousarray(A, dtype=dt).reshape(3, 3)
    V = np.empty((3, 3), dt)
    d = np.empty(3, dt)
    getattr(lib(), "orc_eig3" + s)(_ptr(A), _ptr(V), _ptr(d))
    return d, V


def tdf_circle(field4: np.ndarray, rmin: float, rmax: float, rstep: float,
               f64: bool = False, samples: int = 32, stride: int = 1, eigen: int = 0):
    """circleFittingTDF, kernels.cl:1071-1157 -> (T, R) float volumes.
    samples / stride: samples per radius taking table entries j * stride
    (32 / 1 in the reference); eigen 1: the closed-form eigensolver (float
    only)."""
    dt, s = _real(f64)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    Z, Y, X = field4.shape[:3]
    T = np.empty((Z, Y, X), dt)
    R = np.empty((Z, Y, X), dt)
    getattr(lib(), "orc_tdf_circle_ex" + s)(_ptr(field4), X, Y, Z, float(rmin), float(rmax),
                                            float(rstep), int(samples), int(stride), int(eigen), _ptr(T), _ptr(R))
    return T, R


def eig3_closed(A: np.ndarray):
    """The closed-form eigensolver of the TDF's eigen mode 1 -> (d, V)."""
    A = np.ascontiguousarray(A, dtype=np.float32).reshape(3, 3)
    V = np.empty((3, 3), np.float32)
    d = np.empty(3, np.float32)
    lib().orc_eig3_closed_f32(_ptr(A), _ptr(V), _ptr(d))
    return d, V


def tdf_spline(field4: np.ndarray, rmin: float, rmax: float, rstep: float, f64: bool = False):
    """splineTDF, kernels.cl:1159-1254, with runSplineTDF's constants
    (rMin = max(1, rmin), 12 arms, minAverageMag 0.1) -> (T, R) float volumes."""
    dt, s = _real(f64)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    Z, Y, X = field4.shape[:3]
    T = np.empty((Z, Y, X), dt)
    R = np.empty((Z, Y, X), dt)
    getattr(lib(), "orc_tdf_spline" + s)(_ptr(field4), X, Y, Z, float(rmin), float(rmax), float(rstep), _ptr(T),
                                         _ptr(R))
    return T, R


def combine(Ts, Rs, Tl, Rl, f64: bool = False):
    """combine, kernels.cl:561-572 (returns new arrays)."""
    dt, s = _real(f64)
    Ts = np.ascontiguousarray(Ts, dtype=dt)
    Rs = np.ascontiguousarray(Rs, dtype=dt)
    Tl = np.ascontiguousarray(Tl, dtype=dt).copy()
    Rl = np.ascontiguousarray(Rl, dtype=dt).copy()
    getattr(lib(), "orc_combine" + s)(_ptr(Ts), _ptr(Rs), _ptr(Tl), _ptr(Rl), Tl.size)
    return Tl, Rl


def threshold(T: np.ndarray, thr: float) -> np.ndarray:
    """findCandidateCenterpoints, kernels.cl:1296-1307."""
    T = np.ascontiguousarray(T, dtype=np.float32)
    m = np.empty(T.shape, np.int8)
    lib().orc_threshold_f32(_ptr(T), T.size, float(thr), _ptr(m))
    return m


def hp_compact(mask: np.ndarray) -> np.ndarray:
    """Histogram-pyramid enumeration (kernels.cl:63-299) -> int32 [count, 3] (x,y,z)."""
    mask = np.ascontiguousarray(mask, dtype=np.int8)
    X, Y, Z = _dims(mask)
    cnt = int(np.count_nonzero(mask))
    pos = np.zeros((max(cnt, 1), 3), np.int32)
    total = lib().orc_hp_compact(_ptr(mask), X, Y, Z, _ptr(pos), cnt)
    assert total == cnt
    return pos[:cnt].copy()


def candidates2(radius, field4, positions, f64: bool = False) -> np.ndarray:
    """findCandidateCenterpoints2, kernels.cl:1309-1390 -> int8 mask."""
    dt, s = _real(f64)
    radius = np.ascontiguousarray(radius, dtype=dt)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    positions = np.ascontiguousarray(positions, dtype=np.int32)
    X, Y, Z = _dims(radius)
    out = np.zeros(radius.shape, np.int8)
    getattr(lib(), "orc_candidates2" + s)(_ptr(radius), _ptr(field4), X, Y, Z,
                                          _ptr(positions), len(positions), _ptr(out))
    return out


def dd(T, cand, cube_size: int, f64: bool = False) -> np.ndarray:
    """dd, kernels.cl:1260-1292 -> int8 vertex mask."""
    dt, s = _real(f64)
    T = np.ascontiguousarray(T, dtype=dt)
    cand = np.ascontiguousarray(cand, dtype=np.int8)
    X, Y, Z = _dims(T)
    out = np.zeros(T.shape, np.int8)
    getattr(lib(), "orc_dd" + s)(_ptr(T), _ptr(cand), X, Y, Z, int(cube_size), _ptr(out))
    return out


def fmg_gvf(field4, mu: float, iterations: int, storage: str = "f32", f64: bool = False):
    """runFMGGVF, gradientVectorFlow.cpp:729-1005 -> field4 (vx, vy, vz, |v|)."""
    dt, s = _real(f64)
    field4 = np.ascontiguousarray(field4, dtype=dt)
    Z, Y, X = field4.shape[:3]
    out = np.empty((Z, Y, X, 4), dt)
    getattr(lib(), "orc_fmg_gvf" + s)(_ptr(field4), X, Y, Z, float(mu), int(iterations),
                                      STORAGE[storage], _ptr(out))
    return out


# ---- composite: the candidate stage (runNewCenterlineAlg front half) --------

def link_centerpoints(vertices, T, min_mean_tdf: float, max_distance: float):
    """runNewCenterlineAlg back half (parallelCenterlineExtraction.cpp:911-1161,
    kernels.cl:327-508): vertices (n, 3) int (x, y, z); T the TDF as read by
    the linear sampler (float; unorm16 already divided by 65535).  Returns
    (edges (m, 2) in the 2-D pyramid order, labels, tree sizes)."""
    v = np.ascontiguousarray(vertices, dtype=np.int32)
    n = v.shape[0]
    T32 = np.ascontiguousarray(T, dtype=np.float32)
    Z, Y, X = T32.shape
    edges = np.zeros((2 * n, 2), np.int32)
    labels = np.zeros(n, np.int32)
    sizes = np.zeros(n, np.int32)
    ne = lib().orc_link_centerpoints(_ptr(v), n, _ptr(T32), X, Y, Z, float(min_mean_tdf), float(max_distance),
                                     _ptr(edges), _ptr(labels), _ptr(sizes))
    return edges[:ne].copy(), labels, sizes


def rasterize_trees(vertices, edges, labels, sizes, min_tree_length: int, shape):
    """removeSmallTrees (kernels.cl:510-534) into a zeroed int8 volume."""
    v = np.ascontiguousarray(vertices, dtype=np.int32)
    e = np.ascontiguousarray(edges, dtype=np.int32)
    out = np.zeros(shape, np.int8)
    Z, Y, X = shape
    lib().orc_rasterize_trees(_ptr(v), _ptr(e), e.shape[0], _ptr(np.ascontiguousarray(labels, dtype=np.int32)),
                              _ptr(np.ascontiguousarray(sizes, dtype=np.int32)), int(min_tree_length), _ptr(out),
                              X, Y, Z)
    return out


RAW_TYPES = {np.dtype(np.uint8): 0, np.dtype(np.int8): 1, np.dtype(np.uint16): 2, np.dtype(np.int16): 3,
             np.dtype(np.float32): 4}


def crop_scan_lines(vol, method: int, threshold: float = 0.0):
    """cropDatasetThreshold (method 0) / cropDatasetLung (method 1),
    kernels.cl:813-946, over the three slice directions: (counts_x, counts_y,
    counts_z) int16 of the raw volume (Z, Y, X) of a MET_* dtype."""
    v = np.ascontiguousarray(vol)
    Z, Y, X = v.shape
    counts = np.zeros(X + Y + Z, np.int16)
    lib().orc_crop_scan_lines(_ptr(v), RAW_TYPES[v.dtype], X, Y, Z, int(method), float(threshold), _ptr(counts))
    return counts[:X], counts[X:X + Y], counts[X + Y:]


def segment_inverse_gradient(centerlines, field4, radius):
    """runInverseGradientSegmentation (segmentation.cpp:5-205; initGrowing,
    grow, dilate, erode, kernels_no_3d_write.cl:1100-1207, 1370-1412).
    centerlines (Z, Y, X) int8; field4 (Z, Y, X, 4) as read (float32, storage
    already converted); radius (Z, Y, X) float32.  Returns (segmentation int8,
    grow iterations).  Grow iterations decide first and apply second with the
    precedence accepted > to check > dropped."""
    cl = np.ascontiguousarray(centerlines, dtype=np.int8)
    F = np.ascontiguousarray(field4, dtype=np.float32)
    R = np.ascontiguousarray(radius, dtype=np.float32)
    Z, Y, X = cl.shape
    assert F.shape == (Z, Y, X, 4) and R.shape == cl.shape
    out = np.zeros(cl.shape, np.int8)
    it = lib().orc_segment_inverse_gradient(_ptr(cl), _ptr(F), _ptr(R), X, Y, Z, _ptr(out))
    return out, it


def segment_spheres(centerlines, radius):
    """runSphereSegmentation (segmentation.cpp:207-307; sphereSegmentation,
    kernels_no_3d_write.cl:1209-1234)."""
    cl = np.ascontiguousarray(centerlines, dtype=np.int8)
    R = np.ascontiguousarray(radius, dtype=np.float32)
    Z, Y, X = cl.shape
    out = np.zeros(cl.shape, np.int8)
    lib().orc_segment_spheres(_ptr(cl), _ptr(R), X, Y, Z, _ptr(out))
    return out


def centerpoints(T, R, field4, tdf_high: float, cube_size: int, f64: bool = False):
    """parallelCenterlineExtraction.cpp:667-899 up to the vertex list.

    T is the TDF as read by the candidate kernels (floats; unorm16 already
    divided by 65535 in 16-bit mode).  Returns dict with the candidate list
    (pyramid order), the filtered candidate mask, the vertex mask and the
    vertex list (pyramid order)."""
    dt, _ = _real(f64)
    T32 = np.ascontiguousarray(T, dtype=np.float32)
    m1 = threshold(T32, tdf_high)
    cand = hp_compact(m1)
    m2 = candidates2(R, field4, cand, f64=f64)
    m3 = dd(np.ascontiguousarray(T, dtype=dt), m2, cube_size, f64=f64)
    verts = hp_compact(m3)
    return {"candidates": cand, "mask1": m1, "mask2": m2, "mask3": m3, "vertices": verts}
