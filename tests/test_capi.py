"""CPU tests of the C ABI boundary: the library loads without a GPU, exports
every function include/tsf/tsf_c.h declares, and its host-side paths
(workspace queries, the blur mask, argument validation) work without one."""
import ctypes as C

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(tsf):
    lib = tsf.load()
    declared = tsf.declared_symbols()
    assert len(declared) >= 15
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version(tsf):
    assert tsf.load().tsf_abi_version() == 1


def test_storage_bytes(tsf):
    L = tsf.load()
    assert [L.tsf_storage_bytes(s) for s in range(5)] == [4, 2, 2, 2, 0]


def test_workspace_queries(tsf):
    L = tsf.load()
    assert L.tsf_gvf_workspace_size(256, 256, 256, 1) == 3 * 256 ** 3 * 2
    assert L.tsf_gvf_workspace_size(256, 256, 256, 0) == 3 * 256 ** 3 * 4
    assert L.tsf_gvf_workspace_size(8, 8, 8, 9) == 0
    n = 64 ** 3
    assert L.tsf_candidates_workspace_size(64, 64, 64) >= 2 * n + 12 * (n // 2 + 1)
    assert L.tsf_gvf_fmg_workspace_size(64, 64, 64, 1) > 3 * n * 2


def test_adjoint_checkpoint_interval(tsf):
    """The smallest interval whose workspace fits the budget: every state
    when there is room, about sqrt(K) when memory is tight, 0 when nothing
    fits."""
    L = tsf.load()
    X = Y = Z = 64
    K = 100
    ws = lambda C: L.tsf_gvf_adjoint_workspace_size(X, Y, Z, 0, K, C)
    state = 3 * X * Y * Z * 4
    assert ws(1) >= (K - 1) * state and ws(1) < (K + 2) * state
    assert L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, ws(1)) == 1
    assert L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, 1 << 50) == 1
    assert L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, ws(1) - 1) > 1
    best = min(ws(C) for C in range(1, K + 1))
    C = L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, best)
    assert C > 1 and ws(C) == best and all(ws(c) > best for c in range(1, C))
    assert L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, best - 1) == 0
    for budget in (ws(1) // 2, ws(1) // 4, (best + ws(1) // 4) // 2):
        C = L.tsf_gvf_adjoint_checkpoint_interval(X, Y, Z, 0, K, budget)
        assert C > 1 and ws(C) <= budget
        assert all(ws(c) > budget for c in range(1, C))


def test_blur_mask_matches_oracle(tsf, oracle):
    for sigma in (0.5, 1.0, 1.7, 3.0):
        m, mask = tsf.blur_mask(sigma)
        om, omask = oracle.blur_mask(sigma)
        assert m == om and np.array_equal(mask, omask)


def test_argument_validation_without_gpu(tsf):
    L = tsf.load()
    # extents below 4 are rejected before any device call
    assert L.tsf_blur(None, None, 2, 8, 8, C.c_float(1.0), None) == 1
    assert b"extents" in L.tsf_last_error_string()
    assert L.tsf_gvf(None, None, 8, 8, 8, C.c_float(0.1), 5, 7, None, 0, None) == 1
    assert L.tsf_gvf(C.c_void_p(16), C.c_void_p(16), 8, 8, 8, C.c_float(0.1), 5, 0, None, 0, None) == 3
    assert L.tsf_blur_mask(C.c_float(1.0), None, None) == 1


def test_centerline_cell_functions_validate_without_gpu(tsf):
    """The cell path of the centerline stage: argument errors, an empty cell
    list (nothing to launch), and the replay of an empty graph."""
    L = tsf.load()
    i64 = C.c_int64
    # device side: bad extents, a negative count, null buffers with cells; zero cells launch nothing
    assert L.tsf_gather_cells(None, 2, 8, 8, None, i64(4), None, None) == 1
    assert L.tsf_gather_cells(None, 8, 8, 8, None, i64(-1), None, None) == 1
    assert L.tsf_gather_cells(None, 8, 8, 8, None, i64(4), None, None) == 1
    assert L.tsf_gather_cells(None, 8, 8, 8, None, i64(0), None, None) == 0
    assert L.tsf_centerline_apply(None, None, 8, 8, 8, None, None, i64(3), None) == 1
    assert L.tsf_centerline_apply(C.c_void_p(16), C.c_void_p(16), 8, 8, 8, C.c_void_p(16), None, i64(3), None) == 1
    assert L.tsf_centerline_apply(None, None, 8, 8, 8, None, None, i64(0), None) == 0
    # host side: null outputs are argument errors; no edges replay to no cells
    nv, ne, nc = C.c_int(0), C.c_int(0), i64(0)
    assert L.tsf_centerline_graph_cells(None, 0, None, 0, None, None, 3, 0, 8, 8, 8, None, None, 0, C.byref(nv),
                                        C.byref(ne), None, None, i64(0), C.byref(nc)) == 1
    start = np.zeros(1, np.int64)
    cells = np.zeros(1, np.int64)
    vals = np.zeros(1, np.float32)
    uc, uv = np.zeros(1, np.int64), np.zeros(1, np.float32)
    nu = i64(-1)
    assert L.tsf_centerline_smooth_radius(tsf._np_ptr(cells), tsf._np_ptr(start), 0, tsf._np_ptr(vals),
                                          tsf._np_ptr(uc), tsf._np_ptr(uv), C.byref(nu)) == 0
    assert nu.value == 0
