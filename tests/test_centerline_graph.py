"""Host centerline graph stage (no GPU): removeLoops, the large-tree filter,
edge splitting, rasterisation with radius averaging, and the VTK writer
(parallelCenterlineExtraction.cpp:129-321, 1168-1247; inputOutput.cpp:48-63)."""
import math

import numpy as np
import pytest


def _pairs(v, e):
    """undirected edges as sets of vertex positions"""
    return {frozenset((tuple(v[a]), tuple(v[b]))) for a, b in e}


def _components(n, e):
    parent = list(range(n))

    def find(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    for a, b in e:
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[ra] = rb
    return len({find(i) for i in range(n)})


def test_chain_is_kept(tsf):
    v = np.array([[2 + 3 * i, 5, 5] for i in range(7)])
    e = np.array([[i, i + 1] for i in range(6)])
    ov, oe = tsf.remove_loops(v, e, (16, 16, 32))
    assert {tuple(p) for p in ov} == {tuple(p) for p in v}
    assert _pairs(ov, oe) == _pairs(v, e)


def test_loop_keeps_the_shorter_path(tsf):
    """Junctions A and B joined by a short and a long chain, each with a tail:
    the long chain's inner vertices are dropped."""
    A, B = [10, 10, 5], [20, 10, 5]
    TA, TB = [4, 10, 5], [26, 10, 5]
    p = [[13, 11, 5], [17, 11, 5]]                                  # short path
    q = [[11, 16, 5], [14, 19, 5], [17, 19, 5], [19, 15, 5]]      # long path
    v = np.array([A, B, TA, TB] + p + q)
    e = np.array([[0, 2], [1, 3], [0, 4], [4, 5], [5, 1], [0, 6], [6, 7], [7, 8], [8, 9], [9, 1]])
    ov, oe = tsf.remove_loops(v, e, (16, 32, 32))
    kept = {tuple(x) for x in ov}
    assert kept == {tuple(x) for x in [A, B, TA, TB] + p}
    assert _pairs(ov, oe) == {frozenset((tuple(a), tuple(b))) for a, b in
                              [(A, TA), (B, TB), (A, p[0]), (p[0], p[1]), (p[1], B)]}


def test_random_graph_becomes_a_forest(tsf):
    rng = np.random.default_rng(3)
    pos = set()
    while len(pos) < 60:
        pos.add(tuple(rng.integers(0, 40, 3).tolist()))
    v = np.array(sorted(pos))
    e = set()
    for i in range(1, len(v)):                                     # a random tree ...
        e.add((int(rng.integers(0, i)), i))
    while len(e) < 75:                                             # ... plus loops
        a, b = rng.integers(0, len(v), 2)
        if a != b and (b, a) not in e:
            e.add((int(a), int(b)))
    e = np.array(sorted(e))
    ov, oe = tsf.remove_loops(v, e, (40, 40, 40))
    assert len(oe) == len(ov) - _components(len(ov), oe)         # no cycles
    assert {tuple(x) for x in ov} <= {tuple(x) for x in v}
    assert _pairs(ov, oe) <= _pairs(v, e)


def test_empty_graph_is_an_error(tsf):
    v = np.array([[1, 1, 1], [5, 5, 5]])
    e = np.array([[0, 1]])
    labels, sizes = np.array([0, 0]), np.array([2, 0])
    with pytest.raises(tsf.TSFError) as err:
        tsf.centerline_graph(v, e, labels, sizes, 5, np.zeros((8, 8, 8), np.float32))
    assert err.value.code == 4


def _raster(v, e, radius):
    """createCenterlineVoxels restated: ceil(|ab|) steps from a, radius replaced
    by its mean along each edge."""
    cl = np.zeros(radius.shape, np.int8)
    rad = radius.copy()
    for a, b in e:
        A, B = v[a].astype(np.float32), v[b].astype(np.float32)
        d = np.float32(math.sqrt(float(np.float32((A[0] - B[0]) ** 2 + (A[1] - B[1]) ** 2) + (A[2] - B[2]) ** 2)))
        n = int(math.ceil(d))
        cells = []
        for j in range(n):
            r = np.float32(j) / np.float32(n)
            # round half away from zero of the float32 position (coordinates are >= 0)
            p = [int(math.floor(float(A[k] + (B[k] - A[k]) * r) + 0.5)) for k in range(3)]
            cl[p[2], p[1], p[0]] = 1
            cells.append((p[2], p[1], p[0]))
        if cells:
            avg = np.float32(sum(np.float64(rad[c]) for c in cells) / len(cells))
            for c in cells:
                rad[c] = avg
    return cl, rad


def test_graph_stage_filters_trees_and_rasterises(tsf):
    # two trees: a 6-vertex chain (kept) and a 2-vertex stub (dropped at min 5)
    v = np.array([[2 + 3 * i, 6, 6] for i in range(6)] + [[4, 20, 20], [7, 20, 20]])
    e = np.array([[i, i + 1] for i in range(5)] + [[6, 7]])
    labels = np.array([0] * 6 + [6, 6])
    sizes = np.zeros(8, np.int32)
    sizes[0], sizes[6] = 6, 2
    rng = np.random.default_rng(1)
    radius = rng.random((28, 28, 20)).astype(np.float32)
    cl, rad, ov, oe = tsf.centerline_graph(v, e, labels, sizes, 5, radius)
    assert {tuple(x) for x in ov} == {tuple(x) for x in v[:6]}
    ref_cl, _ = _raster(ov, oe, radius)
    assert np.array_equal(cl, ref_cl)
    assert cl[20, 20, :].sum() == 0                                # the stub is gone
    on = cl.astype(bool)
    assert not np.array_equal(rad[on], radius[on])                 # radius averaged along edges
    assert np.array_equal(rad[~on], radius[~on])


def test_short_capacity_writes_nothing(tsf):
    """TSF_ERR_CAPACITY returns both counts and leaves radius and centerlines
    as they were, so a second call with enough room gives the full result."""
    import ctypes as C
    L = tsf.load()
    v = np.array([[2 + 3 * i, 6, 6] for i in range(6)], np.int32)
    e = np.array([[i, i + 1] for i in range(5)], np.int32)
    labels, sizes = np.zeros(6, np.int32), np.array([6, 0, 0, 0, 0, 0], np.int32)
    radius = np.random.default_rng(2).random((12, 12, 20)).astype(np.float32)
    Z, Y, X = radius.shape

    def call(cap, rad, cl):
        ov, oe = np.zeros((max(cap, 1), 3), np.int32), np.zeros((max(cap, 1), 2), np.int32)
        nv, ne = C.c_int(0), C.c_int(0)
        code = L.tsf_centerline_graph(tsf._np_ptr(v), 6, tsf._np_ptr(e), 5, tsf._np_ptr(labels),
                                      tsf._np_ptr(sizes), 1, 0, X, Y, Z, tsf._np_ptr(rad), tsf._np_ptr(cl),
                                      tsf._np_ptr(ov), tsf._np_ptr(oe), cap, C.byref(nv), C.byref(ne))
        return code, nv.value, ne.value

    rad, cl = radius.copy(), np.zeros(radius.shape, np.int8)
    code, nv, ne = call(3, rad, cl)
    assert code == 6 and (nv, ne) == (6, 5)                        # TSF_ERR_CAPACITY with the counts
    assert np.array_equal(rad, radius) and not cl.any()            # nothing written
    code, nv, ne = call(8, rad, cl)
    assert code == 0 and (nv, ne) == (6, 5)
    ref_cl, ref_rad = _raster(v, e, radius)
    assert np.array_equal(cl, ref_cl)
    assert cl.any() and not np.array_equal(rad, radius)


def _graph_cells(tsf, v, e, labels, sizes, min_tree, shape, split=0, cap=4096, ccap=1 << 16):
    import ctypes as C
    Z, Y, X = shape
    v, e = np.ascontiguousarray(v, np.int32), np.ascontiguousarray(e, np.int32)
    labels, sizes = np.ascontiguousarray(labels, np.int32), np.ascontiguousarray(sizes, np.int32)
    ov, oe = np.zeros((cap, 3), np.int32), np.zeros((cap, 2), np.int32)
    cells, start = np.zeros(ccap, np.int64), np.zeros(cap + 1, np.int64)
    nv, ne, nc = C.c_int(0), C.c_int(0), C.c_int64(0)
    code = tsf.load().tsf_centerline_graph_cells(
        tsf._np_ptr(v), len(v), tsf._np_ptr(e), len(e), tsf._np_ptr(labels), tsf._np_ptr(sizes), min_tree, split,
        X, Y, Z, tsf._np_ptr(ov), tsf._np_ptr(oe), cap, C.byref(nv), C.byref(ne), tsf._np_ptr(cells),
        tsf._np_ptr(start), C.c_int64(ccap), C.byref(nc))
    return code, ov[:nv.value], oe[:ne.value], cells[:nc.value], start[:ne.value + 1]


def test_cells_and_smoothing_equal_the_volume_stage(tsf):
    """tsf_centerline_graph_cells + tsf_centerline_smooth_radius, applied to
    the volumes, give exactly tsf_centerline_graph's centerlines and radius
    (loops, shared cells between edges, a dropped small tree)."""
    import ctypes as C
    rng = np.random.default_rng(7)
    pos = set()
    while len(pos) < 50:
        pos.add(tuple(rng.integers(0, 30, 3).tolist()))
    v = np.array(sorted(pos))
    e = {(int(rng.integers(0, i)), i) for i in range(1, 45)}
    while len(e) < 60:
        a, b = rng.integers(0, 45, 2)
        if a != b and (b, a) not in e:
            e.add((int(a), int(b)))
    e = np.array(sorted(e) + [(45, 46), (47, 48)])               # plus two 2-vertex trees (dropped at 3)
    labels = np.array([0] * 45 + [45, 45, 47, 47, 49])
    sizes = np.zeros(50, np.int32)
    sizes[0], sizes[45], sizes[47], sizes[49] = 45, 2, 2, 1
    shape = (30, 30, 30)
    radius = rng.random(shape).astype(np.float32)
    cl_ref, rad_ref, ov_ref, oe_ref = tsf.centerline_graph(v, e, labels, sizes, 3, radius)
    code, ov, oe, cells, start = _graph_cells(tsf, v, e, labels, sizes, 3, shape)
    assert code == 0
    assert np.array_equal(ov, ov_ref) and np.array_equal(oe, oe_ref)
    assert start[0] == 0 and start[-1] == len(cells) and np.all(np.diff(start) >= 0)
    assert len(np.unique(cells)) < len(cells)                      # edges share their end cells
    flat = radius.reshape(-1)
    vals = np.ascontiguousarray(flat[cells])
    uc, uv = np.zeros(len(cells), np.int64), np.zeros(len(cells), np.float32)
    nu = C.c_int64(0)
    assert tsf.load().tsf_centerline_smooth_radius(tsf._np_ptr(cells), tsf._np_ptr(start), len(oe),
                                                   tsf._np_ptr(vals), tsf._np_ptr(uc), tsf._np_ptr(uv),
                                                   C.byref(nu)) == 0
    uc, uv = uc[:nu.value], uv[:nu.value]
    assert len(np.unique(uc)) == len(uc) and set(uc.tolist()) == set(cells.tolist())
    cl, rad = np.zeros(flat.shape, np.int8), flat.copy()
    cl[uc], rad[uc] = 1, uv
    assert np.array_equal(cl.reshape(shape), cl_ref)
    assert np.array_equal(rad.reshape(shape).view(np.uint32), rad_ref.view(np.uint32))
    # a short cell capacity: the counts come back, nothing else is needed
    code, _, _, short, _ = _graph_cells(tsf, v, e, labels, sizes, 3, shape, ccap=len(cells) - 1)
    assert code == 6


def test_edge_splitting_for_the_vtk_file(tsf):
    v = np.array([[2, 4, 4], [14, 4, 4], [20, 4, 4]])
    e = np.array([[0, 1], [1, 2]])
    labels, sizes = np.zeros(3, np.int32), np.array([3, 0, 0], np.int32)
    _, _, ov, oe = tsf.centerline_graph(v, e, labels, sizes, 1, np.zeros((8, 8, 24), np.float32),
                                        max_edge_distance=3)
    xs = sorted(p[0] for p in ov)
    assert xs == [2, 5, 8, 11, 14, 17, 20]                         # vertices every 3 voxels
    assert len(oe) == 6


def test_vtk_writer(tsf, tmp_path):
    v = np.array([[1, 2, 3], [4, 5, 6]], np.int32)
    e = np.array([[0, 1]], np.int32)
    path = str(tmp_path / "c.vtk")
    L = tsf.load()
    assert L.tsf_write_centerline_vtk(path.encode(), tsf._np_ptr(v), 2, tsf._np_ptr(e), 1) == 0
    txt = open(path).read()
    assert txt == ("# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET POLYDATA\nPOINTS 2 int\n"
                   "1 2 3\n4 5 6\n\nLINES 1 3\n2 0 1\n")
