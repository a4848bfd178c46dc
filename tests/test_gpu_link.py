"""GPU tests of centerline linking (tsf_link_centerpoints, tsf_rasterize_trees)
against the oracle: the edge list in the reference's 2-D pyramid order, the
component labels and sizes, and the rasterised trees, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.fixture(scope="module")
def phantom(oracle, synth):
    """A 64^3 vessel tree through the oracle: TDF, radius, field, vertices."""
    shape = (64, 64, 64)
    vol = synth.vascular_tree(shape, seed=11)
    f4 = oracle.vector_field(oracle.blur(vol, 0.5), 0.2, 1, "f32")
    field = oracle.gvf_finish(oracle.gvf(f4, 0.05, 60, "f32"), "f32")
    T, R = oracle.tdf_circle(field, 1.0, 7.0, 0.5)
    ref = oracle.centerpoints(T, R, field, tdf_high=0.3, cube_size=3)
    return T, R, field, ref["vertices"]


@pytest.mark.parametrize("unorm", [False, True])
@pytest.mark.parametrize("maxd,min_avg", [(10.0, 0.3), (25.0, 0.5)])
def test_link_bitexact(torch_dev, tsf, oracle, phantom, unorm, maxd, min_avg):
    torch = torch_dev
    T, R, field, verts = phantom
    assert len(verts) > 20
    if unorm:
        u = oracle.to_unorm16(T)
        dT = torch.from_numpy(u.view(np.int16)).cuda()
        T_read = oracle.from_unorm16(u)
    else:
        dT = torch.from_numpy(T).cuda()
        T_read = T
    dv = torch.from_numpy(np.ascontiguousarray(verts, dtype=np.int32)).cuda()
    edges, labels, sizes = tsf.link_centerpoints(dv, dT, min_avg, maxd, unorm16=unorm)
    oe, ol, os_ = oracle.link_centerpoints(verts, T_read, min_avg, maxd)
    assert len(oe) > 0
    assert np.array_equal(edges.cpu().numpy(), oe)
    assert np.array_equal(labels.cpu().numpy(), ol)
    assert np.array_equal(sizes.cpu().numpy(), os_)
    for min_tree in (1, 5, 30):
        cl = tsf.rasterize_trees(dv, edges, labels, sizes, min_tree, T.shape)
        assert np.array_equal(cl.cpu().numpy(), oracle.rasterize_trees(verts, oe, ol, os_, min_tree, T.shape))


def test_link_chain(torch_dev, tsf, oracle):
    torch = torch_dev
    T = np.zeros((12, 12, 40), np.float32)
    T[4:8, 4:8, :] = 1.0
    v = np.array([[2 + 3 * i, 6, 6] for i in range(12)], np.int32)
    edges, labels, sizes = tsf.link_centerpoints(torch.from_numpy(v).cuda(), torch.from_numpy(T).cuda(), 0.5, 5.0)
    oe, ol, os_ = oracle.link_centerpoints(v, T, 0.5, 5.0)
    assert np.array_equal(edges.cpu().numpy(), oe)
    assert (labels.cpu().numpy() == 0).all() and sizes.cpu().numpy()[0] == 12


def test_link_no_edges(torch_dev, tsf):
    """Two vertices farther apart than max-distance: the reference's 'No edges
    were found'."""
    torch = torch_dev
    T = torch.ones((16, 16, 16), dtype=torch.float32, device="cuda")
    v = torch.tensor([[2, 2, 2], [13, 13, 13]], dtype=torch.int32, device="cuda")
    with pytest.raises(tsf.TSFError) as e:
        tsf.link_centerpoints(v, T, 0.5, 5.0)
    assert e.value.code == 4 and "No edges" in str(e.value)


def test_gather_and_apply_cells(torch_dev, tsf):
    """tsf_gather_cells / tsf_centerline_apply (createCenterlineVoxels'
    device side): the radius read at the listed cells, the centerline mark and
    the new radius written there, cells outside the volume skipped (read as
    0, nothing written)."""
    torch = torch_dev
    L = tsf.load()
    Z, Y, X = 20, 24, 28
    n = X * Y * Z
    rng = np.random.default_rng(5)
    rad = rng.random((Z, Y, X)).astype(np.float32)
    cells = np.concatenate([rng.choice(n, 500, replace=False), [-1, n, n + 7]]).astype(np.int64)
    d_rad = torch.from_numpy(rad).cuda()
    d_cells = torch.from_numpy(cells).cuda()
    d_vals = torch.empty(len(cells), dtype=torch.float32, device="cuda")
    assert L.tsf_gather_cells(tsf._ptr(d_rad), X, Y, Z, tsf._ptr(d_cells), len(cells), tsf._ptr(d_vals), None) == 0
    got = d_vals.cpu().numpy()
    assert np.array_equal(got[:500], rad.reshape(-1)[cells[:500]]) and not got[500:].any()
    new = rng.random(len(cells)).astype(np.float32)
    d_cl = torch.zeros((Z, Y, X), dtype=torch.int8, device="cuda")
    assert L.tsf_centerline_apply(tsf._ptr(d_cl), tsf._ptr(d_rad), X, Y, Z, tsf._ptr(d_cells),
                                  tsf._ptr(torch.from_numpy(new).cuda()), len(cells), None) == 0
    want_cl, want_rad = np.zeros(n, np.int8), rad.reshape(-1).copy()
    want_cl[cells[:500]], want_rad[cells[:500]] = 1, new[:500]
    assert np.array_equal(d_cl.cpu().numpy().reshape(-1), want_cl)
    assert np.array_equal(d_rad.cpu().numpy().reshape(-1), want_rad)
    # the centerline mark alone (no radius)
    d_cl.zero_()
    assert L.tsf_centerline_apply(tsf._ptr(d_cl), None, X, Y, Z, tsf._ptr(d_cells), None, len(cells), None) == 0
    assert np.array_equal(d_cl.cpu().numpy().reshape(-1), want_cl)
