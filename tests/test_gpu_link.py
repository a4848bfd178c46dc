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
