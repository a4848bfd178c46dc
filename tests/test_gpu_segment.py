"""GPU tests of the segmentation (tsf_segment_inverse_gradient,
tsf_segment_spheres) against the oracle, bit for bit: the grown and closed
mask and the number of grow iterations, in every storage format, on the
linked centerlines of a vessel phantom and on random fields, odd extents and
centerlines touching the borders."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STORAGES = ["f32", "f16", "bf16", "snorm16"]


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _to_device_field4(torch, field4, storage):
    """float field4 holding stored-exact values -> device tensor of the storage dtype."""
    if storage == "f32":
        return torch.from_numpy(field4.astype(np.float32)).cuda()
    if storage == "f16":
        return torch.from_numpy(field4.astype(np.float16)).cuda()
    if storage == "bf16":
        return torch.from_numpy(field4.astype(np.float32)).to(torch.bfloat16).cuda()
    s = np.rint(field4.astype(np.float32) * np.float32(32767.0)).clip(-32768, 32767).astype(np.int16)
    return torch.from_numpy(s).cuda()


@pytest.fixture(scope="module")
def phantom(oracle, synth):
    """A 64^3 vessel tree: the blurred volume, radius and linked centerlines."""
    shape = (64, 64, 64)
    vol = oracle.blur(synth.vascular_tree(shape, seed=11), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1, "f32")
    field = oracle.gvf_finish(oracle.gvf(f4, 0.05, 60, "f32"), "f32")
    T, R = oracle.tdf_circle(field, 1.0, 7.0, 0.5)
    ref = oracle.centerpoints(T, R, field, tdf_high=0.3, cube_size=3)
    verts = ref["vertices"]
    edges, labels, sizes = oracle.link_centerpoints(verts, T, 0.3, 15.0)
    cl = oracle.rasterize_trees(verts, edges, labels, sizes, 5, shape)
    assert cl.sum() > 50
    return vol, R, cl


def _case(tsf, torch, cl, F, R, storage):
    d_cl = torch.from_numpy(np.ascontiguousarray(cl, dtype=np.int8)).cuda()
    d_F = _to_device_field4(torch, F, storage)
    d_R = torch.from_numpy(np.ascontiguousarray(R, dtype=np.float32)).cuda()
    return tsf.segment_inverse_gradient(d_cl, d_F, d_R, storage=storage)


@pytest.mark.parametrize("storage", STORAGES)
def test_inverse_gradient_phantom(torch_dev, tsf, oracle, phantom, storage):
    vol, R, cl = phantom
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    F = oracle.gvf_finish(oracle.gvf(f4, 0.05, 40, storage), storage)
    seg, it = _case(tsf, torch_dev, cl, F, R, storage)
    ref, rit = oracle.segment_inverse_gradient(cl, F, R)
    assert rit > 2 and ref.sum() > cl.sum()
    assert it == rit
    assert np.array_equal(seg.cpu().numpy(), ref)


def _random_field(rng, shape, storage, oracle):
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    w = rng.random(shape).astype(np.float32)
    n = np.sqrt((v * v).sum(-1))
    F = np.concatenate([v / n[..., None] * w[..., None], w[..., None]], -1).astype(np.float32)
    return oracle.quantize(F, storage)


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("shape,p_cl", [((20, 24, 33), 0.02), ((37, 29, 45), 0.005), ((4, 5, 6), 0.1)])
def test_inverse_gradient_random(torch_dev, tsf, oracle, storage, shape, p_cl):
    rng = np.random.default_rng(sum(shape))
    cl = (rng.random(shape) < p_cl).astype(np.int8)
    cl[0, 0, 0] = cl[-1, -1, -1] = cl[0, -1, 3 % shape[2]] = 1      # border centerline voxels
    F = _random_field(rng, shape, storage, oracle)
    R = (rng.random(shape) * 9.0).astype(np.float32)
    seg, it = _case(tsf, torch_dev, cl, F, R, storage)
    ref, rit = oracle.segment_inverse_gradient(cl, F, R)
    assert it == rit
    assert np.array_equal(seg.cpu().numpy(), ref)


def test_inverse_gradient_radial(torch_dev, tsf, oracle):
    """Field pointing at the axis with magnitude peaking at distance 6: many
    grow iterations (more than one batch between flag reads)."""
    Z, Y, X = 16, 40, 40
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    dy, dx = (yy - 19.5).astype(np.float32), (xx - 19.5).astype(np.float32)
    d = np.sqrt(dx * dx + dy * dy)
    w = np.where(d <= 16.0, d / 16.0, np.maximum(0.0, 1.0 - (d - 16.0))).astype(np.float32)
    F = np.stack([-dx / d * w, -dy / d * w, np.zeros_like(d), w], -1).astype(np.float32)
    cl = np.zeros((Z, Y, X), np.int8)
    cl[:, 19:21, 19:21] = 1
    R = np.full((Z, Y, X), 2.0, np.float32)
    seg, it = _case(tsf, torch_dev, cl, F, R, "f32")
    ref, rit = oracle.segment_inverse_gradient(cl, F, R)
    assert rit > 8 and it == rit
    assert np.array_equal(seg.cpu().numpy(), ref)


def test_inverse_gradient_empty(torch_dev, tsf):
    torch = torch_dev
    cl = torch.zeros((8, 9, 10), dtype=torch.int8, device="cuda")
    F = torch.ones((8, 9, 10, 4), dtype=torch.float32, device="cuda")
    R = torch.ones((8, 9, 10), dtype=torch.float32, device="cuda")
    seg, it = tsf.segment_inverse_gradient(cl, F, R)
    assert it == 1 and int(seg.sum()) == 0


@pytest.mark.parametrize("shape,rmax", [((20, 24, 33), 4.0), ((37, 29, 45), 9.0), ((64, 64, 64), 2.5)])
def test_spheres(torch_dev, tsf, oracle, shape, rmax):
    torch = torch_dev
    rng = np.random.default_rng(int(rmax * 10))
    cl = (rng.random(shape) < 0.003).astype(np.int8)
    cl[0, 0, 0] = cl[-1, -1, -1] = 1
    R = (rng.random(shape) * rmax).astype(np.float32)
    out = tsf.segment_spheres(torch.from_numpy(cl).cuda(), torch.from_numpy(R).cuda())
    assert np.array_equal(out.cpu().numpy(), oracle.segment_spheres(cl, R))


def test_segment_invalid_arguments(torch_dev, tsf):
    torch = torch_dev
    cl = torch.zeros((8, 8, 8), dtype=torch.int8, device="cuda")
    F = torch.zeros((8, 8, 8, 4), dtype=torch.float32, device="cuda")
    R = torch.zeros((8, 8, 8), dtype=torch.float32, device="cuda")
    L = tsf.load()
    need = L.tsf_segment_workspace_size(8, 8, 8)
    ws = torch.empty(need - 1, dtype=torch.uint8, device="cuda")
    out = torch.empty((8, 8, 8), dtype=torch.int8, device="cuda")
    code = L.tsf_segment_inverse_gradient(cl.data_ptr(), F.data_ptr(), 0, R.data_ptr(), 8, 8, 8, out.data_ptr(),
                                          None, ws.data_ptr(), need - 1, None)
    assert code == 3                               # TSF_ERR_WORKSPACE
    assert L.tsf_segment_spheres(cl.data_ptr(), R.data_ptr(), 3, 8, 8, out.data_ptr(), None) == 1
