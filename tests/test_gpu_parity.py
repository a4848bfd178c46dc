"""GPU parity: libtsf_gb300 (through its C ABI) against the oracle.

The float oracle evaluates every expression in the kernels' order with
separately rounded products and sums, and both sides use IEEE division and
square root, so the expected result is bit-identical: the tests assert exact
equality (tolerance 0).  The spec bar for FP32 fields is 1e-4 maximum
relative error; exactness is stronger.
"""
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


def _vol(synth, shape, seed):
    return synth.vascular_tree(shape, seed=seed)


def _np_stored(t, storage):
    """device tensor of stored values -> float32 numpy, using the oracle's rules."""
    import oracle as O
    a = t.detach().cpu()
    if storage == "snorm16":
        s = a.numpy().astype(np.float32)
        return np.maximum(np.float32(-1.0), s / np.float32(32767.0)).astype(np.float32)
    return a.float().numpy()


def _u16(t):
    return t.cpu().numpy().view(np.uint16)


@pytest.mark.parametrize("sigma", [0.5, 1.0, 1.5, 2.0, 2.5])
def test_blur_bitexact(torch_dev, tsf, oracle, synth, sigma):
    torch = torch_dev
    vol = _vol(synth, (20, 24, 36), 1)
    m, mask = tsf.blur_mask(sigma)
    om, omask = oracle.blur_mask(sigma)
    assert m == om and np.array_equal(mask, omask)
    out = tsf.blur(torch.from_numpy(vol).cuda(), sigma)
    assert np.array_equal(out.cpu().numpy(), oracle.blur(vol, sigma))


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("vsign", [1, -1])
def test_vector_field_bitexact(torch_dev, tsf, oracle, synth, storage, vsign):
    torch = torch_dev
    vol = oracle.blur(_vol(synth, (24, 20, 28), 2), 1.0)
    p, f4 = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, vsign, storage, planar=True, field4=True)
    ref = oracle.vector_field(vol, 0.2, vsign, storage)
    assert np.array_equal(_np_stored(f4, storage), ref)
    assert np.array_equal(_np_stored(p, storage), np.moveaxis(ref[..., :3], -1, 0))


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("mu,iters", [(0.05, 17), (0.1, 8)])
@pytest.mark.parametrize("shape", [(21, 26, 33), (19, 22, 40), (35, 9, 136), (5, 6, 8), (7, 5, 264), (6, 7, 130), (9, 10, 256),
                                   (19, 37, 136), (5, 32, 128), (21, 50, 264)])
@pytest.mark.parametrize("mode", [0, 1, 3])
def test_gvf_bitexact(torch_dev, tsf, oracle, synth, storage, mu, iters, shape, mode):
    """mode 0: the z-streaming TMA kernel wherever rows are a multiple of 16
    bytes -- tiles shifted back inside at the +x / +y edges (X = 136, 264;
    Y = 9, 22), rows shorter than a tile (X = 8, 40), z ranges split into
    several chunks (Z = 19, 35), the thinnest volumes (Z = 5); X = 33 and, for
    the 16-bit formats, X = 130 take the other kernels; taller volumes
    (Y = 32, 37, 50) cover several row tiles, the last shifted back inside.
    mode 1: the register-vector kernel (16- or 8-byte vectors, ragged last
    warps) or, for odd rows, the one-thread-per-voxel kernel.  mode 3: two
    iterations per launch where X >= 128 (X = 128, 136, 264: edge tiles shifted
    inside), with a last one-iteration launch for an odd count (17), else as
    mode 0."""
    torch = torch_dev
    vol = oracle.blur(_vol(synth, shape, 4), 0.5)
    ref4 = oracle.vector_field(vol, 0.2, 1, storage)
    p, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    v = tsf.gvf(p, mu, iters, storage, mode=mode)
    ov = oracle.gvf(ref4, mu, iters, storage)
    assert np.array_equal(_np_stored(v, storage), ov)
    assert tsf.gvf_device_error() == 0
    # the finish pass
    f4 = tsf.gvf_finish(v, storage)
    assert np.array_equal(_np_stored(f4, storage), oracle.gvf_finish(ov, storage))


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("shape", [(40, 36, 44), (30, 48, 160)])
def test_gvf_modes_identical(torch_dev, tsf, synth, oracle, storage, shape):
    """The register-vector kernel (mode 1) and the streaming kernel (modes 0
    and 2) give the same bits."""
    torch = torch_dev
    vol = oracle.blur(_vol(synth, shape, 5), 0.5)
    p, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    a = tsf.gvf(p, 0.05, 23, storage, mode=1)
    b = tsf.gvf(p, 0.05, 23, storage, mode=2)
    c = tsf.gvf(p, 0.05, 23, storage, mode=0)
    assert torch.equal(a, b) and torch.equal(a, c)
    assert tsf.gvf_device_error() == 0


@pytest.mark.parametrize("storage", ["f16", "f32"])
def test_gvf_many_waves(torch_dev, tsf, oracle, synth, storage):
    """256 tiles of 128 x 8 (X = 256, Y = 1024) fill few of the resident-CTA
    slots in one wave, so the streaming kernel cuts each tile's planes into
    several shorter z-chunks (several waves)."""
    torch = torch_dev
    vol = oracle.blur(_vol(synth, (40, 1024, 256), 6), 0.5)
    ref4 = oracle.vector_field(vol, 0.2, 1, storage)
    p, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    v = tsf.gvf(p, 0.05, 6, storage)
    assert np.array_equal(_np_stored(v, storage), oracle.gvf(ref4, 0.05, 6, storage))
    assert tsf.gvf_device_error() == 0


def test_gvf_minimum_extent(torch_dev, tsf, oracle):
    torch = torch_dev
    rng = np.random.default_rng(0)
    vol = rng.random((4, 4, 4), dtype=np.float32)
    ref4 = oracle.vector_field(vol, 0.2, 1, "f32")
    p, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, "f32")
    v = tsf.gvf(p, 0.05, 5, "f32")
    assert np.array_equal(v.cpu().numpy(), oracle.gvf(ref4, 0.05, 5, "f32"))


def _field(oracle, synth, shape, seed, storage, iters=30, mu=0.05):
    vol = oracle.blur(_vol(synth, shape, seed), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    v = oracle.gvf(f4, mu, iters, storage)
    return oracle.gvf_finish(v, storage), f4


def _to_device_field4(torch, field4, storage):
    """oracle float field4 (already stored-exact) -> device tensor of the storage dtype."""
    if storage == "f32":
        return torch.from_numpy(field4.astype(np.float32)).cuda()
    if storage == "f16":
        return torch.from_numpy(field4.astype(np.float16)).cuda()
    if storage == "bf16":
        return torch.from_numpy(field4.astype(np.float32)).to(torch.bfloat16).cuda()
    s = np.rint(field4.astype(np.float32) * np.float32(32767.0)).clip(-32768, 32767).astype(np.int16)
    return torch.from_numpy(s).cuda()


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("rng_", [(1.0, 3.0, 0.5), (2.5, 7.0, 0.5)])
@pytest.mark.parametrize("unorm", [False, True])
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_tdf_bitexact(torch_dev, tsf, oracle, synth, storage, rng_, unorm, mode):
    """Every TDF kernel (0: the default per storage format, 1: one voxel per
    lane, 2: one sample per lane, 3: load-balanced sweeps over 8^3 bricks).  X = 26 and X = 150 end in ragged bricks; both shapes hold voxels
    whose samples all lie inside (the unclamped sampler) and voxels near the
    faces (the clamped one)."""
    torch = torch_dev
    shape = (28, 30, 26) if mode == 1 or storage != "f32" else (24, 22, 150)
    field4, _ = _field(oracle, synth, shape, 6, storage)
    d4 = _to_device_field4(torch, field4, storage)
    assert np.array_equal(_np_stored(d4, storage), field4)
    T, R = tsf.tdf_circle(d4, *rng_, storage=storage, unorm16=unorm, mode=mode)
    oT, oR = oracle.tdf_circle(field4, *rng_)
    if unorm:
        assert np.array_equal(_u16(T), oracle.to_unorm16(oT))
    else:
        assert np.array_equal(T.cpu().numpy(), oT)
    assert np.array_equal(R.cpu().numpy(), oR)


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("rng_", [(1.0, 3.0, 0.5), (2.5, 7.0, 0.5), (2.5, 9.0, 0.5)])
def test_tdf_paired_texels(torch_dev, tsf, oracle, synth, storage, rng_):
    """tsf_tdf_circle_ws: for 16-bit storage the samples read the x-paired
    copy of the field (four 16-byte loads per sample) -- unclamped while the
    current radius's margin fits inside the volume, clamped to the edge near
    the faces (radii up to 9 reach past every face of a 40 x 44 x 49 volume
    from most voxels); T and R are the oracle's bit for bit, and a workspace
    that is too small or misaligned falls back to the plain path with the same
    result."""
    torch = torch_dev
    shape = (40, 44, 49)
    field4, _ = _field(oracle, synth, shape, 8, storage)
    d4 = _to_device_field4(torch, field4, storage)
    L = tsf.load()
    need = L.tsf_tdf_workspace_size(shape[2], shape[1], shape[0], tsf.STORAGE[storage])
    assert need == (0 if storage == "f32" else 16 * field4[..., 0].size)
    oT, oR = oracle.tdf_circle(field4, *rng_)
    for unorm in (False, True):
        for ws in (tsf.workspace(need), tsf.workspace(need + 64)[8:], tsf.workspace(need // 2)):
            T, R = tsf.tdf_circle(d4, *rng_, storage=storage, unorm16=unorm, ws=ws)
            if unorm:
                assert np.array_equal(_u16(T), oracle.to_unorm16(oT))
            else:
                assert np.array_equal(T.cpu().numpy(), oT)
            assert np.array_equal(R.cpu().numpy(), oR)


@pytest.mark.parametrize("unorm", [False, True])
def test_combine(torch_dev, tsf, oracle, unorm):
    torch = torch_dev
    rng = np.random.default_rng(1)
    Ts, Tl = rng.random((2, 9, 10, 11), dtype=np.float32)
    Rs, Rl = rng.random((2, 9, 10, 11), dtype=np.float32) * 7
    eT, eR = oracle.combine(Ts, Rs, Tl, Rl)
    if unorm:
        us, ul = oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)
        dTs = torch.from_numpy(us.view(np.int16)).cuda()
        dTl = torch.from_numpy(ul.view(np.int16).copy()).cuda()
        dRl = torch.from_numpy(Rl.copy()).cuda()
        tsf.tdf_combine(dTs, torch.from_numpy(Rs).cuda(), dTl, dRl, unorm16=True)
        m = us > ul
        assert np.array_equal(_u16(dTl), np.where(m, us, ul))
        assert np.array_equal(dRl.cpu().numpy(), np.where(m, Rs, Rl))
    else:
        dTl = torch.from_numpy(Tl.copy()).cuda()
        dRl = torch.from_numpy(Rl.copy()).cuda()
        tsf.tdf_combine(torch.from_numpy(Ts).cuda(), torch.from_numpy(Rs).cuda(), dTl, dRl)
        assert np.array_equal(dTl.cpu().numpy(), eT)
        assert np.array_equal(dRl.cpu().numpy(), eR)


@pytest.mark.parametrize("shape", [(8, 8, 8), (13, 17, 30), (40, 9, 21), (64, 64, 64)])
def test_compaction_order(torch_dev, tsf, oracle, shape):
    """Ballot + scan compaction reproduces the pyramid enumeration exactly."""
    torch = torch_dev
    rng = np.random.default_rng(7)
    m = (rng.random(shape) < 0.07).astype(np.int8)
    pos = tsf.compact_mask(torch.from_numpy(m).cuda())
    assert np.array_equal(pos.cpu().numpy(), oracle.hp_compact(m))


def test_compaction_empty_and_full(torch_dev, tsf, oracle):
    torch = torch_dev
    z = np.zeros((12, 8, 16), np.int8)
    assert tsf.compact_mask(torch.from_numpy(z).cuda()).shape[0] == 0
    o = np.ones((12, 8, 16), np.int8)
    assert np.array_equal(tsf.compact_mask(torch.from_numpy(o).cuda()).cpu().numpy(), oracle.hp_compact(o))


@pytest.mark.parametrize("storage,unorm", [("f32", False), ("snorm16", True), ("f16", False)])
def test_candidates_bitexact(torch_dev, tsf, oracle, synth, storage, unorm):
    torch = torch_dev
    field4, _ = _field(oracle, synth, (48, 48, 48), 8, storage, iters=40)
    oT, oR = oracle.tdf_circle(field4, 1.0, 7.0, 0.5)
    T_used = oracle.from_unorm16(oracle.to_unorm16(oT)) if unorm else oT
    ref = oracle.centerpoints(T_used, oR, field4, tdf_high=0.3, cube_size=3)
    d4 = _to_device_field4(torch, field4, storage)
    if unorm:
        dT = torch.from_numpy(oracle.to_unorm16(oT).view(np.int16)).cuda()
    else:
        dT = torch.from_numpy(oT).cuda()
    out = tsf.candidates(dT, torch.from_numpy(oR).cuda(), d4, storage, 0.3, 3, unorm16=unorm,
                         want_centerpoints=True, want_candidates=True, raise_on_range=False)
    assert out["n_candidates"] == len(ref["candidates"])
    assert np.array_equal(out["candidates"].cpu().numpy(), ref["candidates"])
    assert np.array_equal(out["centerpoints"].cpu().numpy(), ref["mask2"])
    assert out["n_vertices"] == len(ref["vertices"])
    assert np.array_equal(out["vertices"].cpu().numpy(), ref["vertices"])


def test_candidates_count_range_error(torch_dev, tsf, oracle, synth):
    torch = torch_dev
    field4, _ = _field(oracle, synth, (16, 16, 16), 9, "f32", iters=4)
    T = torch.zeros((16, 16, 16), dtype=torch.float32, device="cuda")
    R = torch.ones_like(T)
    with pytest.raises(tsf.TSFError, match="TSF_ERR_COUNT_RANGE"):
        tsf.candidates(T, R, _to_device_field4(torch, field4, "f32"), "f32", 0.5, 4)


@pytest.mark.parametrize("storage", ["f32", "snorm16", "f16"])
@pytest.mark.parametrize("shape", [(32, 32, 32), (28, 32, 36), (24, 20, 40)])
def test_fmg_bitexact(torch_dev, tsf, oracle, synth, storage, shape):
    torch = torch_dev
    vol = oracle.blur(_vol(synth, shape, 10), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    ref = oracle.fmg_gvf(f4, 0.2, 2, storage)
    out = tsf.gvf_fmg(_to_device_field4(torch, f4, storage), 0.2, 2, storage)
    assert np.array_equal(_np_stored(out, storage), ref)


def test_invalid_arguments(torch_dev, tsf):
    torch = torch_dev
    v = torch.zeros((3, 3, 3), device="cuda")
    with pytest.raises(tsf.TSFError, match="TSF_ERR_INVALID_ARG"):
        tsf.blur(v, 1.0)
    f0 = torch.zeros((3, 8, 8, 8), device="cuda")
    with pytest.raises(tsf.TSFError, match="TSF_ERR_WORKSPACE"):
        tsf.gvf(f0, 0.05, 3, "f32", ws=torch.zeros(16, dtype=torch.uint8, device="cuda"))


@pytest.mark.parametrize("storage", ["f16", "f32"])
def test_gvf_on_two_devices(torch_dev, tsf, oracle, synth, storage):
    """The streaming kernel's shared-memory attribute and occupancy figures
    are kept per device: GVF on a second GPU of the same process, after the
    first, gives the oracle's bits.  Skips with fewer than two GPUs."""
    torch = torch_dev
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    vol = oracle.blur(_vol(synth, (20, 24, 64), 11), 0.5)
    ov = oracle.gvf(oracle.vector_field(vol, 0.2, 1, storage), 0.05, 9, storage)
    for dev in (0, 1):
        with torch.cuda.device(dev):
            p, _ = tsf.vector_field(torch.from_numpy(vol).to(f"cuda:{dev}"), 0.2, 1, storage)
            v = tsf.gvf(p, 0.05, 9, storage)
            torch.cuda.synchronize()
            assert np.array_equal(_np_stored(v, storage), ov)


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("shape,iters", [((5, 8, 128), 4), ((12, 20, 136), 9), ((40, 1024, 256), 6),
                                          ((33, 37, 264), 10), ((130, 24, 128), 6)])
def test_gvf_two_iterations_per_launch(torch_dev, tsf, oracle, synth, storage, shape, iters):
    """The temporal-blocking kernel (tsf_gvf_mode 3): the thinnest volume
    (Z = 5), edge tiles shifted back inside in x and y, z-chunks over many
    waves (Y = 1024), a long z range (Z = 130); even and odd counts."""
    torch = torch_dev
    vol = oracle.blur(_vol(synth, shape, 12), 0.5)
    ref4 = oracle.vector_field(vol, 0.2, 1, storage)
    p, _ = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage)
    tsf.gvf_device_error()
    v = tsf.gvf(p, 0.05, iters, storage, mode=3)
    assert np.array_equal(_np_stored(v, storage), oracle.gvf(ref4, 0.05, iters, storage))
    assert tsf.gvf_device_error() == 0


@pytest.mark.parametrize("src", STORAGES)
@pytest.mark.parametrize("dst", STORAGES)
def test_convert_field(torch_dev, tsf, oracle, src, dst):
    """tsf_convert_field: each stored value as it reads, rounded to the target
    format -- the oracle's quantisation of the read value."""
    torch = torch_dev
    rng = np.random.default_rng(4)
    a = np.concatenate([rng.uniform(-1.2, 1.2, 5000), [0.0, -0.0, 1.0, -1.0, 1e-7, 3e-5]]).astype(np.float32)
    a = oracle.quantize(a, src)
    if src == "snorm16":
        t = torch.from_numpy(np.rint(a.astype(np.float64) * 32767).astype(np.int16)).cuda()
    elif src == "bf16":
        t = torch.from_numpy(a).to(torch.bfloat16).cuda()
    else:
        t = torch.from_numpy(a.astype(np.float16 if src == "f16" else np.float32)).cuda()
    out = tsf.convert_field(t, src, dst)
    assert np.array_equal(_np_stored(out, dst), oracle.quantize(a, dst))
