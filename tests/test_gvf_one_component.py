"""The low-memory GVF (runLowMemoryGVF, gradientVectorFlow.cpp:1172-1300;
GVF3D{Init,Iteration,Finish}_one_component, kernels_no_3d_write.cl:1669-1741
and kernels.cl:1392-1462).

No GPU: the oracle's restatement is pinned against a pure-Python restatement
of the three kernel texts on a small volume in every storage format, and, with
FP32 storage, against the three-component GVF (identical by construction: only
the stored |f0|^2 differs, and FP32 stores it exactly).
GPU: tsf_gvf_one_component against the oracle, bit for bit -- rows that split
into 16-byte vectors (X = 136: a ragged last warp; X = 256: whole warps) and
rows that do not (X = 12 for 16-bit formats, 33)."""
import numpy as np
import pytest

STORAGES = ["f32", "f16", "bf16", "snorm16"]


def _py_one_component(oracle, field4, mu, iters, storage):
    f32 = np.float32
    Q = lambda a: oracle.quantize(np.asarray(a, np.float32), storage)
    Z, Y, X = field4.shape[:3]
    mirror = lambda w, n: 2 if w == 0 else (n - 3 if w >= n - 1 else w)
    sq = Q((field4[..., 0] * field4[..., 0] + field4[..., 1] * field4[..., 1]) + field4[..., 2] * field4[..., 2])
    out = []
    for c in range(3):
        f = Q(field4[..., c])
        v = f.copy()
        for _ in range(iters):
            w = np.empty_like(v)
            for z in range(Z):
                for y in range(Y):
                    for x in range(X):
                        px, py, pz = mirror(x, X), mirror(y, Y), mirror(z, Z)
                        vv = v[pz, py, px]
                        lap = f32(-6) * vv
                        for (a, b, d) in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                            lap = f32(lap + v[pz + d, py + b, px + a])
                        upd = f32(f32(mu) * lap) - f32(f32(vv - f[pz, py, px]) * sq[pz, py, px])
                        w[z, y, x] = f32(vv + upd)
            v = Q(w)
        out.append(v)
    x, y, z = out
    length = np.sqrt((x * x + y * y) + z * z, dtype=np.float32)
    return np.stack([x, y, z, Q(np.where(length > 0, length, np.float32(1)))], axis=-1)


def _field(oracle, shape, storage, seed=0):
    rng = np.random.default_rng(seed)
    vol = oracle.blur(rng.random(shape, dtype=np.float32), 1.0)
    return oracle.vector_field(vol, 0.2, 1, storage)


@pytest.mark.parametrize("storage", STORAGES)
def test_oracle_matches_kernel_text(oracle, storage):
    f4 = _field(oracle, (5, 6, 7), storage)
    want = _py_one_component(oracle, f4, 0.05, 3, storage)
    assert np.array_equal(oracle.gvf_one_component(f4, 0.05, 3, storage), want)


def test_fp32_equals_three_component_gvf(oracle):
    f4 = _field(oracle, (12, 14, 18), "f32", seed=1)
    a = oracle.gvf_one_component(f4, 0.05, 9, "f32")
    b = oracle.gvf_finish(oracle.gvf(f4, 0.05, 9, "f32"), "f32")
    assert np.array_equal(a, b)


@pytest.mark.parametrize("storage", ["f16", "snorm16"])
def test_16bit_differs_only_by_the_stored_square(oracle, storage):
    """In 16-bit formats the stored |f0|^2 is rounded: close to the
    three-component result, not equal."""
    f4 = _field(oracle, (12, 14, 18), storage, seed=2)
    a = oracle.gvf_one_component(f4, 0.05, 9, storage)
    b = oracle.gvf_finish(oracle.gvf(f4, 0.05, 9, storage), storage)
    assert np.abs(a - b).max() < 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("shape", [(9, 10, 12), (20, 17, 33), (6, 40, 136), (7, 12, 256)])
def test_gpu_bitexact(tsf, oracle, storage, shape):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(3)
    vol = oracle.blur(rng.random(shape, dtype=np.float32), 1.0)
    _, f4 = tsf.vector_field(torch.from_numpy(vol).cuda(), 0.2, 1, storage, planar=True, field4=True)
    out = tsf.gvf_one_component(f4, 0.05, 11, storage)
    want = oracle.gvf_one_component(oracle.vector_field(vol, 0.2, 1, storage), 0.05, 11, storage)
    a = out.cpu()
    if storage == "snorm16":
        got = np.maximum(np.float32(-1.0), a.numpy().astype(np.float32) / np.float32(32767.0))
    else:
        got = a.float().numpy()
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_gpu_fp32_equals_tsf_gvf(tsf, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    rng = np.random.default_rng(4)
    vol = torch.from_numpy(oracle.blur(rng.random((16, 24, 40), dtype=np.float32), 1.0)).cuda()
    p, f4 = tsf.vector_field(vol, 0.2, 1, "f32", planar=True, field4=True)
    a = tsf.gvf_one_component(f4, 0.05, 20, "f32")
    b = tsf.gvf_finish(tsf.gvf(p, 0.05, 20, "f32"), "f32")
    assert torch.equal(a, b)
