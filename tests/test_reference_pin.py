"""The oracle pinned to the reference's own kernel text.

oracle/_ref is the reference's kernels.cl compiled for the CPU under an
OpenCL C shim (oracle/clshim/) and driven in the order of the reference's host
code (ref.py).  These tests run the oracle (the C restatement the GPU parity
tests compare with) and the reference's text on the same seeded volumes and
require identical results, bit for bit, stage by stage: blur, vector field,
GVF (init, iterations, finish), circle-fitting TDF in both TDF formats,
combine, the candidate stage (candidate list in pyramid order, filtered
mask, vertex list) and the eigen-decomposition.  Field formats: the
reference's two, CL_FLOAT and CL_SNORM_INT16.

What the shim restates rather than takes from the reference: the OpenCL
runtime's image sampling and format conversions (from the OpenCL 1.1
specification) and the histogram-pyramid host class (OpenCLUtilityLibrary,
not part of the reference's source).  They skip where the reference source
tree is absent (the GPU machines).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(reference_dir):
    import ref as R
    R.build()
    return R


def _vol(synth, shape, seed):
    return synth.vascular_tree(shape, seed=seed)


@pytest.mark.parametrize("sigma", [0.5, 1.0, 2.0])
def test_blur_matches_reference(ref, oracle, synth, sigma):
    vol = _vol(synth, (14, 17, 19), 1)
    m, mask = oracle.blur_mask(sigma)
    assert np.array_equal(ref.blur(vol, m, mask), oracle.blur(vol, sigma))


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
@pytest.mark.parametrize("vsign", [1, -1])
def test_vector_field_matches_reference(ref, oracle, synth, storage, vsign):
    vol = oracle.blur(_vol(synth, (15, 18, 21), 2), 1.0)
    assert np.array_equal(ref.vector_field(vol, 0.2, vsign, storage), oracle.vector_field(vol, 0.2, vsign, storage))


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
@pytest.mark.parametrize("mu,iters", [(0.05, 12), (0.1, 8), (0.05, 7)])
@pytest.mark.parametrize("shape", [(13, 16, 22), (6, 5, 9)])
def test_gvf_matches_reference(ref, oracle, synth, storage, mu, iters, shape):
    """Jacobi iterations with the mirror rule; for an odd count the
    reference's host loop hands the finish pass the result of one iteration
    fewer (the ping-pong ends in the other image)."""
    vol = oracle.blur(_vol(synth, shape, 3), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    rv, rfin = ref.gvf(f4, mu, iters, storage)
    k = iters if iters % 2 == 0 else iters - 1
    ov = oracle.gvf(f4, mu, k, storage)
    assert np.array_equal(np.moveaxis(rv[..., :3], -1, 0), ov)
    # w carries f0z, copied from the evaluated (mirrored) voxel
    m = [np.array([2 if i == 0 else (n - 3 if i >= n - 1 else i) for i in range(n)]) for n in f4.shape[:3]]
    assert np.array_equal(rv[..., 3], f4[..., 2][np.ix_(*m)])
    assert np.array_equal(rfin, oracle.gvf_finish(ov, storage))


def _field(oracle, synth, shape, seed, storage, iters=16):
    vol = oracle.blur(_vol(synth, shape, seed), 0.5)
    f4 = oracle.vector_field(vol, 0.2, 1, storage)
    return oracle.gvf_finish(oracle.gvf(f4, 0.05, iters, storage), storage)


@pytest.mark.parametrize("storage", ["f32", "snorm16"])
@pytest.mark.parametrize("rng_", [(1.0, 3.0, 0.5), (2.5, 7.0, 0.5), (1.0, 7.0, 0.5)])
def test_tdf_matches_reference(ref, oracle, synth, storage, rng_):
    field = _field(oracle, synth, (20, 22, 24), 6, storage)
    oT, oR = oracle.tdf_circle(field, *rng_)
    rT, rR = ref.tdf_circle(field, *rng_, storage=storage)
    assert np.array_equal(rT, oT)
    assert np.array_equal(rR, oR)
    uT, uR = ref.tdf_circle(field, *rng_, storage=storage, unorm16=True)
    assert np.array_equal(uT, oracle.to_unorm16(oT))
    assert np.array_equal(uR, oR)


def test_combine_matches_reference(ref, oracle):
    rng = np.random.default_rng(3)
    Ts, Tl = rng.random((2, 6, 7, 8), dtype=np.float32)
    Rs, Rl = rng.random((2, 6, 7, 8), dtype=np.float32) * 7
    for a, b in zip(ref.combine(Ts, Rs, Tl, Rl), oracle.combine(Ts, Rs, Tl, Rl)):
        assert np.array_equal(a, b)
    uT, uR = ref.combine(oracle.to_unorm16(Ts), Rs, oracle.to_unorm16(Tl), Rl)
    assert np.array_equal(uT, np.maximum(oracle.to_unorm16(Ts), oracle.to_unorm16(Tl)))


@pytest.mark.parametrize("storage,unorm", [("f32", False), ("snorm16", True), ("f32", True)])
@pytest.mark.parametrize("shape,cube", [((40, 40, 40), 3), ((36, 28, 44), 4)])
def test_candidates_match_reference(ref, oracle, synth, storage, unorm, shape, cube):
    field = _field(oracle, synth, shape, 8, storage, iters=30)
    oT, oR = oracle.tdf_circle(field, 1.0, 7.0, 0.5)
    T_read = oracle.from_unorm16(oracle.to_unorm16(oT)) if unorm else oT
    want = oracle.centerpoints(T_read, oR, field, tdf_high=0.3, cube_size=cube)
    got = ref.candidates(oracle.to_unorm16(oT) if unorm else oT, oR, field, storage, 0.3, cube)
    assert len(want["candidates"]) > 0 and len(want["vertices"]) > 0
    assert np.array_equal(got["candidates"], want["candidates"])
    assert np.array_equal(got["mask2"], want["mask2"])
    assert np.array_equal(got["vertices"], want["vertices"])


def test_eigen_matches_reference(ref, oracle):
    """Random symmetric matrices, diagonal ones, repeated and zero
    eigenvalues, a nearly singular one."""
    rng = np.random.default_rng(5)
    A = rng.normal(size=(400, 3, 3)).astype(np.float32)
    A = (A + np.transpose(A, (0, 2, 1))).astype(np.float32)
    D = np.zeros((6, 3, 3), np.float32)
    D[0] = np.diag([1, 2, 3]); D[1] = np.diag([3, -1, 2]); D[2] = np.diag([1, 1, 1])
    D[3] = np.diag([0, 0, 0]); D[4] = [[2, 1, 0], [1, 2, 0], [0, 0, 2]]; D[5] = [[1e-8, 0, 0], [0, 1, 0], [0, 0, -1]]
    A = np.concatenate([A, D])
    V, d = ref.eigen(A)
    for i in range(A.shape[0]):
        od, oV = oracle.eig3(A[i])
        assert np.array_equal(d[i], od), i
        assert np.array_equal(V[i], oV), i
