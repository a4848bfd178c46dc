"""Writes tests/golden/reference_*.npz: outputs of the reference's own kernel
text (kernels.cl compiled for the CPU under the OpenCL C shim, oracle/ref.py)
on small seeded vessel-tree volumes, for the GPU tests to compare with
(tests/test_gpu_golden.py).  Needs the reference source tree
($TSF_REFERENCE_DIR, default /root/reference).

    python tests/golden/make_golden.py

Per case (field format f32 = CL_FLOAT or snorm16 = CL_SNORM_INT16, the
reference's two): the input volume; the blur (sigma 0.5, the mask of
createBlurMask); the vector fields of the blurred and of the raw volume
(Fmax 0.2, white tubes); GVF (mu 0.05, 20 iterations: GVF3DInit,
GVF3DIteration x 20, GVF3DFinish); the small-radius TDF (r 1..3 on the raw
volume's field) and the large-radius TDF (r 2.5..7 on the GVF field), combined;
the candidate stage (threshold 0.3, cube 3): candidate list, filtered mask,
vertex list.  TDF stored as float (f32 case) or unorm16 (snorm16 case, the
reference's 16-bit mode).  Stored fields are written in their storage type.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tube-segmentation-framework_gb300")]

import oracle as O  # noqa: E402  (host-side blur mask only)
import ref as R  # noqa: E402
import synthetic  # noqa: E402

SHAPE = (16, 20, 24)
P = dict(seed=12, sigma=0.5, fmax=0.2, vsign=1, mu=0.05, iterations=20, tdf_high=0.3, cube=3)


def stored(a, storage):
    if storage == "snorm16":   # values are exact multiples of 1/32767
        return np.rint(a.astype(np.float64) * 32767.0).astype(np.int16)
    return a.astype(np.float32)


def case(storage):
    unorm = storage == "snorm16"
    vol = synthetic.vascular_tree(SHAPE, seed=P["seed"])
    m, mask = O.blur_mask(P["sigma"])
    b = R.blur(vol, m, mask)
    f4 = R.vector_field(b, P["fmax"], P["vsign"], storage)
    fs = R.vector_field(vol, P["fmax"], P["vsign"], storage)
    v, fin = R.gvf(f4, P["mu"], P["iterations"], storage)
    Ts, Rs = R.tdf_circle(fs, 1.0, 3.0, 0.5, storage, unorm)
    Tl, Rl = R.tdf_circle(fin, 2.5, 7.0, 0.5, storage, unorm)
    T, Rr = R.combine(Ts, Rs, Tl, Rl)
    c = R.candidates(T, Rr, fin, storage, P["tdf_high"], P["cube"])
    return dict(volume=vol, blurred=b, field=stored(f4, storage), field_small=stored(fs, storage),
                gvf=stored(np.moveaxis(v[..., :3], -1, 0), storage), gvf_field=stored(fin, storage),
                T_small=Ts, R_small=Rs, T=T, R=Rr, candidates=c["candidates"], mask2=c["mask2"],
                vertices=c["vertices"], params=np.array([P[k] for k in sorted(P)], np.float64),
                param_names=np.array(sorted(P)))


def main():
    for storage in ("f32", "snorm16"):
        d = case(storage)
        path = os.path.join(HERE, "reference_%s.npz" % storage)
        np.savez_compressed(path, **d)
        print(path, os.path.getsize(path), "bytes;", len(d["candidates"]), "candidates,",
              len(d["vertices"]), "vertices")


if __name__ == "__main__":
    main()
