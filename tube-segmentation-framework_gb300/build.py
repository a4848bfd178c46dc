"""Build recipe of libtsf_gb300.so (sm_103a) and its C++ test driver.

Plain nvcc invocations, one translation unit per process in parallel, one
-gencode target.  Kernels are built with -fmad=false (no contraction of
products into fused multiply-adds) so that they round exactly like the
float oracle; host code gets -ffp-contract=off for the same reason.

    python build.py            # build into ./lib
    python build.py --clean
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libtsf_gb300.so")
API_TESTS = os.path.join(LIB_DIR, "tsf_api_tests")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-I", INCLUDE]

CU_SOURCES = ["capi.cu", "vector_field.cu", "gvf.cu", "gvf_zs.cu", "gvf_tb2.cu", "gvf_one.cu", "tdf.cu", "tdf_closed.cu", "candidates.cu", "fmg.cu", "noalloc.cu", "input.cu", "gvf_adjoint.cu", "gvf_adjoint_zs.cu", "tdf_adjoint.cu", "link.cu", "segment.cu", "crop.cu", "tdf_spline.cu", "residual.cu", "convert.cu"]


def _cuda_lib_dir():
    for cand in (os.path.join(os.path.dirname(os.path.dirname(NVCC)), "lib64"),
                 "/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
                 "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(cand, "libcudart.so")):
            return cand
    return "/usr/local/cuda/lib64"


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _deps():
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdr += [os.path.join(INCLUDE, "tsf", f) for f in os.listdir(os.path.join(INCLUDE, "tsf"))
            if f.endswith((".h", ".hpp"))]
    if os.path.isdir(HOST):
        hdr += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".h", ".hpp"))]
    return hdr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _newer([src] + deps, obj) or ptxas_info:
            cmd = [NVCC] + CUDA_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    if os.path.isdir(HOST):
        for f in sorted(os.listdir(HOST)):
            if not f.endswith(".cpp"):
                continue
            src = os.path.join(HOST, f)
            obj = os.path.join(BUILD, "host_" + f + ".o")
            objs.append(obj)
            if _newer([src] + deps, obj):
                jobs.append(["g++"] + CXX_FLAGS + ["-I", "/usr/local/cuda/include", "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    cudadir = _cuda_lib_dir()
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-cudart", "shared", "-lpthread", "-L", cudadir, "-Xlinker", "-rpath," + cudadir])
    # C++ test driver of the drop-in API (tests/cpp/test_api.cpp)
    src = os.path.join(ROOT, "tests", "cpp", "test_api.cpp")
    if os.path.exists(src) and _newer([src, LIB] + deps, API_TESTS):
        _run(["g++"] + CXX_FLAGS + [src, "-o", API_TESTS, "-L", LIB_DIR, "-ltsf_gb300",
                                     "-Wl,-rpath," + LIB_DIR, "-L", cudadir, "-lcudart", "-Wl,-rpath," + cudadir])
    return LIB


if __name__ == "__main__":
    if "--clean" in sys.argv:
        shutil.rmtree(BUILD, ignore_errors=True)
        shutil.rmtree(LIB_DIR, ignore_errors=True)
    else:
        print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
