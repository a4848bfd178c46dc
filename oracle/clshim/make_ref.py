"""Builds oracle/_ref/libtsf_ref.so: the reference's own OpenCL kernel source,
compiled for the CPU under the OpenCL C shim (clshim.hpp) -- test
infrastructure that pins the oracle to the reference's text.

    python make_ref.py [REFERENCE_DIR]     (default: $TSF_REFERENCE_DIR or /root/reference)

Reads REFERENCE_DIR/kernels.cl and writes, under oracle/_ref/ only:
  kernels_f.cpp / kernels_u.cpp   translation units holding the kernel text,
                                   once as is (TDF stored as float) and once
                                   with -D VECTORS_16BIT (TDF stored as
                                   unorm16), each followed by the host driver
                                   (ref_driver.inc);
  libtsf_ref.so                   both, linked with clshim.cpp.
The kernel text is taken as it is with one mechanical rewrite: OpenCL vector
literals "(float4)(a, b, c, d)" become calls "make_vec<float4>(a, b, c, d)"
(in C++ the former would be a cast of a comma expression).  Nothing of the
reference is copied into the repository; the generated files stay in the
git-ignored _ref/ folder.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT, "libtsf_ref.so")

LITERAL = re.compile(r"\(\s*((?:u?(?:char|short|int|long))|float|double)(2|3|4|8|16)\s*\)\s*\(")


def reference_dir(arg=None):
    return arg or os.environ.get("TSF_REFERENCE_DIR", "/root/reference")


def translate(src: str) -> str:
    return LITERAL.sub(lambda m: "make_vec<%s%s>(" % (m.group(1), m.group(2)), src)


def unit(kernel_text: str, sixteen: bool) -> str:
    ns = "refcl_u" if sixteen else "refcl_f"
    return "\n".join([
        "// generated by make_ref.py from the reference's kernels.cl -- do not edit",
        '#include "clshim.hpp"',
        "#define VECTORS_16BIT" if sixteen else "",
        "namespace %s {" % ns,
        '#line 1 "kernels.cl"',
        kernel_text,
        "}  // namespace %s" % ns,
        "#define REFNS %s" % ns,
        "#define REF_TDF_UNORM16 %d" % (1 if sixteen else 0),
        "#define REFFN(name) name##_%s" % ("u" if sixteen else "f"),
        '#include "ref_driver.inc"',
        "",
    ])


FLAGS = ["-O2", "-std=gnu++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-w",
         "-Wno-narrowing", "-I", HERE]


def build(ref_dir=None, force=False) -> str:
    ref = reference_dir(ref_dir)
    src_path = os.path.join(ref, "kernels.cl")
    if not os.path.exists(src_path):
        raise FileNotFoundError(src_path)
    deps = [src_path, __file__] + [os.path.join(HERE, f) for f in ("clshim.hpp", "clshim.cpp", "ref_driver.inc")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    text = translate(open(src_path).read())
    jobs = []
    objs = []
    for sixteen in (False, True):
        tu = os.path.join(OUT, "kernels_%s.cpp" % ("u" if sixteen else "f"))
        open(tu, "w").write(unit(text, sixteen))
        obj = tu[:-4] + ".o"
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + ["-c", tu, "-o", obj])
    obj = os.path.join(OUT, "clshim.o")
    objs.append(obj)
    jobs.append(["g++"] + FLAGS + ["-c", os.path.join(HERE, "clshim.cpp"), "-o", obj])

    def run(cmd):
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout[-20000:])

    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(run, jobs))
    run(["g++", "-shared", "-fopenmp", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
