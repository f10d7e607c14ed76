"""Build the CUDA library libsg.so (sm_103a) in-tree.

Each translation unit is compiled by nvcc in parallel, then linked into
specfem3d_geotech_gb300/_lib/libsg.so.  No cmake, no torch extension
machinery: the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libsg.so")
SOURCES = ["sg_kernels.cu", "sg_api.cu", "sg_host_mesh.cu", "sg_noalloc.cu", "sg_serve.cu", "sg_apply_tc.cu",
           "sg_apply_lanes.cu", "sg_apply_mf.cu",
           "sg_output.cu", "sg_pcg_persist.cu"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def _needs(obj: str, srcs) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "sg_solver.h"))
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        if force or _needs(o, [s] + headers):
            jobs.append([NVCC, *FLAGS, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(r.args))
            if verbose and (r.stdout or r.stderr):
                sys.stderr.write(r.stdout + r.stderr)
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        r = subprocess.run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", LIB,
                            "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
