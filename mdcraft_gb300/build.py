"""Builds libmdg.so (the C-ABI of include/mdg.h) for sm_103a, in-tree.

Each .cu translation unit is compiled in parallel with nvcc, then linked into
mdcraft_gb300/_build/libmdg.so. Host code is compiled without FP contraction
so the spline set-up matches the reference's host arithmetic bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmdg.so")
SOURCES = ["nlist.cu", "forces.cu", "integrate.cu", "capi.cu", "measure_static.cu", "serve.cu", "solo.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libmdg needs the CUDA toolkit (sm_103a)")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-Xptxas", "-O3", "--expt-relaxed-constexpr", *extra]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "mdg.h"))
    return os.path.getmtime(obj) < max(os.path.getmtime(d) for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(SRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        if force or _stale(obj, src):
            jobs.append([cc, *_flags(extra), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stderr or r.stdout):
            print(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB):
        run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True, extra=["-Xptxas", "-v"] if "-v" in sys.argv else []))
