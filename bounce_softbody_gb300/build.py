"""Builds libb3g.so (the C ABI of include/b3g.h) in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``bounce_softbody_gb300/_lib/libb3g.so``. Host code is portable C++ (no intrinsics), so the
same recipe builds on x86 and on the Arm host of a GB300.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libb3g.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "kernels.cu", "batch.cu", "persistent.cu", "persistent_f32.cu", "persistent_f64.cu",
           "persistent_bf16.cu", "server.cu", "sparse.cu", "pattern.cpp", "partition.cpp", "shapes.cpp", "forces.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        extra = os.environ.get("B3G_NVCC_FLAGS", "").split()
        return common + ARCH + ["-lineinfo", "-Xptxas", "-O3", "--expt-relaxed-constexpr"] + extra
    return common


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "b3g.h"))
    deps.append(os.path.join(HERE, "..", "include", "b3g_sparse.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cc, *_flags(s), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd))

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
