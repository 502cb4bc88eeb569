"""Build libimsrg_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in its own nvcc process (in parallel), then one link
step produces eom-imsrg_gb300/lib/libimsrg_gb300.so.  The library links the CUDA
runtime statically and exports only the C ABI of include/imsrg_gb300.h.
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
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libimsrg_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]
SOURCES = ["layout.cpp", "gemm_plan.cpp", "hamiltonian.cpp", "engine.cu", "kernels_fp64.cu", "kernels_ops.cu",
           "gemm_fp64.cu", "gemm_tc.cu", "kernels_mixed.cu", "recouple.cu", "comm122.cu", "noalloc.cu", "graph.cu", "adjoint.cu", "kernels_adjoint.cu", "tensor_layout.cpp", "tensor.cu", "hf.cu", "pair_groups.cpp", "checkpoint.cpp",
           "kernels_tensor.cu", "eom.cu", "triples.cu", "quads.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "imsrg_gb300.h"))
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if force or _needs(obj, [path] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append(([nv] + ARCH + FLAGS + list(extra) + lang + ["-c", path, "-o", obj], src))

    def run(job):
        cmd, src = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"nvcc failed on {src}")
        return src

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s + ".o") for s in SOURCES]
    if force or jobs or _needs(LIB, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-ldl", "-lpthread", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
