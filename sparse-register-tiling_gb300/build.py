"""Build libspreg.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Usage: python sparse-register-tiling_gb300/build.py [--force]

Every translation unit under csrc/ is compiled by nvcc in parallel into _build/, then linked
(with the CUDA runtime linked statically) into spreg/libspreg.so.  Rebuilds only what changed.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "spreg", "libspreg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
    "-I", INCLUDE,
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libspreg.so")


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return [src] + hdrs + [os.path.join(INCLUDE, "spreg.h")]


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


# Executor instantiations: one generated translation unit per (M_r, dtype combination).
EXEC_MR = (2, 4, 6, 8)
EXEC_COMBOS = (0, 1, 2, 3)  # ExecCombo in csrc/exec_kernel.cuh


def _gen_exec_units() -> list[str]:
    out = []
    for mr in EXEC_MR:
        for c in EXEC_COMBOS:
            path = os.path.join(BUILD, f"exec_mr{mr}_c{c}.cu")
            text = (f'// generated by build.py: executor kernels for M_r = {mr}, dtype combination {c}\n'
                    f'#include "{os.path.join(CSRC, "exec_tile.cuh")}"\n'
                    f'namespace spreg {{ SPREG_INSTANTIATE_EXEC({mr}, {c}) SPREG_INSTANTIATE_TILE({mr}, {c}) }}\n')
            if not os.path.exists(path) or open(path).read() != text:
                with open(path, "w") as f:
                    f.write(text)
            out.append(path)
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu")) + _gen_exec_units()
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, _deps(src)):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), max(os.cpu_count() or 4, 4))) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(OUT) or any(os.path.getmtime(o) > os.path.getmtime(OUT) for o in objs):
        run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", OUT, *objs])
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
