"""Build libgrmp_gpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel; the objects go to ``_build/``
next to this file and the shared library to ``libgrmp_gpu.so`` beside it.
Host code is compiled without FMA contraction (-ffp-contract=off) so that the
quadrature / basis tables agree bit for bit on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgrmp_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cpp", "tables.cpp", "server.cpp", "nd_symbolic.cpp", "pattern.cu", "assemble.cu", "br.cu", "solve.cu",
           "batch.cu", "multifrontal.cu", "integrate.cu", "br3.cu", "topology.cu", "duo.cpp", "import.cu",
           "p2b.cu", "nonlinear.cu", "faces.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgrmp_gpu.so")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "grmp.h"))
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(HERE, "..", "include")] + ARCH + list(extra_flags or [])
    jobs = []
    objs = []
    for src in _sources():
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [sp] + headers):
            cmd = [nvcc()] + common + ["-c", sp, "-o", obj]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-warn-spills"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objs):
        run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-Xcompiler", "-pthread"])
    return LIB


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv, verbose=True))
