"""Builds liblightne_gb300.so (sm_103a) in-tree with nvcc.

Each ``csrc/*.cu`` file is compiled in parallel to an object under
``_build/`` and the objects are linked into ``lightne_gb300/liblightne_gb300.so``.
The CLI binary ``lightne_gb300/bin/LightNE`` is linked against it.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build", "lib")
LIB = os.path.join(HERE, "liblightne_gb300.so")
CLI = os.path.join(HERE, "bin", "LightNE")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-O2", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, headers, verbose: bool) -> str:
    if not _stale(obj, [src] + headers):
        return obj
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int = 8) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                     glob.glob(os.path.join(ROOT, "include", "*.h")))
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], headers, verbose), zip(srcs, objs)))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    cli_src = os.path.join(CSRC, "cli", "lightne_main.cpp")
    if os.path.exists(cli_src):
        os.makedirs(os.path.dirname(CLI), exist_ok=True)
        if _stale(CLI, [cli_src, LIB] + headers):
            cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), cli_src, "-o", CLI,
                   "-L", HERE, "-llightne_gb300", "-Wl,-rpath,$ORIGIN/..", "-lm"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("CLI build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
