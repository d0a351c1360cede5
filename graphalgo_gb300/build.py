"""Build recipe for libgraphalgo_gb300.so (in-tree, sm_103a only).

Compiles every CUDA translation unit under ``csrc/`` with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` in parallel, the host generator
with g++, and links them into ``graphalgo_gb300/_lib/libgraphalgo_gb300.so``.
No cmake; the result is git-ignored and rebuilt on each machine.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libgraphalgo_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build graphalgo_gb300")
    return cand


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _newest_input() -> float:
    t = 0.0
    for f in os.listdir(CSRC):
        t = max(t, os.path.getmtime(os.path.join(CSRC, f)))
    t = max(t, os.path.getmtime(os.path.join(HERE, "..", "include", "graphalgo_gb300.h")))
    return t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _newest_input():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    jobs = []
    for f in cu:
        o = os.path.join(obj_dir, f + ".o")
        cmd = [nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
               "-c", os.path.join(CSRC, f), "-o", o]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, o))
    for f in cpp:
        o = os.path.join(obj_dir, f + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-pthread", "-c",
               os.path.join(CSRC, f), "-o", o]
        jobs.append((cmd, o))

    def run(job):
        cmd, _ = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        results = list(ex.map(run, jobs))
    failed = [(c, r) for c, r in results if r.returncode != 0]
    for c, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
    if failed:
        raise RuntimeError("graphalgo_gb300 build failed:\n" + "\n".join(" ".join(c) for c, _ in failed))
    tmp = LIB_PATH + ".tmp"
    link = [nvcc, "-shared", *ARCH, "-o", tmp, *[o for _, o in jobs], "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("graphalgo_gb300 link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
