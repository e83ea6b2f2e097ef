"""Build recipe of libaccrqa.so, the GB300 RQA engine (in-tree, no cmake).

CUDA translation units are compiled by nvcc for sm_103a only, host C++ by the
host compiler, in parallel; the shared library lands in ``accrqa_gb300/lib``
(git-ignored).  Objects are rebuilt when their source or any header under
``csrc/`` or ``include/`` is newer.

    python -m accrqa_gb300.build [-j N] [-v]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libaccrqa.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"),
                 "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _headers_mtime() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".hpp", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _jobs(cuda: str):
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cxx = os.environ.get("CXX", "g++")
    common_inc = ["-I", CSRC, "-I", INCLUDE, "-I", os.path.join(cuda, "include")]
    jobs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        if f.endswith(".cu"):
            obj = os.path.join(BUILD, f[:-3] + ".o")
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17",
                   "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   *common_inc, "-c", src, "-o", obj]
            jobs.append((src, obj, cmd))
        elif f.endswith(".cpp"):
            obj = os.path.join(BUILD, f[:-4] + ".o")
            cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                   "-Wall", *common_inc, "-c", src, "-o", obj]
            jobs.append((src, obj, cmd))
    return jobs


def build(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile and link libaccrqa.so; returns its path."""
    cuda = cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdr = _headers_mtime()
    todo = []
    for src, obj, cmd in _jobs(cuda):
        if (not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src)
                or os.path.getmtime(obj) < hdr):
            todo.append((src, obj, cmd))

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {os.path.basename(src)}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    n = jobs or max(1, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=n) as ex:
        list(ex.map(run, todo))

    objs = [obj for _, obj, _ in _jobs(cuda)]
    out = lib_path()
    newest = max(os.path.getmtime(o) for o in objs)
    if todo or not os.path.exists(out) or os.path.getmtime(out) < newest:
        cxx = os.environ.get("CXX", "g++")
        tmp = out + ".tmp"
        cmd = [cxx, "-shared", "-o", tmp, *objs,
               "-L", os.path.join(cuda, "lib64"), "-lcudart_static", "-lrt",
               "-lpthread", "-ldl", "-Wl,-soname," + LIBNAME]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stderr}")
        os.replace(tmp, out)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("-j", "--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.jobs, a.verbose))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
