"""Build the GB300 extension liba2ds_gpu.so in-tree (a2d-shells_gb300/lib/).

Every translation unit in csrc/ is compiled by nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and linked into one
shared library with the C ABI of include/a2ds.h.  Rebuilds only what is
stale.  Usage:  python a2d-shells_gb300/build.py [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "liba2ds_gpu.so")
INCLUDE = os.path.join(REPO, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra_ptxas: bool):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]
    if extra_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "a2ds.h"))
    return hs


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    newest_header = max(os.path.getmtime(h) for h in headers())
    jobs = []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        stale = force or not os.path.exists(o) or \
            os.path.getmtime(o) < max(os.path.getmtime(s), newest_header)
        jobs.append((s, o, stale))
    todo = [(s, o) for s, o, st in jobs if st]

    def compile_one(so):
        s, o = so
        cmd = [nvcc(), "-c", s, "-o", o + ".tmp"] + _flags(verbose)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(s)}:\n{r.stderr}")
        os.replace(o + ".tmp", o)
        return r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
            for out in ex.map(compile_one, todo):
                if verbose and out:
                    sys.stderr.write(out)
    objs = [o for _, o, _ in jobs]
    if todo or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), "-shared", "-o", tmp] + ARCH + objs + ["-lcudart_static", "-lpthread",
                                                             "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
