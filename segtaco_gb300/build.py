"""Build recipe of libsegtaco.so (nvcc, sm_103a only, in-tree).

Every ``csrc/*.cu`` translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``segtaco_gb300/libsegtaco.so`` (with cuSPARSE for the vendor comparator
names).  Objects go to ``segtaco_gb300/_build/``.  The build is incremental:
an object is rebuilt when its source or any header under csrc/ or include/
is newer.
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
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsegtaco.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src, obj, extra):
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return r.stderr


def _compile_host(src, obj, extra):
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-I", CSRC,
           "-I", os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include"),
           "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return r.stderr


def build(force: bool = False, verbose: bool = False, jobs: int | None = None,
          extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    todo, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.splitext(os.path.basename(s))[0] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_mtime):
            todo.append((s, o))
    if todo:
        jobs = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(jobs) as ex:
            futs = {ex.submit(_compile_host if s.endswith(".cpp") else _compile, s, o,
                              list(extra)): s for s, o in todo}
            for f in cf.as_completed(futs):
                msg = f.result()
                if verbose and msg:
                    print(msg, file=sys.stderr)
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcusparse"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force="--force" in sys.argv, verbose=v,
                extra=["-Xptxas", "-v"] if v else []))
