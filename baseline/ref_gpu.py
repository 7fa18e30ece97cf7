"""Build recipe for timing segTACO's own generic SpMM kernels on the GPU
(reference-arm infrastructure: nothing in the product path uses it, and it
uses nothing of the oracle).

* ``stage()`` (where the segTACO source tree is present) copies the headers
  the four generic kernels need -- ``gpu_library.h``, ``taco_tensor_t.h`` and
  ``matrix_kernels/spmm_{rb,eb}_{sr,pr}.h``, unchanged -- into the git-ignored
  ``baseline/_ref/segtaco/``.  That folder travels with the working tree to a
  GPU host that has no reference tree; the reference sources are never
  committed.  No source fix is needed: of segTACO's two cuBLAS headers only
  ``gpu_library.h:12`` (cublas.h) is included here, so CUDA 13's guard against
  including both cublas.h and cublas_v2.h does not trip.
* ``start_build()`` / ``finish_build()`` compile ``baseline/ref_gpu_timing.cu`` (a harness that calls
  segTACO's host wrappers the way its driver does) against the staged headers
  for sm_103a into ``baseline/_ref/ref_gpu_timing``.
* ``run(...)`` feeds it one CSR product and returns segTACO's
  ``get_gpu_timer_result()`` times per kernel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGED = os.path.join(OUT, "segtaco")
BIN = os.path.join(OUT, "ref_gpu_timing")
SRC = os.path.join(HERE, "ref_gpu_timing.cu")
# Where the segTACO source tree lies (present only where it was checked out).
REFERENCE_TREE = os.environ.get("SEGTACO_REFERENCE_TREE", "/root/reference")


def reference_tree_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_TREE, "gpu_library.h"))
HEADERS = ["gpu_library.h", "taco_tensor_t.h"] + [
    os.path.join("matrix_kernels", "spmm_%s.h" % s) for s in ("rb_sr", "rb_pr", "eb_sr", "eb_pr")]
# segTACO's generic kernels (the ones that take any N <= 256), by host wrapper.
KERNELS = ("spmm_rb_sr", "spmm_rb_pr", "spmm_eb_sr", "spmm_eb_pr")


def staged() -> bool:
    return all(os.path.isfile(os.path.join(STAGED, h)) for h in HEADERS)


def stage() -> bool:
    if not reference_tree_present():
        return staged()
    for h in HEADERS:
        src = os.path.join(REFERENCE_TREE, h)
        dst = os.path.join(STAGED, h)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
            shutil.copyfile(src, dst)
    return True


def build_cmd():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
            "-I", STAGED, SRC, "-o", BIN + ".tmp", "-lcusparse", "-lcublas"]


def start_build():
    """Starts the harness compile in the background (about 20 s, one
    translation unit); returns the process or None when nothing is to be
    built.  finish_build() waits for it."""
    if not stage():
        return None
    if os.path.exists(BIN) and os.path.getmtime(BIN) >= max(
            os.path.getmtime(SRC), *(os.path.getmtime(os.path.join(STAGED, h)) for h in HEADERS)):
        return None
    return subprocess.Popen(build_cmd(), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                            text=True)


def finish_build(proc) -> str | None:
    if proc is None:
        return BIN if os.path.exists(BIN) else None
    out, _ = proc.communicate()
    if proc.returncode != 0:
        raise RuntimeError("reference GPU harness build failed:\n" + out[-4000:])
    os.replace(BIN + ".tmp", BIN)
    return BIN


def available() -> bool:
    return os.path.isfile(BIN) and os.access(BIN, os.X_OK)


def run(A, B, kernels=KERNELS, warmup=2, reps=10, timeout=600):
    """segTACO's get_gpu_timer_result() for each kernel on C = A B (host
    operands; every call copies in, times {zero C, kernel}, copies out).
    Returns {name: {"ms": [...], "checksum": sum of C}}."""
    M, K = int(A.M), int(A.K)
    N = int(B.shape[1])
    tmp = tempfile.mkdtemp(prefix="segtaco_refgpu_")
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.txt")
    try:
        with open(fin, "wb") as f:
            f.write(np.array([M, K, N, A.nnz], np.int64).tobytes())
            for a, t in ((A.row_ptr, np.int32), (A.col, np.int32), (A.val, np.float32),
                         (B, np.float32)):
                f.write(np.ascontiguousarray(a, t).tobytes())
        subprocess.run([BIN, fin, fout, str(warmup), str(reps), *kernels], check=True,
                       timeout=timeout, capture_output=True)
        out = {}
        for line in open(fout):
            p = line.split()
            out[p[0]] = {"ms": [float(x) for x in p[1:-1]], "checksum": float(p[-1])}
        return out
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
