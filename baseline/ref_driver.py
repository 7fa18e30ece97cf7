"""Build recipe for running segTACO's own, unmodified sweep driver
(``matrix_main.cpp`` -> ``spmm_csr_gpu``) on this library: its kernel names
resolve to ``libsegtaco.so`` instead of segTACO's ``gpu_kernels.cu``.

Test infrastructure: nothing in the product path uses it, and it uses nothing
of the oracle.

* ``stage()`` (where the segTACO source tree is present) copies the driver's
  source and headers, Eigen 3.4's headers (the driver builds its CSR with
  them) and the bundled ``matrix_subset/192bit/192bit.mtx`` fixture, unchanged,
  into the git-ignored ``baseline/_ref/driver/``, which travels with the
  working tree to a GPU host that has no reference tree.  The reference sources
  are never committed.
* ``build()`` compiles the driver there with g++ and links it against
  ``segtaco_gb300/libsegtaco.so`` (``--no-undefined``: every name the sweep
  calls must come from this library).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref", "driver")
EXE = os.path.join(OUT, "matrix-eval-gpu")
LIBDIR = os.path.join(ROOT, "segtaco_gb300")
# Where the segTACO source tree lies (present only where it was checked out).
REFERENCE_TREE = os.environ.get("SEGTACO_REFERENCE_TREE", "/root/reference")
FILES = ["matrix_main.cpp", "ds.h", "timers.h", "mmio.h", "taco_tensor_t.h", "gpu_kernels.cuh",
         os.path.join("matrix_experiments", "spmm_csr_gpu.h"),
         os.path.join("matrix_subset", "192bit", "192bit.mtx")]
EIGEN = os.path.join("eigen-3.4.0", "Eigen")


def staged() -> bool:
    return all(os.path.isfile(os.path.join(OUT, f)) for f in FILES) and \
        os.path.isdir(os.path.join(OUT, EIGEN))


def stage() -> bool:
    """Copy the driver's files out of the reference tree (a no-op without it)."""
    if not os.path.isfile(os.path.join(REFERENCE_TREE, "matrix_main.cpp")):
        return staged()
    for f in FILES:
        src, dst = os.path.join(REFERENCE_TREE, f), os.path.join(OUT, f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
            shutil.copyfile(src, dst)
    if not os.path.isdir(os.path.join(OUT, EIGEN)):
        shutil.copytree(os.path.join(REFERENCE_TREE, EIGEN), os.path.join(OUT, EIGEN))
    return True


def fixture_dir() -> str:
    return os.path.join(OUT, "matrix_subset", "192bit")


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def build() -> str:
    """Compile the staged driver against libsegtaco.so; returns the executable."""
    if not staged():
        raise RuntimeError("segTACO's driver is not staged (baseline/_ref/driver)")
    obj = os.path.join(OUT, "matrix_main.o")
    subprocess.run(["g++", "-std=c++14", "-O1", "-fopenmp", "-I", OUT,
                    "-I", os.path.join(OUT, "eigen-3.4.0"), "-I", _cuda_include(),
                    "-c", os.path.join(OUT, "matrix_main.cpp"), "-o", obj], check=True)
    subprocess.run(["g++", "-fopenmp", obj, "-o", EXE, "-L", LIBDIR, "-lsegtaco",
                    "-Wl,-rpath," + LIBDIR, "-Wl,--no-undefined"], check=True)
    return EXE
