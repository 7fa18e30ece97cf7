"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles ``segtaco_oracle.c`` (exact restatement, built with
  ``-ffp-contract=off``, portable flags) and ``segtaco_cpu_baseline.c`` (the
  timed CPU baseline, ``timed_flags()``: -O3, OpenMP, Grace-tuned on Grace)
  into ``oracle/_build/liboracle.so`` with gcc.  The same recipe works on
  x86-64 and aarch64 hosts.
* ``build_ref()`` compiles segTACO's own CPU code from the reference source tree
  (when that tree is present) into ``oracle/_ref/``: ``ref_golden`` (Eigen
  product, spmm_cpu_naive, the SDDMM and SpMSpV CPU references, the .mtx reader)
  and ``ref_search`` (taco_binarySearchBefore/After from gpu_library.h, host
  side).  These generate the golden fixtures under ``tests/golden/``; nothing at
  run time depends on them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
REFERENCE_TREE = os.environ.get("SEGTACO_REFERENCE_TREE", "/root/reference")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def timed_flags() -> list:
    """Flags of the timed CPU baseline: -O3 with OpenMP, tuned for the host's
    cores where they are Grace's (Neoverse V2: -mcpu=neoverse-v2 names that
    core explicitly); elsewhere portable.  The exact restatement keeps
    portable flags and -ffp-contract=off (its results are compared bit for
    bit; the timed product's are not)."""
    import platform
    flags = ["-O3", "-fopenmp"]
    if platform.machine() in ("aarch64", "arm64"):
        try:
            part = [l for l in open("/proc/cpuinfo") if l.lower().startswith("cpu part")]
        except OSError:
            part = []
        if part and part[0].split(":")[1].strip().lower() == "0xd4f":  # Neoverse V2
            flags.append("-mcpu=neoverse-v2")
    return flags


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    exact = os.path.join(HERE, "segtaco_oracle.c")
    timed = os.path.join(HERE, "segtaco_cpu_baseline.c")
    if not force and not _stale(LIB, [exact, timed, __file__]):
        return LIB
    o1 = os.path.join(BUILD, "segtaco_oracle.o")
    o2 = os.path.join(BUILD, "segtaco_cpu_baseline.o")
    _run(["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=gnu11", "-c", exact, "-o", o1])
    _run(["gcc", *timed_flags(), "-fPIC", "-std=gnu11", "-c", timed, "-o", o2])
    tmp = LIB + ".tmp"
    _run(["gcc", "-shared", "-fopenmp", o1, o2, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def reference_tree_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_TREE, "gpu_library.h"))


# The one source fix the SpMSpV experiment header needs to compile against the
# current taco_tensor_t (int32_t*** indices, float* vals): its driver builds the
# sparse x with uint8_t pointers (matrix_experiments/spmspv_csr_gpu.h:54-58).
# Only those allocations are retyped; spmspv_csr_cpu_taco_ref (:9-32), the CPU
# reference the fixtures come from, is compiled as written.
SPMSPV_HEADER = os.path.join("matrix_experiments", "spmspv_csr_gpu.h")
SPMSPV_CAST_FIX = (
    ("x_taco.indices = new uint8_t**[1*4];", "x_taco.indices = new int32_t**[1*4];"),
    ("x_taco.indices[0] = new uint8_t*[2*4];", "x_taco.indices[0] = new int32_t*[2*4];"),
    ("x_taco.indices[0][0] = (uint8_t*)malloc", "x_taco.indices[0][0] = (int32_t*)malloc"),
    ("x_taco.indices[0][1] = (uint8_t*)malloc", "x_taco.indices[0][1] = (int32_t*)malloc"),
    ("x_taco.vals = (uint8_t*)malloc", "x_taco.vals = (float*)malloc"),
)
PATCHED = os.path.join(REF_OUT, "patched")


def _patched_spmspv_header() -> str:
    """Scratch copy of the SpMSpV experiment header with SPMSPV_CAST_FIX applied
    (written under the git-ignored oracle/_ref/patched, which precedes the
    reference tree on the include path)."""
    src = os.path.join(REFERENCE_TREE, SPMSPV_HEADER)
    dst = os.path.join(PATCHED, SPMSPV_HEADER)
    text = open(src).read()
    for old, new in SPMSPV_CAST_FIX:
        if text.count(old) != 1:
            raise RuntimeError("SpMSpV cast fix does not apply: %r" % old)
        text = text.replace(old, new)
    os.makedirs(os.path.dirname(dst), exist_ok=True)
    if not os.path.exists(dst) or open(dst).read() != text:
        with open(dst, "w") as f:
            f.write(text)
    return dst


def build_ref(force: bool = False) -> dict:
    """Compile the reference's own CPU code into oracle/_ref (x86 container only)."""
    if not reference_tree_present():
        return {}
    os.makedirs(REF_OUT, exist_ok=True)
    out = {}
    golden_src = os.path.join(HERE, "ref", "ref_golden.cpp")
    golden_bin = os.path.join(REF_OUT, "ref_golden")
    patched = _patched_spmspv_header()
    if force or _stale(golden_bin, [golden_src, __file__, patched]):
        # The experiment drivers reference the GPU entry points, which are never
        # called here, hence the unresolved-symbol link option.  -ffp-contract=off keeps Eigen's
        # multiply and add separate, as on a host without FMA.
        _run(["g++", "-O2", "-std=c++14", "-fopenmp", "-w",
              "-ffp-contract=off", "-DNDEBUG", "-I", PATCHED,
              "-I", REFERENCE_TREE, "-I", os.path.join(REFERENCE_TREE, "eigen-3.4.0"),
              "-I", "/usr/local/cuda/include",
              golden_src, "-o", golden_bin,
              "-Wl,--unresolved-symbols=ignore-all"])
    out["ref_golden"] = golden_bin
    # Eigen's product timed with the timed port's flags (-O3, OpenMP, portable)
    time_src = os.path.join(HERE, "ref", "ref_eigen_time.cpp")
    time_bin = os.path.join(REF_OUT, "ref_eigen_time")
    if force or _stale(time_bin, [time_src, __file__]):
        _run(["g++", "-O3", "-std=c++14", "-fopenmp", "-w", "-DNDEBUG",
              "-I", REFERENCE_TREE, "-I", os.path.join(REFERENCE_TREE, "eigen-3.4.0"),
              "-I", "/usr/local/cuda/include", time_src, "-o", time_bin])
    out["ref_eigen_time"] = time_bin
    search_src = os.path.join(HERE, "ref", "ref_search.cu")
    search_bin = os.path.join(REF_OUT, "ref_search")
    if force or _stale(search_bin, [search_src, __file__]):
        _run(["nvcc", "-O2", "-std=c++17", "-w", "-I", REFERENCE_TREE, search_src,
              "-o", search_bin])
    out["ref_search"] = search_bin
    return out


def main(argv):
    force = "--force" in argv
    print(build_oracle(force))
    print(build_ref(force))


if __name__ == "__main__":
    main(sys.argv[1:])
