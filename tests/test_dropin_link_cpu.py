"""segTACO's unmodified driver (matrix_main.cpp with its headers) compiles and
links against libsegtaco.so in place of gpu_kernels.cu: every kernel name it
calls resolves to this library (it is not run: no GPU here)."""
import os
import subprocess

import pytest

from oracle.build import REFERENCE_TREE as REF_TREE  # the recipe resolves the tree
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "segtaco_gb300")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_TREE, "matrix_main.cpp")),
                    reason="segTACO source tree not present")
def test_segtaco_driver_links_against_libsegtaco(tmp_path, native_lib):
    obj, exe = str(tmp_path / "matrix_main.o"), str(tmp_path / "matrix-eval-gpu")
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(
        subprocess.run(["bash", "-c", "command -v nvcc || echo /usr/local/cuda/bin/nvcc"],
                       capture_output=True, text=True).stdout.strip())), "include")
    subprocess.run(["g++", "-std=c++14", "-O1", "-fopenmp", "-I", REF_TREE,
                    "-I", os.path.join(REF_TREE, "eigen-3.4.0"), "-I", cuda_inc,
                    "-c", os.path.join(REF_TREE, "matrix_main.cpp"), "-o", obj], check=True)
    undefined = subprocess.run(["nm", "-uC", obj], capture_output=True, text=True).stdout
    called = sorted({l.strip()[2:].split("(")[0] for l in undefined.splitlines()
                     if "taco_tensor_t" in l or "get_gpu_timer_result" in l})
    assert len(called) >= 40  # the sweep's spmm_* names and the timer
    r = subprocess.run(["g++", "-fopenmp", obj, "-o", exe, "-L", LIBDIR, "-lsegtaco",
                        "-Wl,-rpath," + LIBDIR, "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    dyn = subprocess.run(["nm", "-DC", os.path.join(LIBDIR, "libsegtaco.so")],
                         capture_output=True, text=True).stdout
    exported = {l.split(" T ", 1)[1].split("(")[0] for l in dyn.splitlines() if " T " in l}
    assert set(called) <= exported
