"""Every segTACO-named entry point, called with host taco_tensor_t operands
through segtaco_taco_call (the drop-in path), against segTACO's own Eigen
output for the same inputs."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_util import TOL
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import synth, taco

pytestmark = pytest.mark.gpu
SPMM_NAMES = [n for n in N.taco_names() if n.startswith("spmm_")]


@pytest.mark.parametrize("name", SPMM_NAMES)
@pytest.mark.parametrize("case", ["powerlaw_n33", "refvals_ones_n4"])
def test_spmm_name(cuda, name, case):
    d = load_golden("spmm_", case)
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    C, ms = taco.spmm(name, A, d["B"])
    assert ms > 0.0
    ref = O.spmm_f64(A.row_ptr, A.col, A.val, d["B"])
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, d["B"])
    assert O.max_bound_err(C, ref, S) <= TOL
    assert O.max_bound_err(C, d["C_eigen"].astype(np.float64), S) <= 2 * TOL


def test_spmv_name(cuda):
    d = load_golden("spmm_", "powerlaw_n33")
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    y = np.zeros((A.M, 1), np.float32)
    tA, h1 = taco.csr(A.row_ptr, A.col, A.val, A.M, A.K)
    tx, h2 = taco.dense(d["x"].reshape(-1, 1).copy())
    ty, h3 = taco.dense(y)
    taco.call("spmv_csr_gpu_taco", ty, tA, tx)
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, d["x"].reshape(-1, 1)).reshape(-1)
    assert O.max_bound_err(y.reshape(-1), d["y_eigen"].astype(np.float64), S) <= 2 * TOL


@pytest.mark.parametrize("name", ["sddmm_csr_gpu_taco", "sddmm_csr_gpu_warp"])
def test_sddmm_names(cuda, name):
    d = load_golden("sddmm_", "powerlaw_d64")
    M, K = int(d["M"]), int(d["K"])
    out = np.zeros(d["col"].shape[0], np.float32)
    tOut, h0 = taco.csr(d["row_ptr"], d["col"], out, M, K)
    tOut.vals = out.ctypes.data_as(type(tOut.vals))
    tB, h1 = taco.csr(d["row_ptr"], d["col"], d["val"], M, K)
    tC, h2 = taco.dense(d["X"])
    tD, h3 = taco.dense(d["Y"])
    taco.call(name, tOut, tB, tC, tD)
    _, bound = O.sddmm_f64(d["row_ptr"], d["col"], d["val"], d["X"], d["Y"])
    assert O.max_bound_err(out, d["out"], bound) <= TOL


@pytest.mark.parametrize("case", ["rand_nx10", "long_col", "empty_cols"])
def test_spmspv_name_golden(cuda, case):
    """spmspv_csr_gpu_taco against segTACO's spmspv_csr_cpu_taco_ref output."""
    d = load_golden("spmspv_", case)
    M, K = int(d["M"]), int(d["K"])
    y = np.full((M, 1), np.nan, np.float32)
    tA, h1 = taco.csr(d["col_ptr"], d["row_idx"], d["val"], K, M)
    tx, h2 = taco.sparse_vector(d["x_idx"], d["x_val"], K)
    ty, h3 = taco.dense(y)
    taco.call("spmspv_csr_gpu_taco", ty, tA, tx)
    _, bound = O.spmspv_f64(d["col_ptr"], d["row_idx"], d["val"], M, d["x_idx"], d["x_val"])
    assert O.max_bound_err(y.reshape(-1), d["y"], bound) <= TOL


def test_spmspv_name(cuda):
    A = synth.random_csr(400, 300, 0.03, seed=21, p_empty=0.1)
    At = A.transpose()
    rng = np.random.default_rng(2)
    idx = rng.permutation(A.K)[:30].astype(np.int32)
    xv = rng.uniform(-1, 1, 30).astype(np.float32)
    y = np.zeros((A.M, 1), np.float32)
    tA, h1 = taco.csr(At.row_ptr, At.col, At.val, At.M, At.K)
    tx, h2 = taco.sparse_vector(idx, xv, A.K)
    ty, h3 = taco.dense(y)
    taco.call("spmspv_csr_gpu_taco", ty, tA, tx)
    ref, bound = O.spmspv_f64(At.row_ptr, At.col, At.val, A.M, idx, xv)
    assert O.max_bound_err(y.reshape(-1), ref, bound) <= TOL


def test_shape_mismatch_is_an_error_not_a_fault(cuda):
    A = synth.random_csr(50, 40, 0.1, seed=3)
    B = synth.dense(41, 4, seed=1)  # wrong K is not detectable; wrong N is:
    Cm = np.zeros((50, 5), np.float32)
    tA, h1 = taco.csr(A.row_ptr, A.col, A.val, A.M, A.K)
    tB, h2 = taco.dense(B)
    tC, h3 = taco.dense(Cm)
    with pytest.raises(N.SegtacoError):
        taco.call("spmm_eb_sr", tC, tA, tB)


@pytest.mark.parametrize("n", [128, 96, 40])
@pytest.mark.parametrize("name", ["spmm_eb_pr", "spmm_rb_sr"])
def test_spmm_name_pipelined_tiles(cuda, name, n):
    """A product large enough that the drop-in cuts it into several column
    slabs and row blocks (copies overlapping the tiles' kernels)."""
    A = synth.power_law(400_000, 400_000, 1.8, 20_000, 0.02, seed=31)
    B = synth.dense(A.K, n, seed=32)
    C, ms = taco.spmm(name, A, B)
    assert ms > 0.0
    ref = O.spmm_f64(A.row_ptr, A.col, A.val, B)
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, B)
    assert O.max_bound_err(C, ref, S) <= TOL
