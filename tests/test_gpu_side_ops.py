"""SpMV, SDDMM and SpMSpV parity against the oracle and segTACO's own CPU
outputs (golden), through the C ABI."""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden
from gpu_util import TOL, dev, small_cases, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu
CASES = small_cases()


def check_vec(got, ref, bound, tol=TOL):
    if ref.size:
        err = O.max_bound_err(got, ref, bound)
        assert err <= tol, err


@pytest.mark.parametrize("name", golden_cases("spmm_"))
def test_spmv_golden(cuda, name):
    d = load_golden("spmm_", name)
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    y = ops.spmv(dev(A), torch.from_numpy(d["x"]).cuda()).cpu().numpy()
    ref = O.spmv_f64(A.row_ptr, A.col, A.val, d["x"])
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, d["x"].reshape(-1, 1)).reshape(-1)
    check_vec(y, ref, S)
    check_vec(y, d["y_eigen"].astype(np.float64), S, 2 * TOL)


@pytest.mark.parametrize("name", list(CASES))
def test_spmv_small(cuda, name):
    A = CASES[name]
    x = synth.dense(A.K, 1, seed=3).reshape(-1)
    y = ops.spmv(dev(A), torch.from_numpy(x).cuda()).cpu().numpy()
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, x.reshape(-1, 1)).reshape(-1)
    check_vec(y, O.spmv_f64(A.row_ptr, A.col, A.val, x), S)


@pytest.mark.parametrize("name", ["powerlaw", "half_empty", "one_long_row", "empty_run"])
def test_spmv_writes_every_row(cuda, name):
    """y starts as NaN: every row must be written (rows split across chunks
    are zeroed by the partition, then accumulated); values default to 1."""
    A = CASES[name]
    x = synth.dense(A.K, 1, seed=4).reshape(-1)
    for with_values in (True, False):
        Ad = dev(A, with_values=with_values)
        y = torch.full((A.M,), float("nan"), device="cuda")
        ops.spmv(Ad, torch.from_numpy(x).cuda(), y)
        val = A.val if with_values else np.ones_like(A.val)
        S = O.spmm_absbound(A.row_ptr, A.col, val, x.reshape(-1, 1)).reshape(-1)
        check_vec(y.cpu().numpy(), O.spmv_f64(A.row_ptr, A.col, val, x), S)
    Z = synth.random_csr(1100, 10, 0.0, seed=6)  # no nonzeros: y = 0
    y = torch.full((Z.M,), float("nan"), device="cuda")
    ops.spmv(dev(Z), torch.zeros(Z.K, device="cuda"), y)
    assert torch.all(y == 0)


@pytest.mark.parametrize("zipf_s", [1.8, 1.922])
def test_spmv_full_power_law(cuda, zipf_s):
    A = synth.power_law(s=zipf_s, seed=0)
    x = synth.dense(A.K, 1, seed=2).reshape(-1)
    y = ops.spmv(dev(A), torch.from_numpy(x).cuda()).cpu().numpy()
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, x.reshape(-1, 1)).reshape(-1)
    check_vec(y, O.spmv_f64(A.row_ptr, A.col, A.val, x), S)


@pytest.mark.parametrize("name", golden_cases("sddmm_"))
def test_sddmm_golden(cuda, name):
    d = load_golden("sddmm_", name)
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    out = ops.sddmm(dev(A), torch.from_numpy(d["X"]).cuda(), torch.from_numpy(d["Y"]).cuda())
    _, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, d["X"], d["Y"])
    check_vec(out.cpu().numpy(), d["out"], bound)  # sddmm_csr_cpu_taco_ref, in double


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("D", [1, 5, 16, 64, 100])
def test_sddmm_small(cuda, name, D):
    A = CASES[name]
    X = synth.dense(A.M, D, seed=4)
    Y = synth.dense(A.K, D, seed=5)
    out = ops.sddmm(dev(A), torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda())
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y)
    check_vec(out.cpu().numpy(), ref, bound)


@pytest.mark.parametrize("bf16", [False, True])
@pytest.mark.parametrize("D", [4, 8, 16, 32, 128, 256, 512, 1024])
def test_sddmm_fixed_shapes(cuda, D, bf16):
    """Every shape of the fixed-shape kernel (D / vector width a power of two
    up to 128), on a matrix with long and empty rows."""
    A = CASES["powerlaw"]
    X = synth.dense(A.M, D, seed=8)
    Y = synth.dense(A.K, D, seed=9)
    if bf16:
        X, Y = synth.to_bf16_bits(X), synth.to_bf16_bits(Y)
        out = ops.sddmm(dev(A), to_torch_bf16(X), to_torch_bf16(Y))
    else:
        out = ops.sddmm(dev(A), torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda())
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y, bf16=bf16)
    check_vec(out.cpu().numpy(), ref, bound)


@pytest.mark.parametrize("bf16", [False, True])
@pytest.mark.parametrize("aligned", [True, False])
@pytest.mark.parametrize("D", [64, 128])
def test_sddmm_alignment(cuda, bf16, aligned, D):
    """Rows 32-byte aligned take 32-byte lanes (8 fp32 / 16 bf16 values); a
    base only 16-byte aligned falls back to 16-byte lanes: same results."""
    A = CASES["powerlaw"]
    per16 = 8 if bf16 else 4  # elements in 16 bytes
    off = 0 if aligned else per16
    Xh = synth.dense(A.M, D + 2 * per16, seed=10)
    Yh = synth.dense(A.K, D + 2 * per16, seed=11)
    if bf16:
        Xh, Yh = synth.to_bf16_bits(Xh), synth.to_bf16_bits(Yh)
        Xb, Yb = to_torch_bf16(Xh), to_torch_bf16(Yh)
    else:
        Xb, Yb = torch.from_numpy(Xh).cuda(), torch.from_numpy(Yh).cuda()
    X, Y = Xb[:, off:off + D], Yb[:, off:off + D]  # ld = D + 32 bytes
    out = ops.sddmm(dev(A), X, Y)
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, Xh[:, off:off + D], Yh[:, off:off + D],
                             bf16=bf16)
    check_vec(out.cpu().numpy(), ref, bound)


@pytest.mark.parametrize("D", [8, 64])
def test_sddmm_bf16(cuda, D):
    A = CASES["banded"]
    X = synth.to_bf16_bits(synth.dense(A.M, D, seed=6))
    Y = synth.to_bf16_bits(synth.dense(A.K, D, seed=7))
    out = ops.sddmm(dev(A), to_torch_bf16(X), to_torch_bf16(Y))
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y, bf16=True)
    check_vec(out.cpu().numpy(), ref, bound)


@pytest.mark.parametrize("name", golden_cases("spmspv_"))
def test_spmspv_golden(cuda, name):
    """Against segTACO's own spmspv_csr_cpu_taco_ref output (tests/golden)."""
    d = load_golden("spmspv_", name)
    M = int(d["M"])
    At = synth.CSR(d["col_ptr"], d["row_idx"], d["val"], int(d["K"]), M)
    y = ops.spmspv(dev(At), torch.from_numpy(d["x_idx"]).cuda(),
                   torch.from_numpy(d["x_val"]).cuda(), M).cpu().numpy()
    _, bound = O.spmspv_f64(d["col_ptr"], d["row_idx"], d["val"], M, d["x_idx"], d["x_val"])
    check_vec(y, d["y"], bound)


@pytest.mark.parametrize("name", list(CASES))
def test_spmspv(cuda, name):
    A = CASES[name]
    At = A.transpose()
    rng = np.random.default_rng(1)
    nx = max(1, A.K // 10)
    idx = rng.permutation(A.K)[:nx].astype(np.int32)
    xv = rng.uniform(-1, 1, nx).astype(np.float32)
    y = ops.spmspv(dev(At), torch.from_numpy(idx).cuda(), torch.from_numpy(xv).cuda(), A.M)
    ref, bound = O.spmspv_f64(At.row_ptr, At.col, At.val, A.M, idx, xv)
    check_vec(y.cpu().numpy(), ref, bound)
