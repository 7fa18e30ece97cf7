"""Parity at the benchmark configurations' full sizes (seeded synthetic
stand-ins for segTACO's SuiteSparse sweep), against the FP64 oracle:

* uniform 16,384 x 16,384, 16 nonzeros per row, N = 32: every schedule, every
  element of C;
* banded-plus-random 262,144 x 262,144 (|i - j| <= 32 plus 8 random columns
  per row, 19,135,456 nonzeros), D = N = 64: SDDMM with fp32 and bf16 dense
  operands (every output), and the bf16-B SpMM (every element of C);
* SpMSpV on the 1M x 1M power-law matrix stored by columns, x 10 % nonzero;
* C and SDDMM's X past 2^31 elements (20M x 128).

The 1M x 1M power-law SpMM and SpMV at full size are in test_gpu_spmm.py and
test_gpu_side_ops.py; the 256-matrix pool in test_gpu_batch.py."""
import numpy as np
import pytest
import torch

from gpu_util import TOL, assert_spmm_close, dev, spmm_ref, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def banded():
    A = synth.banded_plus_random(seed=0)
    assert A.nnz == 19_135_456
    return A


def test_uniform16_all_schedules(cuda):
    A = synth.uniform_rows(seed=0)
    assert (A.M, A.K, A.nnz) == (16384, 16384, 262_144)
    B = synth.dense(A.K, 32, seed=1)
    ref = spmm_ref(A, B)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    for sched in ("rb_sr", "rb_pr", "eb_sr", "eb_pr"):
        C = torch.full((A.M, 32), float("nan"), device="cuda")
        ops.spmm(Ad, Bd, C_out=C, config=N.Config.make(schedule=sched))
        torch.cuda.synchronize()
        assert_spmm_close(C.cpu().numpy(), A, B, ref=ref)


@pytest.mark.parametrize("bf16", [False, True])
def test_banded_sddmm_full(cuda, banded, bf16):
    A = banded
    X = synth.dense(A.M, 64, seed=4)
    Y = synth.dense(A.K, 64, seed=5)
    if bf16:
        X, Y = synth.to_bf16_bits(X), synth.to_bf16_bits(Y)
        Xd, Yd = to_torch_bf16(X), to_torch_bf16(Y)
    else:
        Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    out = torch.full((A.nnz,), float("nan"), device="cuda")
    ops.sddmm(dev(A), Xd, Yd, out)
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y, bf16=bf16)
    assert O.max_bound_err(out.cpu().numpy(), ref, bound) <= TOL


def test_power_law_spmspv_full(cuda):
    """SpMSpV on the 1M x 1M power-law matrix stored by columns, x with 10 %
    of K nonzero (distinct random indices), every element of y."""
    A = synth.power_law(seed=0)
    At = A.transpose()
    rng = np.random.default_rng(0)
    nx = A.K // 10
    idx = np.sort(rng.permutation(A.K)[:nx]).astype(np.int32)
    xv = rng.uniform(-1, 1, nx).astype(np.float32)
    y = ops.spmspv(dev(At), torch.from_numpy(idx).cuda(), torch.from_numpy(xv).cuda(), A.M)
    ref, bound = O.spmspv_f64(At.row_ptr, At.col, At.val, A.M, idx, xv)
    assert O.max_bound_err(y.cpu().numpy(), ref, bound) <= TOL


def test_banded_bf16_spmm_full(cuda, banded):
    A = banded
    bits = synth.to_bf16_bits(synth.dense(A.K, 64, seed=6))
    C = torch.full((A.M, 64), float("nan"), device="cuda")
    ops.spmm(dev(A), to_torch_bf16(bits), C_out=C)
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, bits, bf16=True)


def test_beyond_2g_elements(cuda):
    """C (and SDDMM's X) with more than 2^31 elements: A 20,000,000 x 4,096
    with one nonzero per row, N = D = 128, so offsets past 2^31 are reached
    by the rows at the end.  One product per element makes every schedule's
    result bit-exact (fp32 val * b); sampled rows include the last ones."""
    M, K, NC = 20_000_000, 4096, 128
    assert M * NC > 2**31
    rng = np.random.default_rng(0)
    col = rng.integers(0, K, M).astype(np.int32)
    val = rng.uniform(-1, 1, M).astype(np.float32)
    A = synth.CSR(np.arange(M + 1, dtype=np.int32), col, val, M, K)
    B = synth.dense(K, NC, seed=1)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    rows = np.unique(np.concatenate([np.arange(4), np.arange(M - 4, M),
                                     rng.integers(2**31 // NC, M, 200), rng.integers(0, M, 100)]))
    rows_d = torch.from_numpy(rows).cuda()
    want = val[rows, None] * B[col[rows]]  # fp32 products, one rounding each
    C = torch.empty((M, NC), device="cuda")
    for sched in ("rb_sr", "rb_pr", "eb_sr", "eb_pr"):
        C.fill_(float("nan"))
        ops.spmm(Ad, Bd, C_out=C, config=N.Config.make(schedule=sched))
        torch.cuda.synchronize()
        assert np.array_equal(C[rows_d].cpu().numpy(), want), sched
    del C
    g = torch.Generator(device="cuda").manual_seed(3)
    X = torch.rand((M, NC), device="cuda", generator=g) * 2 - 1
    Y = torch.from_numpy(synth.dense(K, NC, seed=4)).cuda()
    out = ops.sddmm(Ad, X, Y)
    torch.cuda.synchronize()
    Xr = X[rows_d].double().cpu().numpy()
    Yr = Y.double().cpu().numpy()[col[rows]]
    ref = val[rows].astype(np.float64) * (Xr * Yr).sum(axis=1)
    bound = np.abs(val[rows].astype(np.float64)) * np.abs(Xr * Yr).sum(axis=1)
    assert O.max_bound_err(out[rows_d].cpu().numpy(), ref, bound) <= TOL
