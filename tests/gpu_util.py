"""Helpers shared by the GPU parity tests: device upload and oracle checks."""
import numpy as np
import torch

from oracle import oracle as O
from segtaco_gb300 import ops, synth

# Tolerance of every FP32 result: |c - c64| <= TOL * sum_p |a_ip b_pk|, i.e. the
# bound-normalised error against the FP64 oracle (order-independent).
TOL = 1e-5


def dev(A, with_values=True):
    return ops.DeviceCSR.from_host(A, "cuda", with_values)


def spmm_ref(A, B, bf16=False):
    val = A.val
    ref = O.spmm_f64(A.row_ptr, A.col, val, B, bf16=bf16)
    S = O.spmm_absbound(A.row_ptr, A.col, val, B, bf16=bf16)
    return ref, S


def assert_spmm_close(C_got, A, B, bf16=False, tol=TOL, ref=None):
    if ref is None:
        ref = spmm_ref(A, B, bf16)
    r, S = ref
    if r.size == 0:
        return 0.0
    err = O.max_bound_err(np.ascontiguousarray(C_got), r, S)
    assert err <= tol, "bound-normalised error %g > %g" % (err, tol)
    return err


def small_cases():
    """Irregular small matrices covering the edge cases the schedules must meet."""
    cases = {
        "powerlaw": synth.power_law(4000, 3500, 1.8, 3000, 0.02, seed=11),
        "uniform16": synth.uniform_rows(2048, 2048, 16, seed=12),
        "banded": synth.banded_plus_random(3000, 8, 4, seed=13),
        "half_empty": synth.random_csr(1500, 900, 0.02, seed=14, p_empty=0.5),
        "one_long_row": synth.random_csr(3, 30000, 0.0, seed=15, long_rows={1: 20000}),
        "empty_run": synth.random_csr(3000, 500, 0.0, seed=16,
                                      long_rows={0: 40, 1500: 300, 2999: 5}),
        "single_nnz": synth.random_csr(1, 1, 1.0, seed=17),
    }
    A, _, _ = synth.pool_matrix(1)
    cases["pool1_banded"] = A
    return cases


def to_torch_bf16(bits):
    return torch.from_numpy(bits.view(np.int16)).cuda().view(torch.bfloat16)
