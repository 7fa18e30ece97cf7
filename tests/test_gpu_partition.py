"""Partition and index arrays: bit-exact against segTACO's own
taco_binarySearchBefore (golden) and the oracle's restatements."""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden
from gpu_util import dev, small_cases
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("name", golden_cases("spmm_"))
def test_block_starts_taco_match_reference(cuda, name):
    d = load_golden("spmm_", name)
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    Ad = dev(A)
    for P in (1, 7, 32, 256, 3584):
        assert np.array_equal(host(ops.block_starts_taco(Ad, P)), d["starts_P%d" % P])


CASES = dict(small_cases())


@pytest.mark.parametrize("name", list(CASES))
def test_partitions_match_oracle(cuda, name):
    A = CASES[name]
    Ad = dev(A)
    for P in (1, 5, 32, 256, 2048):
        assert np.array_equal(host(ops.block_starts_taco(Ad, P)), O.block_starts_taco(A.row_ptr, A.M, P))
        assert np.array_equal(host(ops.block_starts_canonical(Ad, P)),
                              O.block_starts_canonical(A.row_ptr, A.M, P))
    for D in (1, 2, 33, 256, 2048):
        xs, ys = ops.merge_path(Ad, D)
        ox, oy = O.merge_path(A.row_ptr, A.M, D)
        assert np.array_equal(host(xs), ox) and np.array_equal(host(ys), oy)
    assert np.array_equal(host(ops.row_ids(Ad)), O.row_ids(A.row_ptr, A.M))


def test_full_size_partitions(cuda):
    A = synth.power_law(seed=0)
    Ad = dev(A, with_values=False)
    for D in (256, 2048):
        xs, ys = ops.merge_path(Ad, D)
        ox, oy = O.merge_path(A.row_ptr, A.M, D)
        assert np.array_equal(host(xs), ox) and np.array_equal(host(ys), oy)
    assert np.array_equal(host(ops.block_starts_taco(Ad, 256)), O.block_starts_taco(A.row_ptr, A.M, 256))
    assert np.array_equal(host(ops.row_ids(Ad)), O.row_ids(A.row_ptr, A.M))


def test_validate_rejects_malformed_csr(cuda):
    A = CASES["powerlaw"]
    ops.csr_validate(dev(A))
    bad_col = synth.CSR(A.row_ptr, A.col.copy(), A.val, A.M, A.K)
    bad_col.col[17] = A.K + 3
    with pytest.raises(N.SegtacoError) as e:
        ops.csr_validate(dev(bad_col))
    assert e.value.code == N.EINVAL and "col out of" in str(e.value) and "17" in str(e.value)
    bad_rp = synth.CSR(A.row_ptr.copy(), A.col, A.val, A.M, A.K)
    bad_rp.row_ptr[10], bad_rp.row_ptr[11] = bad_rp.row_ptr[11] + 1, bad_rp.row_ptr[10]
    with pytest.raises(N.SegtacoError) as e:
        ops.csr_validate(dev(bad_rp))
    assert "decreases" in str(e.value)
