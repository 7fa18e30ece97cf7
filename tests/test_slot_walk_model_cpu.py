"""The slot walk's control flow (tests/slot_walk_model.py) on irregular
matrices and chunk sizes: every row written, interior rows stored once, reads
in bounds, the product exact against a dense reference."""
import numpy as np
import pytest

from slot_walk_model import slot_walk
from segtaco_gb300 import synth


def _cases():
    return {
        "powerlaw": synth.power_law(400, 300, 1.8, 200, 0.05, seed=1),
        "empty_run": synth.random_csr(300, 50, 0.0, seed=2, long_rows={0: 7, 150: 90, 299: 3}),
        "half_empty": synth.random_csr(200, 80, 0.05, seed=3, p_empty=0.5),
        "one_long_row": synth.random_csr(3, 500, 0.0, seed=4, long_rows={1: 400}),
        "single": synth.random_csr(1, 1, 1.0, seed=5),
        "all_empty": synth.CSR(np.zeros(9, np.int32), np.zeros(0, np.int32),
                               np.zeros(0, np.float32), 8, 4),
    }


@pytest.mark.parametrize("D", [1, 2, 3, 7, 16, 64, 100000])
@pytest.mark.parametrize("name", list(_cases()))
def test_slot_walk_model(name, D):
    A = _cases()[name]
    B = np.random.default_rng(7).uniform(-1, 1, (A.K, 3))
    C, log, reads = slot_walk(A.row_ptr, A.col, A.val.astype(np.float64), B, D)
    dense = np.zeros((A.M, A.K))
    dense[np.repeat(np.arange(A.M), A.row_lengths()), A.col] = A.val
    assert not np.isnan(C).any()  # every row written
    assert np.allclose(C, dense @ B, rtol=0, atol=1e-12)
    stores = [r for k, r in log if k == "store"]
    assert len(stores) == len(set(stores))
    assert all(0 <= i < len(A.col) for k, i in reads if k == "col")


def test_slot_walk_single_chunk_is_sequential():
    """With one chunk every row is one chain in storage order (eb_sr)."""
    A = synth.power_law(100, 90, 1.8, 60, 0.05, seed=8)
    B = np.random.default_rng(9).uniform(-1, 1, (A.K, 2))
    C, log, _ = slot_walk(A.row_ptr, A.col, A.val.astype(np.float64), B, 10**9)
    assert all(k == "store" for k, _ in log)
