"""The row-driven merge-path rule of merge_path_kernel / batch_partition_kernel
(merge_path_store_row, segtaco_gb300/csrc/common.cuh) against the oracle's
binary-search partition, on the CPU: thread r writes the chunk edges c with
e_{r-1} <= c*D < e_r, e_r = row_ptr[r+1] + r + 1; thread M the rest."""
import numpy as np
import pytest

from oracle import oracle as O


def row_rule(rp, M, nnz, D, nchunks):
    total = M + nnz
    px = np.full(nchunks + 1, -1, np.int64)
    py = np.full(nchunks + 1, -1, np.int64)
    writes = np.zeros(nchunks + 1, np.int64)
    for r in range(M + 1):
        e_prev = 0 if r == 0 else int(rp[r]) + r
        c0 = (e_prev + D - 1) // D
        c1 = (int(rp[r + 1]) + r + 1 + D - 1) // D - 1 if r < M else nchunks
        for c in range(c0, min(c1, nchunks) + 1):
            d = min(c * D, total)
            px[c], py[c] = r, d - r
            writes[c] += 1
    return px, py, writes


@pytest.mark.parametrize("seed", range(12))
def test_row_rule_matches_oracle_partition(seed):
    rng = np.random.default_rng(seed)
    M = int(rng.integers(0, 600))
    lens = rng.integers(0, int(rng.choice([2, 10, 300])), M)
    if M and rng.random() < 0.4:
        lens[rng.random(M) < 0.5] = 0
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    nnz = int(rp[-1])
    for D in (1, 2, 3, 7, 64, 512):
        xs, ys = O.merge_path(rp, M, D)
        nchunks = len(xs) - 1
        px, py, writes = row_rule(rp, M, nnz, D, nchunks)
        assert np.all(writes == 1)
        assert np.array_equal(px, xs) and np.array_equal(py, ys)
