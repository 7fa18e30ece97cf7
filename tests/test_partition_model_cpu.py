"""The row-driven merge-path rule of merge_path_kernel / batch_partition_kernel
(merge_path_store_row, segtaco_gb300/csrc/common.cuh) against the oracle's
binary-search partition, on the CPU: thread r writes the chunk edges c with
e_{r-1} <= c*D < e_r, e_r = row_ptr[r+1] + r + 1; thread M the rest.  The
batched form's mapping of threads to the rows of many problems (a block's
first problem found once, four rows per thread loaded together when they lie
in one problem) is restated and checked the same way."""
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


def batch_rule(problems, rows_per_thread=4, threads_per_block=256):
    """batch_partition_kernel's thread mapping: global rows t over every problem
    (M + 1 each), a thread per rows_per_thread consecutive rows; the block's
    first problem from one search, then per thread: rows that all lie in one
    problem take the e[k] = row_ptr[r0 + k] + r0 + k form, the others the
    per-row form.  Returns per problem (px, py, writes)."""
    begins, t = [], 0
    for rp, M, D, nchunks in problems:
        begins.append(t)
        t += M + 1
    total_rows = t
    out = [(np.full(n + 1, -1, np.int64), np.full(n + 1, -1, np.int64), np.zeros(n + 1, np.int64))
           for _, _, _, n in problems]

    def store(i, r, c_lo, c_hi):
        rp, M, D, nchunks = problems[i]
        total = M + int(rp[M])
        px, py, w = out[i]
        for c in range(c_lo, min(c_hi, nchunks) + 1):
            d = min(c * D, total)
            px[c], py[c] = r, d - r
            w[c] += 1

    per_block = rows_per_thread * threads_per_block
    for tb in range(0, total_rows, per_block):
        part = max(i for i, b in enumerate(begins) if b <= tb)
        for tid in range(threads_per_block):
            t0 = tb + tid * rows_per_thread
            if t0 >= total_rows:
                break
            lo = part
            while lo + 1 < len(problems) and begins[lo + 1] <= t0:
                lo += 1
            rp, M, D, nchunks = problems[lo]
            r0 = t0 - begins[lo]
            if r0 + rows_per_thread - 1 <= M:
                e = [(int(rp[r0 + k]) + r0 + k) if 0 < r0 + k <= M else 0
                     for k in range(rows_per_thread + 1)]
                c_lo = (e[0] + D - 1) // D
                for k in range(rows_per_thread):
                    r = r0 + k
                    if r < M:
                        nxt = (e[k + 1] + D - 1) // D
                        store(lo, r, c_lo, nxt - 1)
                        c_lo = nxt
                    else:
                        store(lo, r, c_lo, nchunks)
                continue
            for k in range(rows_per_thread):
                t = t0 + k
                if t >= total_rows:
                    break
                while lo + 1 < len(problems) and begins[lo + 1] <= t:
                    lo += 1
                rp, M, D, nchunks = problems[lo]
                r = t - begins[lo]
                e_prev = int(rp[r]) + r if r > 0 else 0
                c_lo = (e_prev + D - 1) // D
                if r < M:
                    store(lo, r, c_lo, (int(rp[r + 1]) + r + 1 + D - 1) // D - 1)
                else:
                    store(lo, r, c_lo, nchunks)
    return out


@pytest.mark.parametrize("seed", range(6))
def test_batch_rule_matches_oracle_partition(seed):
    """Every chunk edge of every problem of a batch written exactly once and
    equal to the oracle's partition, whatever the problems' sizes (rows of one
    thread falling in one problem or across two, tiny problems, empty rows)."""
    rng = np.random.default_rng(50 + seed)
    problems, want = [], []
    for _ in range(int(rng.integers(1, 9))):
        M = int(rng.choice([0, 1, 2, 3, 5, int(rng.integers(6, 400))]))
        lens = rng.integers(0, int(rng.choice([2, 12, 200])), M)
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
        D = int(rng.choice([1, 3, 16, 64, 512]))
        xs, ys = O.merge_path(rp, M, D)
        problems.append((rp, M, D, len(xs) - 1))
        want.append((xs, ys))
    for tpb in (2, 8, 256):
        for (px, py, w), (xs, ys) in zip(batch_rule(problems, threads_per_block=tpb), want):
            assert np.all(w == 1)
            assert np.array_equal(px, xs) and np.array_equal(py, ys)
