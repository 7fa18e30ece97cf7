"""CPU model of the slot walk (spmm_kernels.cuh spmm_slot_unit): one slot
walking one merge-path chunk, step by step as the kernel does -- U positions
per round trip, the rows that end before a position stored first (empty ones
too), then the rows ending after the last position, then the open tail row.
Records every store / atomic add and every index read, so tests can check
bounds, single writes and the result against a dense product."""
import numpy as np


def merge_path_edges(row_ptr, D):
    """Chunk edges (x, y) of the merge path over {row ends} U {nonzeros},
    D items per chunk (the partition kernel's rule, partition.cu)."""
    M = len(row_ptr) - 1
    nnz = int(row_ptr[-1])
    total = M + nnz
    nch = max(1, -(-total // D))
    xs, ys = [], []
    for c in range(nch + 1):
        d = min(c * D, total)
        lo, hi = max(0, d - nnz), min(d, M)
        while lo < hi:  # x = number of row ends taken: row_ptr[x+1] <= d - x - 1
            mid = (lo + hi) // 2
            if row_ptr[mid + 1] <= d - mid - 1:
                lo = mid + 1
            else:
                hi = mid
        xs.append(lo)
        ys.append(d - lo)
    return xs, ys


def slot_walk(row_ptr, col, val, B, D, U=4, G=4):
    """C = A B by the slot walk; returns (C, log) with log of (kind, row)."""
    M = len(row_ptr) - 1
    N = B.shape[1]
    C = np.full((M, N), np.nan)
    xs, ys = merge_path_edges(row_ptr, D)
    nch = len(xs) - 1
    # the partition kernel zeroes rows that straddle a chunk edge
    for c in range(1, nch):
        r = xs[c]
        if r < M and row_ptr[r] < ys[c]:
            C[r] = 0.0
    log = []
    reads = []
    for c in range(nch):
        x, y, x1, y1 = xs[c], ys[c], xs[c + 1], ys[c + 1]
        head = x < M and row_ptr[x] < y
        tail = x1 < M and row_ptr[x1] < y1

        def row_end(r):
            assert 0 <= r + 1 <= M, r
            reads.append(("row_ptr", r + 1))
            return row_ptr[r + 1]
        acc = np.zeros(N)

        def flush(r):
            nonlocal acc
            edge = (r == x and head) or (r == x1 and tail)
            if edge:
                C[r] = (0.0 if np.isnan(C[r]).any() else C[r]) + acc
                log.append(("add", r))
            else:
                assert np.isnan(C[r]).all(), ("row stored twice", r)
                C[r] = acc
                log.append(("store", r))
            acc = np.zeros(N)
        row = x
        rend = row_end(row) if row < M else None
        p = y
        while p < y1:
            for u in range(U):
                pos = p + u
                if pos < y1:
                    while pos >= rend:
                        flush(row)
                        row += 1
                        rend = row_end(row)
                    assert 0 <= pos < len(col)
                    reads.append(("col", pos))
                    acc = acc + val[pos] * B[col[pos]]
            p += U
        while row < x1:
            flush(row)
            row += 1
        if tail:
            flush(x1)
    return C, log, reads
