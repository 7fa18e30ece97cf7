"""Lane-level model of the flat walk (spmm_flat_unit in
segtaco_gb300/csrc/spmm_kernels.cuh), for the CPU tests.

Each warp is 32 numpy lanes; shuffles, ballots and loads follow the kernel
line by line.  Every load index is checked against its buffer, every loop is
bounded, plain stores must hit each row exactly once per slab and atomics only
rows split by the merge-path partition, and the product is compared with a
dense one.  When the kernel's walk changes, this model changes with it.
"""
import numpy as np

from oracle import oracle as O

INT_MAX = 2**31 - 1
L = np.arange(32)

def shfl(x, src):
    src = np.asarray(src) if not np.isscalar(src) else np.full(32, src)
    assert np.all((src >= 0) & (src < 32))
    return x[src]

def shfl_up(x, d):
    out = x.copy()
    out[d:] = x[:32 - d]
    return out

def shfl_down(x, d):
    out = x.copy()
    out[:32 - d] = x[d:]
    return out

class Mem:
    def __init__(self, A, B, N, ldc):
        self.A, self.B, self.N = A, B, N
        self.C = np.full((A.M, ldc), np.nan)
        self.writes = np.zeros(A.M, int)
        self.atom = np.zeros(A.M, int)
    def rp(self, idx):
        idx = np.asarray(idx)
        assert np.all((idx >= 0) & (idx <= self.A.M)), idx
        return self.A.row_ptr[idx].astype(np.int64)
    def col(self, idx):
        assert np.all((idx >= 0) & (idx < self.A.nnz))
        return self.A.col[idx].astype(np.int64)
    def val(self, idx):
        assert np.all((idx >= 0) & (idx < self.A.nnz))
        return self.A.val[idx].astype(np.float64)

def flat_unit(mem, V, G, ROWS, w, slab, part_x=None, part_y=None, R=None):
    A = mem.A
    M = A.M
    P = 32 // G
    Q = G
    U = min(Q, 8)
    slot = L // G
    gl = L & (G - 1)
    col0 = slab * (G * V) + gl * V
    active = col0 < mem.N
    cbase = np.where(active, col0, 0)
    if ROWS:
        x0 = w * R
        x1 = min(x0 + R, M)
        y0 = int(mem.rp(x0)); y1 = int(mem.rp(x1))
        head_split = tail_open = False
    else:
        x0, y0, x1, y1 = int(part_x[w]), int(part_y[w]), int(part_x[w + 1]), int(part_y[w + 1])
        head_split = x0 < M and mem.rp(x0) < y0
        tail_open = x1 < M and mem.rp(x1) < y1
    last = x1 if tail_open else x1 - 1
    acc = np.zeros((32, V)); head = np.zeros((32, V))

    def load_b(j):
        assert np.all((j >= 0) & (j < A.K)), j
        cols = cbase[:, None] + np.arange(V)[None, :]
        assert np.all(cols < mem.B.shape[1])
        return mem.B[j[:, None], cols]

    def store(rows, vals, lanes, atomic):
        for l in np.nonzero(lanes)[0]:
            r = rows[l] if not np.isscalar(rows) else rows
            assert 0 <= r < M
            c = col0[l]
            if atomic[l] if not np.isscalar(atomic) else atomic:
                mem.C[r, c:c + V] += vals[l]
                mem.atom[r] += 1
            else:
                mem.C[r, c:c + V] = vals[l]
                mem.writes[r] += (1 if gl[l] == 0 else 0)

    rp0 = int(mem.rp(x0)) if x0 < M else y0
    if not ROWS:
        assert head_split == (rp0 < y0)
    def load_rw(wb):
        idx = wb + L
        ok = idx < M
        return np.where(ok, mem.rp(np.where(ok, idx + 1, 0)), INT_MAX)
    wb = x0
    rw = load_rw(wb)
    p0 = y0
    okc = L < y1 - p0
    mc = np.where(okc, mem.col(np.where(okc, p0 + L, 0)), 0) if A.nnz else np.zeros(32, np.int64)
    mv = np.where(okc, mem.val(np.where(okc, p0 + L, 0)), 0.0) if A.nnz else np.zeros(32)
    # empty rows from the window
    e = rw.copy(); before = rp0
    rb = x0
    while rb <= last:
        if rb != x0:
            e = load_rw(rb)
        sb = shfl_up(e, 1); sb[0] = before
        empty = (rb + L <= last) & (e == sb)
        before = int(e[31])
        m = int(sum(1 << i for i in range(32) if empty[i]))
        while m:
            mm = m
            pos = np.full(32, -1)
            for q in range(P):
                b = (mm & -mm).bit_length() - 1 if mm else -1
                pos[slot == q] = b
                mm &= mm - 1 if mm else 0
            sel = (pos >= 0) & active
            store(rb + pos, acc, sel, False)
            m = mm
        rb += 32
    iters = 0
    while p0 < y1:
        iters += 1
        assert iters < 10 * (y1 - y0 + 64) + M
        wend = int(rw[31])
        guard = 0
        while wend <= p0:
            guard += 1; assert guard <= M // 32 + 2
            wb += 32
            rw = load_rw(wb)
            wend = int(rw[31])
        pe = min(p0 + 32, y1, wend)
        nb = pe - p0
        assert nb >= 1
        okn = L < y1 - pe
        mcn = np.where(okn, mem.col(np.where(okn, pe + L, 0)), 0)
        mvn = np.where(okn, mem.val(np.where(okn, pe + L, 0)), 0.0)
        p = p0 + L
        rr = np.zeros(32, np.int64)
        for st in (16, 8, 4, 2, 1):
            cand = shfl(rw, rr + st - 1)
            rr = np.where(cand <= p, rr + st, rr)
        rend = shfl(rw, rr)
        code = np.where(L < nb, (rr << 2) | 2 | np.where(rend == p + 1, 1, 0), 0)
        acc[slot != 0] = 0
        flushed = np.zeros(32, bool)
        hrow = np.zeros(32, np.int64)
        kend = min(nb, Q)
        for k0 in range(0, kend, U):
            bs = []; cds = []
            for u in range(U):
                t = slot * Q + k0 + u
                j = shfl(mc, t)
                cd = shfl(code, t)
                valid = (cd & 2) != 0
                jj = np.where(valid, j, 0)
                bb = load_b(jj)
                bb[~valid] = np.nan
                bs.append(bb); cds.append(cd)
            for u in range(U):
                t = slot * Q + k0 + u
                x = shfl(mv, t)
                cd = cds[u]
                valid = (cd & 2) != 0
                acc[valid] = acc[valid] + x[valid, None] * bs[u][valid]
                fl = (cd & 1) != 0
                row = wb + (cd >> 2)
                direct = fl & ((slot == 0) | flushed)
                atomic = np.zeros(32, bool) if ROWS else (((row == x0) & head_split) | ((row == x1) & tail_open))
                store(row, acc, direct & active, atomic)
                defer = fl & ~direct
                head[defer] = acc[defer]
                hrow = np.where(defer, row, hrow)
                flushed |= fl
                acc[fl] = 0
        # every valid position must have been covered by the sub-blocks
        covered = np.zeros(32, bool)
        for k0 in range(0, kend, U):
            for u in range(U):
                t = slot * Q + k0 + u
                covered[t[(t < 32)]] = True
        assert covered[:nb].all()
        if P > 1:
            sc = acc.copy()
            f = flushed.astype(int)
            d = 1
            while d < P:
                fo = shfl_up(f, d * G)
                o = shfl_up(sc, d * G)
                upd = slot >= d
                add = upd & (f == 0)
                sc[add] += o[add]
                f = np.where(upd, f | fo, f)
                d <<= 1
            inn = shfl_up(sc, G)
            sel = (slot > 0) & flushed & active
            head[sel] += inn[sel]
            atomic = np.zeros(32, bool) if ROWS else (((hrow == x0) & head_split) | ((hrow == x1) & tail_open))
            store(hrow, head, sel, atomic)
            acc = sc[(P - 1) * G + gl].copy()
        p0 = pe
        mc, mv = mcn, mvn
    if (not ROWS) and tail_open:
        sel = (slot == 0) & active
        store(x1, acc, sel, np.ones(32, bool))

def run(A, N, V, G, ROWS, R=4, D=64, seed=0):
    rng = np.random.default_rng(seed)
    B = rng.uniform(-1, 1, size=(A.K, max(N, 1) + 8))
    W = G * V
    slabs = (N + W - 1) // W
    # pad B so col0 + V <= width
    Bp = np.zeros((A.K, slabs * W + 8)); Bp[:, :B.shape[1]] = B[:, :min(B.shape[1], Bp.shape[1])]
    Bp[:, N:] = 0
    mem = Mem(A, Bp, N, slabs * W + 8)
    if ROWS:
        units = (A.M + R - 1) // R
        px = py = None
    else:
        px, py = O.merge_path(A.row_ptr, A.M, D)
        units = len(px) - 1
        for c in range(units + 1):
            x, y = int(px[c]), int(py[c])
            if x < A.M and A.row_ptr[x] < y:
                mem.C[x, :] = 0.0
    order = rng.permutation(units)
    for s in range(slabs):
        for w in order:
            flat_unit(mem, V, G, ROWS, int(w), s, px, py, R)
    Cg = mem.C[:, :N]
    return Cg, Bp[:, :N], mem

def dense_of(A):
    D = np.zeros((A.M, A.K))
    for i in range(A.M):
        for p in range(A.row_ptr[i], A.row_ptr[i + 1]):
            D[i, A.col[p]] += A.val[p]
    return D

