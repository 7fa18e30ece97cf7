"""Generate the golden fixtures in this folder from segTACO's own CPU code.

Run where the segTACO source tree is present (oracle/build.py resolves its
location; SEGTACO_REFERENCE_TREE overrides it):

    python tests/golden/make_golden.py

It builds oracle/_ref (oracle/build.py), feeds the seeded inputs below to

* ``ref_golden spmm``  -> Eigen 3.4 ``EigenCSR * EigenRowMajor`` (ds.h:32-33,
  SparseDenseProduct.h:109-146) and ``spmm_cpu_naive`` (spmm_csr_gpu.h:110-127)
* ``ref_golden spmv``  -> Eigen ``EigenCSR * EigenVector``
* ``ref_golden sddmm`` -> ``sddmm_csr_cpu_taco_ref`` (sddmm_csr_gpu.h:9-50), in double
* ``ref_golden spmspv``-> ``spmspv_csr_cpu_taco_ref`` (spmspv_csr_gpu.h:9-32), in double,
                          over A stored by columns (spmspv_csr_gpu.h:37-43)
* ``ref_golden csr``   -> ``to_eigen_csr`` (ds.h:380-397) on an unsorted COO
* ``ref_golden mtx``   -> ``read_mtx_file`` (ds.h:183-268) on the MatrixMarket
                          texts of ``mtx_texts()``
* ``ref_search``       -> ``taco_binarySearchBefore/After`` (gpu_library.h:164-205)
                          and the block-start rule of gpu_library.h:206-240

and stores inputs and outputs as compressed .npz files.  Nothing at test time
reads the reference tree; the tests only read these files.

    python tests/golden/make_golden.py spmspv

writes only the SpMSpV fixtures (the others are left as they are).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from segtaco_gb300 import synth  # noqa: E402

SEARCH_P = (1, 7, 32, 256, 3584)


def _write(path, *arrays):
    with open(path, "wb") as f:
        for a in arrays:
            f.write(np.ascontiguousarray(a).tobytes())


def _run(binary, *args):
    subprocess.run([binary, *args], check=True)


def mtx_texts():
    """MatrixMarket files covering the reader's branches (all entries valid;
    none where deduplication would leave fewer coordinates than the header
    declares, on which segTACO's reader reads past its list)."""
    rng = np.random.default_rng(41)
    t = {}
    # general real: unsorted entries, a duplicate, comments and a blank line
    ent = [(3, 1, 0.5), (1, 2, -1.0), (2, 2, 2.0), (1, 2, 3.0), (4, 4, 1.5), (1, 1, 7.0)]
    t["general_real"] = ("%%MatrixMarket matrix coordinate real general\n% comment\n\n4 5 6\n" +
                         "".join("%d %d %g\n" % e for e in ent))
    # symmetric pattern with diagonal entries (lower triangle stored)
    pairs = sorted({(int(i), int(j)) for i, j in rng.integers(1, 31, (60, 2)) if i >= j})
    t["symmetric_pattern"] = ("%%MatrixMarket matrix coordinate pattern symmetric\n" +
                              "30 30 %d\n" % len(pairs) + "".join("%d %d\n" % p for p in pairs))
    # symmetric real: mirroring exceeds the header count (the cut applies)
    pairs = sorted({(int(i), int(j)) for i, j in rng.integers(1, 41, (120, 2)) if i > j})
    t["symmetric_real_cut"] = ("%%MatrixMarket matrix coordinate real symmetric\n" +
                               "40 40 %d\n" % len(pairs) +
                               "".join("%d %d %.3f\n" % (i, j, (i + j) / 10) for i, j in pairs))
    # skew-symmetric and hermitian (segTACO treats both as general)
    t["skew_real"] = ("%%MatrixMarket matrix coordinate real skew-symmetric\n5 5 3\n"
                      "2 1 1.0\n4 3 -2.0\n5 1 0.5\n")
    t["hermitian_complex"] = ("%%MatrixMarket matrix coordinate complex hermitian\n4 4 4\n"
                              "1 1 1.0 0.0\n3 1 2.0 1.0\n4 2 -1.0 0.5\n4 4 3.0 0.0\n")
    # integer, CRLF line ends, a column-only tail
    t["integer_crlf"] = ("%%MatrixMarket matrix coordinate integer general\r\n3 7 4\r\n"
                         "1 7 5\r\n3 1 -2\r\n2 4 9\r\n3 7 1\r\n")
    t["empty"] = "%%MatrixMarket matrix coordinate real general\n6 3 0\n"
    return t


def spmm_cases():
    cases = {}
    pat = np.array([[1, 0, 1, 0, 0], [0, 0, 0, 0, 0], [0, 1, 0, 1, 1], [1, 0, 0, 0, 1]], bool)
    vals = np.arange(1, 21, dtype=np.float32).reshape(4, 5) / 8.0
    cases["tiny_n3"] = (synth.csr_from_dense_pattern(pat, vals), 3)
    cases["rand_n4"] = (synth.random_csr(300, 280, 0.05, seed=1, p_empty=0.1), 4)
    # The reference harness's own value distribution: rand()%3/10 and B = ones (ds.h:270-285).
    A = synth.random_csr(500, 400, 0.03, seed=2)
    A.val = (np.random.default_rng(2).integers(0, 3, A.nnz) / 10.0).astype(np.float32)
    cases["refvals_ones_n4"] = (A, 4)
    cases["powerlaw_n33"] = (synth.power_law(2000, 2000, 1.8, 1500, 0.02, seed=3), 33)
    cases["uniform16_n32"] = (synth.uniform_rows(1024, 1024, 16, seed=4), 32)
    cases["longrow_n128"] = (synth.random_csr(64, 512, 0.004, seed=5, long_rows={7: 400, 40: 300}), 128)
    cases["rand_n1"] = (synth.random_csr(700, 600, 0.02, seed=6, p_empty=0.05), 1)
    cases["rand_n5"] = (synth.random_csr(700, 600, 0.02, seed=7, p_empty=0.05), 5)
    cases["lastrow_only_n8"] = (synth.random_csr(100, 90, 0.0, seed=8, long_rows={99: 50}), 8)
    empty = synth.CSR(np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 5, 7)
    cases["empty_n4"] = (empty, 4)
    return cases


def spmspv_cases():
    """(A as CSR, x indices, x values): y = A x with A stored by columns.  The
    reference driver draws x as a shuffled index list cut at 10 % of K with
    values in [0, 1) (spmspv_csr_gpu.h:53-72); the cases keep that shape and
    add the edges: empty columns, one long column, an empty x, x over all of K."""
    cases = {}
    rng = np.random.default_rng(51)

    def x_of(K, frac, seed):
        r = np.random.default_rng(seed)
        idx = r.permutation(K)[: int(K * frac)].astype(np.int32)  # unsorted, distinct
        return idx, r.uniform(0.0, 1.0, idx.shape[0]).astype(np.float32)

    A = synth.random_csr(400, 350, 0.04, seed=52, p_empty=0.1)
    cases["rand_nx10"] = (A, *x_of(A.K, 0.1, 53))
    # every second column empty, x over all columns (half of them empty)
    A = synth.random_csr(300, 200, 0.05, seed=54)
    keep = (A.col % 2) == 0
    rows = np.repeat(np.arange(A.M), A.row_lengths())[keep]
    rp = np.zeros(A.M + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=A.M), out=rp[1:])
    A = synth.CSR(rp.astype(np.int32), A.col[keep], A.val[keep], A.M, A.K)
    cases["empty_cols"] = (A, *x_of(A.K, 1.0, 55))
    # one column holding 3,000 of the 3,000 rows, plus scattered others
    A = synth.random_csr(3000, 64, 0.01, seed=56)
    dense = np.zeros((A.M, A.K), bool)
    dense[np.repeat(np.arange(A.M), A.row_lengths()), A.col] = True
    dense[:, 17] = True
    vals = rng.uniform(-1, 1, dense.shape).astype(np.float32)
    A = synth.csr_from_dense_pattern(dense, vals)
    idx, xv = x_of(A.K, 0.25, 57)
    if 17 not in idx:
        idx[0] = 17
    cases["long_col"] = (A, idx, xv)
    A = synth.random_csr(100, 120, 0.05, seed=58)
    cases["empty_x"] = (A, np.zeros(0, np.int32), np.zeros(0, np.float32))
    # power-law column lengths (the transpose of a power-law row matrix)
    A = synth.power_law(2500, 2000, 1.8, 1500, 0.02, seed=59).transpose()
    cases["powerlaw_cols_nx10"] = (A, *x_of(A.K, 0.1, 60))
    return cases


def make_spmspv(g, fin, fout):
    for name, (A, idx, xv) in spmspv_cases().items():
        At = A.transpose()  # CSC of A: col_ptr over K columns, row indices
        _write(fin, np.array([A.M, A.K, A.nnz, idx.shape[0]], np.int64), At.row_ptr, At.col,
               At.val.astype(np.float64), idx, xv.astype(np.float64))
        _run(g, "spmspv", fin, fout)
        y = np.fromfile(fout, np.float64)
        assert y.shape[0] == A.M
        np.savez_compressed(os.path.join(HERE, "spmspv_%s.npz" % name), col_ptr=At.row_ptr,
                            row_idx=At.col, val=At.val, M=A.M, K=A.K, x_idx=idx, x_val=xv, y=y)


def main():
    refs = obuild.build_ref()
    if not refs:
        raise SystemExit("segTACO source tree not found; cannot make golden fixtures")
    g, s = refs["ref_golden"], refs["ref_search"]
    tmp = tempfile.mkdtemp(prefix="segtaco_golden_")
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    make_spmspv(g, fin, fout)
    if sys.argv[1:] == ["spmspv"]:
        print("SpMSpV fixtures written to", HERE)
        return

    # ---- SpMM + SpMV + searches -------------------------------------------
    out = {}
    for name, (A, N) in spmm_cases().items():
        B = synth.dense(A.K, N, seed=1000 + N)
        if name == "refvals_ones_n4":
            B = np.ones((A.K, N), np.float32)
        _write(fin, np.array([A.M, A.K, N, A.nnz], np.int64), A.row_ptr, A.col, A.val, B)
        _run(g, "spmm", fin, fout)
        res = np.fromfile(fout, np.float32)
        C_eigen = res[: A.M * N].reshape(A.M, N)
        C_naive = res[A.M * N:].reshape(A.M, N)
        x = synth.dense(A.K, 1, seed=77).reshape(-1)
        _write(fin, np.array([A.M, A.K, A.nnz], np.int64), A.row_ptr, A.col, A.val, x)
        _run(g, "spmv", fin, fout)
        y = np.fromfile(fout, np.float32)
        nnz = A.nnz
        targets = np.unique(np.concatenate([np.arange(0, nnz + 2), [nnz + 10]])).astype(np.int32) \
            if nnz < 4000 else np.unique(np.linspace(0, nnz + 5, 4000).astype(np.int32))
        _write(fin, np.array([A.M, len(SEARCH_P)], np.int64), A.row_ptr,
               np.array(SEARCH_P, np.int32), np.array([targets.shape[0]], np.int64), targets)
        _run(s, fin, fout)
        sr = np.fromfile(fout, np.int32)
        off = 0
        starts = {}
        for P in SEARCH_P:
            n = (nnz + P - 1) // P + 1
            starts[P] = sr[off: off + n]
            off += n
        before = sr[off: off + targets.shape[0]]
        after = sr[off + targets.shape[0]:]
        rec = dict(row_ptr=A.row_ptr, col=A.col, val=A.val, M=A.M, K=A.K, B=B,
                   C_eigen=C_eigen, C_naive=C_naive, x=x, y_eigen=y,
                   targets=targets, before=before, after=after)
        for P in SEARCH_P:
            rec["starts_P%d" % P] = starts[P]
        out[name] = rec
    for name, rec in out.items():
        np.savez_compressed(os.path.join(HERE, "spmm_%s.npz" % name), **rec)

    # ---- SDDMM (reference computes in double) -----------------------------
    for name, (A, D) in {"rand_d16": (synth.random_csr(300, 280, 0.05, seed=11, p_empty=0.1), 16),
                         "powerlaw_d64": (synth.power_law(800, 800, 1.8, 600, 0.02, seed=12), 64)}.items():
        X = synth.dense(A.M, D, seed=21)
        Y = synth.dense(A.K, D, seed=22)
        _write(fin, np.array([A.M, A.K, D, A.nnz], np.int64), A.row_ptr, A.col,
               A.val.astype(np.float64), X.astype(np.float64), Y.astype(np.float64))
        _run(g, "sddmm", fin, fout)
        o = np.fromfile(fout, np.float64)
        np.savez_compressed(os.path.join(HERE, "sddmm_%s.npz" % name), row_ptr=A.row_ptr,
                            col=A.col, val=A.val, M=A.M, K=A.K, X=X, Y=Y, out=o)

    # ---- CSR construction from an unsorted COO ----------------------------
    rng = np.random.default_rng(31)
    M, K = 50, 40
    keys = np.unique(rng.integers(0, M * K, 300))
    perm = rng.permutation(keys.shape[0])
    rows = (keys // K).astype(np.int32)[perm]
    cols = (keys % K).astype(np.int32)[perm]
    vals = rng.uniform(-1, 1, keys.shape[0]).astype(np.float32)
    _write(fin, np.array([M, K, keys.shape[0]], np.int64), rows, cols, vals)
    _run(g, "csr", fin, fout)
    r = np.fromfile(fout, np.int32)
    rp = r[: M + 1]
    nnz = int(rp[-1])
    col = r[M + 1: M + 1 + nnz]
    val = r[M + 1 + nnz:].view(np.float32)
    np.savez_compressed(os.path.join(HERE, "csr_from_coo.npz"), M=M, K=K, rows=rows, cols=cols,
                        vals=vals, row_ptr=rp, col=col, val=val)
    # ---- MatrixMarket reading -----------------------------------------------
    rec = {}
    for name, text in mtx_texts().items():
        path = os.path.join(tmp, name + ".mtx")
        with open(path, "w", newline="") as f:
            f.write(text)
        _run(g, "mtx", path, fout)
        raw = open(fout, "rb").read()
        nrow, ncol, nnz = np.frombuffer(raw[:24], np.int64)
        ints = np.frombuffer(raw[24:], np.int32)
        rec["text_" + name] = np.frombuffer(text.encode(), np.uint8)
        rec["shape_" + name] = np.array([nrow, ncol, nnz], np.int64)
        rec["rp_" + name] = ints[: nrow + 1]
        rec["col_" + name] = ints[nrow + 1: nrow + 1 + nnz]
    np.savez_compressed(os.path.join(HERE, "mtx_read.npz"), **rec)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
