"""The CPU oracle pinned against segTACO's own code (golden fixtures made by
tests/golden/make_golden.py from the reference's Eigen product,
spmm_cpu_naive, sddmm_csr_cpu_taco_ref, spmspv_csr_cpu_taco_ref,
to_eigen_csr and taco_binarySearchBefore/After)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import oracle as O

SPMM = golden_cases("spmm_")
SDDMM = golden_cases("sddmm_")
SPMSPV = golden_cases("spmspv_")


def test_fixture_inventory():
    assert len(SPMM) >= 10 and len(SDDMM) >= 2 and len(SPMSPV) >= 5


@pytest.mark.parametrize("name", SPMM)
def test_rowseq_matches_eigen_and_naive_bitexact(name):
    d = load_golden("spmm_", name)
    c = O.spmm_f32_rowseq(d["row_ptr"], d["col"], d["val"], d["B"], fma=False)
    assert np.array_equal(c, d["C_eigen"])  # SparseDenseProduct.h:141-146
    assert np.array_equal(c, d["C_naive"])  # spmm_csr_gpu.h:110-127


@pytest.mark.parametrize("name", SPMM)
def test_f64_oracle_bounds_eigen(name):
    d = load_golden("spmm_", name)
    ref = O.spmm_f64(d["row_ptr"], d["col"], d["val"], d["B"])
    S = O.spmm_absbound(d["row_ptr"], d["col"], d["val"], d["B"])
    if ref.size:
        assert O.max_bound_err(d["C_eigen"], ref, S) < 1e-5


@pytest.mark.parametrize("name", SPMM)
def test_taco_searches_bitexact(name):
    d = load_golden("spmm_", name)
    M = int(d["M"])
    for P in (1, 7, 32, 256, 3584):
        assert np.array_equal(O.block_starts_taco(d["row_ptr"], M, P), d["starts_P%d" % P])
    before = [O.taco_search_before(d["row_ptr"], 0, M, int(t)) for t in d["targets"]]
    after = [O.taco_search_after(d["row_ptr"], 0, M, int(t)) for t in d["targets"]]
    assert np.array_equal(before, d["before"]) and np.array_equal(after, d["after"])


@pytest.mark.parametrize("name", SPMM)
def test_partition_definitions(name):
    """Canonical starts / merge path / row ids agree with the linear definition
    and meet the segTACO consumer contract row_ptr[start[b]] <= b*P."""
    d = load_golden("spmm_", name)
    rp, M = d["row_ptr"], int(d["M"])
    nnz = int(rp[M])
    rows = O.row_ids(rp, M)
    assert np.array_equal(rows, np.repeat(np.arange(M), np.diff(rp)))
    for P in (1, 7, 32, 256):
        s = O.block_starts_canonical(rp, M, P)
        b = np.arange(s.shape[0]) * P
        assert np.all(rp[s] <= b)
        inside = b < nnz
        assert np.array_equal(s[inside], rows[b[inside]])
        t = O.block_starts_taco(rp, M, P)
        assert np.all(rp[t] <= np.minimum(b, nnz))  # the reference's own contract
    for D in (1, 3, 64, 256):
        xs, ys = O.merge_path(rp, M, D)
        assert xs[0] == 0 and ys[0] == 0 and xs[-1] == M and ys[-1] == nnz
        assert np.all(np.diff(xs.astype(np.int64) + ys) <= D)
        # every split is consistent: row ends taken precede nonzeros not taken
        for x, y in zip(xs, ys):
            if x > 0:
                assert rp[x] <= y
            if x < M:
                assert y <= rp[x + 1]


@pytest.mark.parametrize("name", golden_cases("spmm_"))
def test_spmv_oracle_vs_eigen(name):
    d = load_golden("spmm_", name)
    y = O.spmv_f64(d["row_ptr"], d["col"], d["val"], d["x"])
    S = O.spmm_absbound(d["row_ptr"], d["col"], d["val"], d["x"].reshape(-1, 1)).reshape(-1)
    if y.size:
        assert O.max_bound_err(d["y_eigen"], y, S) < 1e-5


@pytest.mark.parametrize("name", SDDMM)
def test_sddmm_oracle_vs_reference(name):
    d = load_golden("sddmm_", name)
    out, bound = O.sddmm_f64(d["row_ptr"], d["col"], d["val"], d["X"], d["Y"])
    assert np.all(np.abs(out - d["out"]) <= 1e-12 * np.maximum(bound, 1e-30))


def test_csr_from_coo_matches_to_eigen_csr():
    from segtaco_gb300 import synth
    d = load_golden("", "csr_from_coo")
    M, K = int(d["M"]), int(d["K"])
    keys = d["rows"].astype(np.int64) * K + d["cols"]
    order = np.argsort(keys)
    A = synth.CSR(np.zeros(M + 1, np.int32), d["cols"][order].astype(np.int32),
                  d["vals"][order], M, K)
    np.cumsum(np.bincount(d["rows"], minlength=M), out=A.row_ptr[1:])
    assert np.array_equal(A.row_ptr, d["row_ptr"])
    assert np.array_equal(A.col, d["col"]) and np.array_equal(A.val, d["val"])


def test_spmspv_oracle_matches_dense():
    from segtaco_gb300 import synth
    A = synth.random_csr(300, 250, 0.05, seed=3, p_empty=0.1)
    At = A.transpose()
    rng = np.random.default_rng(0)
    idx = rng.permutation(A.K)[: A.K // 10].astype(np.int32)
    xv = rng.uniform(-1, 1, idx.shape[0]).astype(np.float32)
    y, bound = O.spmspv_f64(At.row_ptr, At.col, At.val, A.M, idx, xv)
    x = np.zeros(A.K)
    x[idx] = xv
    dense = np.zeros((A.M, A.K))
    dense[np.repeat(np.arange(A.M), A.row_lengths()), A.col] = A.val
    assert np.allclose(y, dense @ x, rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", SPMSPV)
def test_spmspv_oracle_matches_segtaco_bitexact(name):
    """The FP64 restatement equals segTACO's spmspv_csr_cpu_taco_ref
    (spmspv_csr_gpu.h:9-32) bit for bit: same x order, same column order,
    multiply then add in double."""
    d = load_golden("spmspv_", name)
    y, bound = O.spmspv_f64(d["col_ptr"], d["row_idx"], d["val"], int(d["M"]), d["x_idx"],
                            d["x_val"])
    assert np.array_equal(y, d["y"])
    assert np.all(bound >= np.abs(y))
