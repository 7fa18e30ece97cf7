"""MatrixMarket ingest (segtaco_mtx_read): segTACO's CSR pattern bit for bit
against its own read_mtx_file (tests/golden/mtx_read.npz, made by
tests/golden/make_golden.py), the complete reading against a dense
restatement of the format, seeded values, and malformed files."""
import os
import subprocess

import numpy as np
import pytest

from segtaco_gb300 import native as N
from segtaco_gb300.mtx import read_mtx

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "mtx_read.npz"))
NAMES = sorted(k[len("text_"):] for k in GOLD.files if k.startswith("text_"))
from oracle.build import REFERENCE_TREE as REF_TREE  # the recipe resolves the tree
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write(tmp_path, name, text):
    p = tmp_path / (name + ".mtx")
    p.write_bytes(text.encode() if isinstance(text, str) else text)
    return str(p)


@pytest.mark.parametrize("name", NAMES)
def test_segtaco_pattern_matches_read_mtx_file(tmp_path, name):
    path = write(tmp_path, name, GOLD["text_" + name].tobytes())
    A = read_mtx(path, segtaco=True, values="segtaco", seed=3)
    nrow, ncol, nnz = GOLD["shape_" + name]
    assert (A.M, A.K, A.nnz) == (nrow, ncol, nnz)
    assert np.array_equal(A.row_ptr, GOLD["rp_" + name])
    assert np.array_equal(A.col, GOLD["col_" + name])


def dense_reading(text):
    """The complete reading of a coordinate file, restated densely."""
    lines = [l.strip() for l in text.replace("\r", "").split("\n")]
    banner = lines[0].lower().split()
    field, sym = banner[3], banner[4]
    body = [l for l in lines[1:] if l and not l.startswith("%")]
    m, n, e = (int(x) for x in body[0].split())
    D = np.zeros((m, n))
    for l in body[1:1 + e]:
        t = l.split()
        i, j = int(t[0]) - 1, int(t[1]) - 1
        v = 1.0 if field == "pattern" else float(t[2])
        D[i, j] += v
        if sym != "general" and i != j:
            D[j, i] += -v if sym == "skew-symmetric" else v
    return D


@pytest.mark.parametrize("name", NAMES)
def test_complete_reading(tmp_path, name):
    text = GOLD["text_" + name].tobytes().decode()
    A = read_mtx(write(tmp_path, name, text), values="file")
    D = np.zeros((A.M, A.K))
    for i in range(A.M):
        cols = A.col[A.row_ptr[i]:A.row_ptr[i + 1]]
        assert np.all(np.diff(cols) > 0)  # sorted, merged
        D[i, cols] = A.val[A.row_ptr[i]:A.row_ptr[i + 1]]
    assert np.allclose(D, dense_reading(text), atol=1e-6)


def test_seeded_values(tmp_path):
    path = write(tmp_path, "s", GOLD["text_symmetric_pattern"].tobytes())
    a = read_mtx(path, segtaco=True, values="segtaco", seed=1)
    b = read_mtx(path, segtaco=True, values="segtaco", seed=1)
    c = read_mtx(path, segtaco=True, values="segtaco", seed=2)
    assert np.array_equal(a.val, b.val) and not np.array_equal(a.val, c.val)
    assert set(np.unique(a.val)) <= {np.float32(0.0), np.float32(0.1), np.float32(0.2)}
    assert np.all(read_mtx(path, values="ones").val == 1.0)


@pytest.mark.parametrize("text,match", [
    ("not a banner\n1 1 1\n1 1 1\n", "banner"),
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", "outside"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n", "missing"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n", "no value"),
    ("%%MatrixMarket matrix coordinate real general\n", "size line"),
])
def test_malformed_files(tmp_path, text, match):
    with pytest.raises(N.SegtacoError, match=match):
        read_mtx(write(tmp_path, "bad", text))


def test_missing_file(tmp_path):
    with pytest.raises(N.SegtacoError, match="cannot open"):
        read_mtx(str(tmp_path / "none.mtx"))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_TREE, "matrix_subset")),
                    reason="segTACO source tree not present")
def test_192bit_against_segtaco_reader(tmp_path):
    """segTACO's bundled matrix, read by both readers."""
    ref = os.path.join(ROOT, "oracle", "_ref", "ref_golden")
    if not os.path.exists(ref):
        pytest.skip("oracle/_ref not built")
    path = os.path.join(REF_TREE, "matrix_subset", "192bit", "192bit.mtx")
    out = tmp_path / "o.bin"
    subprocess.run([ref, "mtx", path, str(out)], check=True)
    raw = out.read_bytes()
    nrow, ncol, nnz = np.frombuffer(raw[:24], np.int64)
    ints = np.frombuffer(raw[24:], np.int32)
    A = read_mtx(path, segtaco=True, values="segtaco")
    assert (A.M, A.K, A.nnz) == (nrow, ncol, nnz) == (13691, 13682, 154303)
    assert np.array_equal(A.row_ptr, ints[:nrow + 1])
    assert np.array_equal(A.col, ints[nrow + 1:])
