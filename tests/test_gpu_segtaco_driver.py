"""segTACO's own sweep driver, unmodified (matrix_main.cpp -> spmm_csr_gpu,
built from the copy that baseline/ref_driver.py stages), run on the GPU with
every kernel name resolving to libsegtaco.so: the sweep over all 61 SpMM
variants (25 trials each, N = 4) on segTACO's bundled 192bit.mtx completes
and its CSV log holds one positive get_gpu_timer_result() per call."""
import collections
import os
import subprocess

import pytest

from baseline import ref_driver

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(not ref_driver.staged(), reason="segTACO's driver is not staged")
def test_segtaco_driver_runs_on_libsegtaco(cuda, tmp_path):
    exe = ref_driver.build()
    r = subprocess.run([exe, ref_driver.fixture_dir(), "192bit", "spmm_csr_gpu", str(tmp_path),
                        "gb300"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    log = tmp_path / "spmm_csr_gpu_4_gb300.csv"
    rows = [l.split(",") for l in log.read_text().splitlines() if l.strip()]
    assert len(rows) == 61 * 25
    assert all(row[4] == "192bit" and float(row[5]) > 0.0 for row in rows)
    per_variant = collections.Counter(tuple(row[1:4]) for row in rows)
    assert all(n % 25 == 0 for n in per_variant.values())
    kinds = {(row[1], row[2]) for row in rows}
    assert {("rb", "sr"), ("rb", "pr"), ("eb", "sr"), ("eb", "pr")} <= kinds
