"""The flat walk's index arithmetic on the CPU (tests/flat_walk_model.py):
results, bounds, single writes and termination over the edge cases."""
import numpy as np
import pytest

from flat_walk_model import dense_of, run
from segtaco_gb300 import synth

CASES = {
    "powerlaw": lambda: synth.power_law(300, 250, 1.8, 200, 0.05, seed=1),
    "half_empty": lambda: synth.random_csr(200, 90, 0.05, seed=2, p_empty=0.5),
    "one_long": lambda: synth.random_csr(3, 3000, 0.0, seed=3, long_rows={1: 1500}),
    "empty_run": lambda: synth.random_csr(300, 50, 0.0, seed=4, long_rows={0: 40, 150: 70, 299: 5}),
    "single": lambda: synth.random_csr(1, 1, 1.0, seed=5),
    "all_empty": lambda: synth.random_csr(70, 10, 0.0, seed=6),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("V,G", [(4, 8), (4, 32), (2, 4), (1, 1)])
@pytest.mark.parametrize("rows", [False, True])
def test_flat_walk_model(name, V, G, rows):
    A = CASES[name]()
    Dn = dense_of(A)
    for N, D in ((5, 16), (40, 64)):
        Cg, Bn, mem = run(A, N, V, G, rows, R=3, D=D, seed=N)
        slabs = (N + G * V - 1) // (G * V)
        split = mem.atom > 0
        assert np.all(mem.writes[~split] == slabs)
        assert np.all(mem.writes[split] == 0)
        assert not np.isnan(Cg).any()
        assert np.max(np.abs(Cg - Dn @ Bn), initial=0.0) < 1e-9
