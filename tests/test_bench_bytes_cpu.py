"""bench.py's algorithmic bytes (the roofline numerator) and workloads: the
SpMM formula nnz*(4+4) + (M+1)*4 + K*N*s_B + M*N*4 at the configurations'
sizes, and the workload names the bench and the driver use."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_uniform_config_bytes():
    # 16,384 x 16,384, 16 nonzeros per row, N = 32, fp32
    assert bench.algorithmic_bytes(16384, 16384, 262_144, 32) == 6_356_996


def test_power_law_bytes():
    M = K = 1_000_000
    nnz, N = 20_567_850, 128
    b = bench.algorithmic_bytes(M, K, nnz, N)
    assert b == nnz * 8 + (M + 1) * 4 + K * N * 4 + M * N * 4
    assert 1.19e9 < b < 1.20e9
    # bf16 B halves the dense-operand read only
    assert b - bench.algorithmic_bytes(M, K, nnz, N, 2) == K * N * 2


def test_workloads():
    A, B, N, desc = bench.make_workload("uniform16")
    assert (A.M, A.K, A.nnz, N, B.shape) == (16384, 16384, 262_144, 32, (16384, 32))
    A, B, N, desc = bench.make_workload("power_law_10m")
    assert (A.M, A.nnz, N) == (1_000_000, 10_083_633, 128) and "1.922" in desc
