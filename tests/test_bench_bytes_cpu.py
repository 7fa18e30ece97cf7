"""bench.py's algorithmic bytes (the roofline numerator) and workloads: the
SpMM formula nnz*(4+4) + (M+1)*4 + K*N*s_B + M*N*4 at the configurations'
sizes, the workload names bench.py accepts, and the launches a timed step
claims."""
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


def test_result_line_is_compact():
    """The result line (printed last) carries the contract keys and a summary
    that stays under 3 KB for a fully populated measurement."""
    import json
    sched = {k: {"kernel_ms": 1.1234, "roofline_frac": 0.1591, "max_err_vs_fp64": 3.1e-7,
                 "config": {"schedule": 3}} for k in ("rb_sr", "rb_pr", "eb_sr", "eb_pr")}
    served = {"batched": {"requests_per_s": 19999.9, "p50_us": 75.1, "p99_us": 510.2},
              "per_call": {"requests_per_s": 5000.1, "p99_us": 15000.2},
              "capacity_vs_per_call": 4.12}
    ref = {"segtaco": {k: {"ms": 3.2} for k in sched}, "ours": {k: {"ms": 1.1} for k in sched},
           "max_err_vs_fp64": 1e-7}
    d = {"schedules": sched,
         "power_law_10m": {"schedules": sched, "spmv": {"ms": 0.088}},
         "reference_gpu": {"power_law": ref, "uniform16": ref},
         "vendor": {"ms_per_step": 2.2},
         "batched": {"speedup_vs_per_call": 3.2, "per_call_graph_ms": 11.9, "per_call_ms": 12.0,
                     "batched_graph_ms": 3.7, "max_err_vs_fp64": 2e-7},
         "served": dict(served, bf16_operands=served,
                        device_operands=dict(served, max_err_vs_fp64=1e-7)),
         "side_ops": {k: {"ms": 0.1234, "roofline_frac": 0.2034, "max_err_vs_fp64": 1e-7}
                      for k in ("spmv_power_law", "spmm_power_law_bf16", "spmspv_power_law",
                                "sddmm_banded_f32", "sddmm_banded_bf16", "spmm_banded_f32",
                                "spmm_banded_bf16")}}
    s = bench.compact_summary(d)
    assert len(json.dumps(s, separators=(",", ":"))) < 2200
    assert s["batched"]["speedup_vs_per_call_graph"] == 3.2
    assert set(s["schedules"]) == {"rb_sr", "rb_pr", "eb_sr", "eb_pr"}


def test_launches_per_step():
    """The launch count a step claims follows the plan: merge path + product;
    rb_pr's list + row blocks (+ the pieces' passes); rb_sr's list + long-row
    CTAs + row blocks; a plain row-block product."""
    P = "rb_pr pieces V=8 G=4 W=32 slabs=4 walk=0 halo=-1 rows_per_unit=64 parts=%d"
    assert bench.launches_per_step(True, 4096, "eb_pr chunks V=8 G=4 parts=1") == 2
    assert bench.launches_per_step(False, 4096, P % 1) == 2
    assert bench.launches_per_step(False, 4096, P % 2) == 3
    assert bench.launches_per_step(False, 4096, "rb_sr long_rows V=4 G=32 parts=1") == 3
    assert bench.launches_per_step(False, 0, "rb_pr rows V=8 G=4 parts=1") == 1


def _sample_detail():
    """A detail record shaped like the bench's, with long-ish numbers."""
    S = ("rb_sr", "rb_pr", "eb_sr", "eb_pr")

    def served_arm():
        return {"requests_per_s": 19759.4321, "p50_us": 121352.8123, "p99_us": 164767.4123}

    def served():
        return {"batched": served_arm(), "per_call": served_arm(), "capacity_vs_per_call": 4.1473,
                "max_err_vs_fp64": 1.8123e-07}
    return {
        "metric": "SpMM HBM GB/s (% of roofline)", "value": 1081.9, "unit": "GB/s", "n_gpus": 1,
        "steps": 20, "warmup": 5, "ms_per_step": 1.1023, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "power-law SpMM: A 1Mx1M Zipf(1.8) cap 50000, 2% empty rows, "
                               "N=128, fp32", "M": 1000000, "K": 1000000, "nnz": 20567850,
                   "N": 128, "schedule": "eb_pr", "col_tile": 32, "items_per_unit": 512,
                   "l2_hints": True,
                   "l2": "no flush: A 169 MB, B 512 MB, C 512 MB each exceed the 129 MB L2",
                   "parallelism": "replicas x1"},
        "roofline": {"bound": "hbm", "achieved": 1096.4, "peak": 6796.5, "unit": "GB/s",
                     "frac": 0.1613, "traffic": 6029844224, "kernel": "spmm_eb_pr_kernel",
                     "gathered_bytes": 10530739200, "gather_GBps": 9681.6, "flops": 5265369600,
                     "tflops": 4.841, "kernel_ms": 1.0877, "peak_source": "measured hbm_gbs",
                     "traffic_GBps": 5543.6, "traffic_frac": 0.8157},
        "gpu_launches": 40,
        "e2e": {"value": 251.134, "unit": "GB/s", "h2d_bytes_per_step": 680542804,
                "d2h_bytes_per_step": 512000000, "ms_per_step": 4.749, "entry_point": "spmm_eb_pr",
                "statistic": "median of 10 calls (mean 4.749 ms)"},
        "cpu_baseline": {"value": 5.154, "unit": "GB/s", "cores": 16, "kind": "port",
                         "cpu_model": "Neoverse-V2",
                         "sample": "full workload, median of 42 runs after warm-up (0.231 s "
                                   "each, 9.7 s in all)",
                         "one_thread": {"value": 0.397, "sample": "rows [0, 794298) (81.0% of "
                                                                  "nonzeros), one run"},
                         "build": "-O3 -fopenmp -mcpu=neoverse-v2"},
        "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 1, "interval_ms": 20,
                   "nvml_samples": 9, "reasons": []},
        "schedules": {s: {"kernel_ms": 1.7344, "roofline_frac": 0.1012, "max_err_vs_fp64": 2.1e-07}
                      for s in S},
        "power_law_10m": {"schedules": {s: {"kernel_ms": 1.0266} for s in S},
                          "spmv": {"ms": 0.0888}},
        "reference_gpu": {w: {"segtaco": {s: {"ms": 26.0697} for s in S},
                              "ours": {s: {"ms": 1.1173} for s in S}, "max_err_vs_fp64": 2e-07}
                          for w in ("power_law", "uniform16")},
        "vendor": {"ms_per_step": 2.2488},
        "batched": {"speedup_vs_per_call": 2.919, "per_call_graph_ms": 10.837,
                    "per_call_ms": 11.882, "batched_graph_ms": 3.712, "max_err_vs_fp64": 1.37e-07},
        "served": dict(served(), bf16_operands=served(), device_operands=served()),
        "side_ops": {k: {"ms": 0.2467, "roofline_frac": 0.2176, "max_err_vs_fp64": 2.2e-07}
                     for k in ("spmv_power_law", "spmm_power_law_bf16", "spmspv_power_law",
                               "sddmm_banded_f32", "spmm_banded_f32", "sddmm_banded_bf16",
                               "spmm_banded_bf16")},
    }


def test_result_line_fits_a_3kb_tail():
    """The result line (printed last) keeps every contract key and, with the
    summary, stays well inside the last 3 KB of output."""
    import json
    line = bench.result_line(_sample_detail())
    assert set(bench.RESULT_KEYS) <= set(line)
    assert "summary" in line and "schedules" in line["summary"]
    assert "gathered_bytes" not in line["roofline"] and line["roofline"]["frac"] == 0.1613
    assert line["cpu_baseline"]["one_thread"] == {"value": 0.397}
    assert line["clocks"] == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []}
    assert len(json.dumps(line, separators=(",", ":"))) < 2750
