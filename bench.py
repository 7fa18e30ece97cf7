"""Benchmark of the CSR SpMM hot path on the GB300.

Workload (default): the power-law SpMM -- A 1,000,000 x 1,000,000, Zipf(1.8)
row lengths capped at 50,000 with 2 % empty rows, uniform columns, values
U[-1,1] (seed 0; about 20.6M nonzeros), B dense 1,000,000 x 128 fp32 U[-1,1]
(seed 1), C 1,000,000 x 128 fp32.  Synthetic stand-in for segTACO's
SuiteSparse sweep.  Every operand is larger than the 129 MB L2, so no flush is
needed between steps.

A step is one SpMM C = A B through the C ABI (segtaco_spmm_partition +
segtaco_spmm), operands resident in HBM.  `value` = algorithmic bytes per
step / device time per step, where algorithmic bytes = nnz*(4+4) + (M+1)*4 +
K*N*4 + M*N*4 (index + value streams, row_ptr, B read once, C written once).
`roofline` is the same byte count over the product kernel's own event-timed
duration, against the measured HBM copy bandwidth; its `traffic` is the DRAM
bytes ncu measured for one launch (profiles/traffic.json), and
`traffic_GBps` / `traffic_frac` that traffic over the same duration.  `clocks`
comes from nvidia-smi and ~1 ms NVML samples during the timed region.  `e2e` runs the drop-in
entry point (segtaco_taco_call, segTACO's spmm_* surface) on pinned host
operands: copies in, product, copy out, per step.  `cpu_baseline` times the
oracle's restatement of segTACO's CPU product (Eigen's row-parallel order) on
this host's cores.

--impl reference runs only that CPU product (the reference arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMM HBM GB/s (% of roofline)"
UNIT = "GB/s"
L2_BYTES = 129e6


def algorithmic_bytes(M, K, nnz, N, esz=4):
    return nnz * 8 + (M + 1) * 4 + K * N * esz + M * N * 4


def make_workload(name):
    from segtaco_gb300 import synth
    if name == "power_law":
        A = synth.power_law(seed=0)
        N = 128
        desc = "power-law SpMM: A 1Mx1M Zipf(1.8) cap 50000, 2% empty rows, N=128, fp32"
    elif name == "power_law_10m":
        A = synth.power_law(s=1.922, seed=0)
        N = 128
        desc = ("power-law SpMM, ~10M-nonzero variant: A 1Mx1M Zipf(1.922) cap 50000, "
                "2% empty rows, N=128, fp32")
    elif name == "power_law_quarter":
        A = synth.power_law(250_000, 250_000, seed=0)
        N = 128
        desc = "power-law SpMM (quarter size, for profiling): A 250kx250k Zipf(1.8) cap 50000, N=128, fp32"
    elif name == "uniform16":
        A = synth.uniform_rows(seed=0)
        N = 32
        desc = "uniform SpMM: A 16384x16384, 16 nnz/row, N=32, fp32"
    elif name == "banded":
        A = synth.banded_plus_random(seed=0)
        N = 64
        desc = "banded+random SpMM: A 262144^2, |i-j|<=32 + 8/row, N=64, fp32"
    else:
        raise SystemExit("unknown workload " + name)
    B = synth.dense(A.K, N, seed=1)
    return A, B, N, desc


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(workload, kernel):
    """Per-launch DRAM bytes of `kernel` on `workload` from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)[workload][kernel]
    except Exception:
        return None


class NvmlReader:
    """Read-only NVML queries (the driver's libnvidia-ml) of the SM clock, its
    maximum and the clock-event reasons, polled by a thread every ~1 ms so a
    region of a few tens of milliseconds still gets many samples.  Settings are
    never changed.  Unavailable NVML leaves it empty."""
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
            0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        import ctypes as C
        import threading
        self.samples, self._stop, self._t = [], threading.Event(), None
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return
            h = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(h)) != 0:
                return
            reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self._q = (lib, h, reasons, C)
        except Exception:
            self._q = None

    def _poll(self):
        lib, h, reasons, C = self._q
        clk, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self._stop.is_set():
            if (lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 and
                    reasons(h, C.byref(rs)) == 0):
                self.samples.append((float(clk.value), float(mx.value),
                                     {n for b, n in self.BITS.items() if rs.value & b}))
            time.sleep(0.001)

    def start(self):
        import threading
        if getattr(self, "_q", None):
            self._t = threading.Thread(target=self._poll, daemon=True)
            self._t.start()

    def stop(self):
        if self._t is not None:
            self._stop.set()
            self._t.join(timeout=2)
        return self.samples


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region
    (plus NvmlReader's ~1 ms samples of the same quantities)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.nvml = NvmlReader(index)

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # nvidia-smi takes a moment to start: wait for its first sample so
            # that sampling covers the timed region that follows
            t0 = time.time()
            while time.time() - t0 < 3.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
            self.first = os.path.getsize(self.path)
        except Exception:
            self.proc = None
        # last, so that its samples start with the timed region
        self.nvml.start()

    def stop(self):
        fine = self.nvml.stop()
        if self.proc is None:
            return self._summary([], fine)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        before, inside = [], []  # samples taken before / after the region began
        with open(self.path) as f:
            data = f.read()
        os.unlink(self.path)
        first = getattr(self, "first", 0)
        pos = 0
        for line in data.splitlines(keepends=True):
            start, pos = pos, pos + len(line)
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rec = (float(parts[1]), float(parts[2]),
                       {nm for nm, v in zip(names, parts[5:9]) if v.lower() == "active"})
            except ValueError:
                continue
            (inside if start >= first else before).append(rec)
        use = inside or before[-1:]  # a region shorter than the interval: the last sample
        return self._summary(use, fine, len(inside))

    @staticmethod
    def _summary(smi, fine, smi_inside=0):
        use = smi + fine
        if not use:
            return None
        return {"sm_mhz": statistics.median(r[0] for r in use), "sm_max_mhz": max(r[1] for r in use),
                "samples": smi_inside, "interval_ms": 20, "nvml_samples": len(fine),
                "reasons": sorted(set().union(*(r[2] for r in use)))}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), read only."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_baseline_build():
    from oracle import build as obuild
    return " ".join(obuild.timed_flags())


def cpu_spmm_timed(A, B, reps, threads=0, frac=1.0):
    """Time the oracle's FP32 row-parallel product (segTACO's Eigen order) on
    the first `frac` of the rows; returns (seconds per rep, rows, nnz, threads)."""
    import numpy as np
    from oracle import oracle as O
    M = max(1, int(A.M * frac))
    rp = np.ascontiguousarray(A.row_ptr[: M + 1])
    nnz = int(rp[M])
    col = A.col[:nnz]
    val = A.val[:nnz]
    Bc = np.ascontiguousarray(B)
    out = np.empty((M, B.shape[1]), np.float32)
    O.cpu_spmm(rp, col, val, Bc, out, threads)  # warm-up (page-in, thread pool)
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.cpu_spmm(rp, col, val, Bc, out, threads)
        t.append(time.perf_counter() - t0)
    used = threads if threads > 0 else O.cpu_threads()
    return statistics.median(t), M, nnz, used


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() and args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference arm: segTACO's CPU product order on this host's cores."""
    if rank != 0:
        return
    A, B, N, desc = make_workload(args.workload)
    byts = algorithmic_bytes(A.M, A.K, A.nnz, N)
    # Size each step so warm-up + steps stay within ~2 minutes.
    t_full, _, _, threads = cpu_spmm_timed(A, B, 1)
    frac = min(1.0, 120.0 / max(1, args.steps + args.warmup) / max(t_full, 1e-9))
    frac = max(frac, 0.01)
    for _ in range(args.warmup):
        cpu_spmm_timed(A, B, 1, frac=frac)
    sec, Ms, nnzs, threads = cpu_spmm_timed(A, B, args.steps, frac=frac)
    share = nnzs / max(1, A.nnz)
    value = byts * share / sec / 1e9
    sample = ("rows [0, %d) of the workload (%.1f%% of nonzeros) per step, median of %d steps"
              % (Ms, 100 * share, args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": desc, "M": A.M, "K": A.K, "nnz": A.nnz, "N": N},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _b_dtype(N_, Bd):
    """The dense operand's type code (bf16 B travels as bf16 or int16 bits)."""
    import torch
    return N_.BF16 if Bd.dtype in (torch.bfloat16, torch.int16) else N_.F32


def time_spmm(ops, N_, Ad, Bd, Cd, cfg, ws, stream, steps, warmup):
    """Per-step device time and product-kernel time (ms) via events on `stream`."""
    import torch
    cfg_ready = N_.Config.make(**{**cfg.as_dict(), "flags": cfg.flags | N_.FLAG_PARTITION_READY})
    dt = _b_dtype(N_, Bd)
    for _ in range(warmup):
        ops.spmm_partition(Ad, Cd, cfg, ws, b_dtype=dt, stream=stream)
        ops.spmm(Ad, Bd, C_out=Cd, config=cfg_ready, workspace=ws, stream=stream)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for i in range(steps):
        ev[i][0].record(stream)
        ops.spmm_partition(Ad, Cd, cfg, ws, b_dtype=dt, stream=stream)
        ev[i][1].record(stream)
        ops.spmm(Ad, Bd, C_out=Cd, config=cfg_ready, workspace=ws, stream=stream)
        ev[i][2].record(stream)
    torch.cuda.synchronize()
    step = sum(e[0].elapsed_time(e[2]) for e in ev) / steps
    kern = sum(e[1].elapsed_time(e[2]) for e in ev) / steps
    return step, kern


def time_spmm_graph(ops, N_, Ad, Bd, Cd, cfg, ws, stream, reps, warmup):
    """Per-step device time (ms) of partition + product replayed from a CUDA
    graph of one step on `stream` (no host work between the launches, as
    segTACO's timer brackets only its own launches)."""
    import torch
    cfg_ready = N_.Config.make(**{**cfg.as_dict(), "flags": cfg.flags | N_.FLAG_PARTITION_READY})
    dt = _b_dtype(N_, Bd)

    def step():
        ops.spmm_partition(Ad, Cd, cfg, ws, b_dtype=dt, stream=stream)
        ops.spmm(Ad, Bd, C_out=Cd, config=cfg_ready, workspace=ws, stream=stream)
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        step()
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            g.replay()
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def sampled_spmm_err(A, B, C, rows):
    """Max over `rows` of |c - c64| / sum_p |a_ip b_pk| (the tests' bound-
    normalised error) against an FP64 product of A and B (host; fp32 values,
    or bf16 values already widened).  C[k] is the computed row rows[k]."""
    import numpy as np
    worst = 0.0
    for k, r in enumerate(rows):
        s0, s1 = int(A.row_ptr[r]), int(A.row_ptr[r + 1])
        a = A.val[s0:s1].astype(np.float64)
        rb = B[A.col[s0:s1]].astype(np.float64)
        exact = a @ rb
        bound = np.abs(a) @ np.abs(rb)
        err = np.abs(C[k].astype(np.float64) - exact) / np.maximum(bound, 1e-30)
        worst = max(worst, float(err.max()) if err.size else 0.0)
    return worst


def sddmm_err(A, X, Y, out, esz, n=200_000, seed=8):
    """Bound-normalised error of SDDMM results at `n` sampled nonzeros:
    |o - o64| / (|a| sum_k |x_ik y_jk|), with X, Y the device factors (bf16
    factors widened exactly)."""
    import numpy as np
    import torch
    from segtaco_gb300 import synth
    torch.cuda.synchronize()

    def host(t):
        if esz == 2:
            return synth.bf16_bits_to_f32(t.view(torch.int16).cpu().numpy().view(np.uint16))
        return t.cpu().numpy()
    Xh, Yh = host(X).astype(np.float64), host(Y).astype(np.float64)
    rng = np.random.default_rng(seed)
    p = np.sort(rng.choice(A.nnz, min(n, A.nnz), replace=False))
    rows = np.searchsorted(A.row_ptr, p, side="right") - 1
    a = A.val[p].astype(np.float64)
    xi, yj = Xh[rows], Yh[A.col[p]]
    exact = a * np.einsum("ij,ij->i", xi, yj)
    bound = np.abs(a) * np.einsum("ij,ij->i", np.abs(xi), np.abs(yj))
    got = out.cpu().numpy()[p].astype(np.float64)
    return float((np.abs(got - exact) / np.maximum(bound, 1e-30)).max())


def vec_err(A, x, yd):
    """Bound-normalised error of y = A x (device yd) against FP64:
    max_i |y_i - y64_i| / sum_p |a_ip x_p|."""
    import numpy as np
    import scipy.sparse as sp
    import torch
    torch.cuda.synchronize()
    S = sp.csr_matrix((A.val.astype(np.float64), A.col, A.row_ptr), shape=(A.M, A.K))
    x64 = x.astype(np.float64)
    exact = S @ x64
    abs_S = sp.csr_matrix((np.abs(A.val.astype(np.float64)), A.col, A.row_ptr), shape=(A.M, A.K))
    bound = abs_S @ np.abs(x64)
    got = yd.cpu().numpy().astype(np.float64)
    return float((np.abs(got - exact) / np.maximum(bound, 1e-30)).max())


def rows_err(A, B, Cd, rows):
    """sampled_spmm_err for the rows `rows` of the device result Cd."""
    import torch
    got = Cd.index_select(0, torch.from_numpy(rows.astype("int64")).to(Cd.device)).cpu().numpy()
    return sampled_spmm_err(A, B, got, rows)


def sample_rows(A, n=4096, longest=16, seed=7):
    """`n` random rows plus the `longest` longest rows of A (sorted, distinct)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    lens = A.row_lengths()
    pick = rng.choice(A.M, min(n, A.M), replace=False)
    top = np.argsort(lens)[-longest:]
    return np.unique(np.concatenate([pick, top]))


def run_reference_gpu(args, N_, ops, stream, peak, A, B, C_ours=None):
    """segTACO's own generic SpMM kernels (K15 rb_sr, K20 rb_pr, K24 eb_sr,
    K30 eb_pr: dgSPARSE-style, any N <= 256) built for sm_103a from its
    headers (baseline/ref_gpu.py) and called through its host wrappers, which
    time {zero C, kernel} with its GPUTimer (get_gpu_timer_result).  Beside
    them, this library's four schedules on the same operands, timed over the
    same region (partition + product).  Runs on the headline workload (passed
    in) and on the uniform 16384^2 SpMM (N = 32)."""
    import numpy as np
    import torch
    from baseline import ref_gpu
    if not ref_gpu.available():
        return {"unavailable": "segTACO's GPU headers were not staged or the harness did not "
                               "build (baseline/ref_gpu.py)"}
    out = {"timer": "segTACO get_gpu_timer_result (zero C + kernel, launched from its C++ "
                    "wrapper), median of 7 calls after 2; ours: partition + product, the "
                    "faster of a CUDA graph of one step replayed 20 times (ms_graph: no host "
                    "work between launches, as segTACO's timer) and the same calls issued "
                    "from Python with events around them (ms_events_per_call)",
           "kernels": "K15 spmm_rb_sr, K20 spmm_rb_pr, K24 spmm_eb_sr, K30 spmm_eb_pr"}
    from segtaco_gb300 import synth
    cases = [("power_law", A, B, C_ours), ("uniform16", synth.uniform_rows(seed=0), None, None)]
    for name, Ah, Bh, Cref in cases:
        if Bh is None:
            Bh = synth.dense(Ah.K, 32, seed=1)
        N = Bh.shape[1]
        byts = algorithmic_bytes(Ah.M, Ah.K, Ah.nnz, N)
        try:
            ref = ref_gpu.run(Ah, Bh, warmup=2, reps=7)
        except Exception as exc:
            out[name] = {"error": str(exc)[:300]}
            continue
        Ad = ops.DeviceCSR.from_host(Ah, "cuda")
        Bd = torch.from_numpy(Bh).cuda()
        Cd = torch.empty((Ah.M, N), dtype=torch.float32, device="cuda")
        mx = int(Ah.row_lengths().max())
        ent = {"M": Ah.M, "nnz": Ah.nnz, "N": N, "segtaco": {}, "ours": {}}
        for s in ("rb_sr", "rb_pr", "eb_sr", "eb_pr"):
            r = ref.get("spmm_" + s)
            ms = statistics.median(r["ms"])
            c = N_.Config.make(schedule=N_.SCHEDULES[s])
            N_.check(N_.lib().segtaco_autotune_heuristic(Ah.M, Ah.K, Ah.nnz, N, N_.F32, mx, c))
            w = torch.empty(max(256, ops.spmm_workspace_size(Ad, N, N_.F32, c)),
                            dtype=torch.uint8, device="cuda")
            st, kt = time_spmm(ops, N_, Ad, Bd, Cd, c, w, stream, 10, 3)
            gt = time_spmm_graph(ops, N_, Ad, Bd, Cd, c, w, stream, 20, 3)
            torch.cuda.synchronize()
            ours_sum = float(Cd.double().sum().item())
            err = rows_err(Ah, Bh, Cd, sample_rows(Ah, 2048))
            ent.setdefault("max_err_vs_fp64", 0.0)
            ent["max_err_vs_fp64"] = max(ent["max_err_vs_fp64"], err)
            ent["segtaco"][s] = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
                                 "roofline_frac": round(byts / ms / 1e6 / peak, 4),
                                 # checksum of segTACO's C against ours (same A, B)
                                 "checksum_rel_diff": float("%.3g" % (
                                     abs(r["checksum"] - ours_sum) / max(abs(ours_sum), 1e-30)))}
            best = min(gt, st)
            ent["ours"][s] = {"ms": round(best, 4), "speedup": round(ms / best, 2),
                              "ms_graph": round(gt, 4), "ms_events_per_call": round(st, 4)}
            del w
        out[name] = ent
        del Ad, Bd, Cd
    return out


def run_power_law_variant(args, N_, ops, stream, Bd, Cd, peak):
    """The power-law configuration at Zipf exponent 1.922 (1M x 1M, cap 50,000,
    2 % empty rows: 10,083,633 nonzeros, the "~10M" of the configuration's text,
    which exponent 1.8 overshoots at 19.9M): the four schedules with the
    library's configs on the same B (N = 128) and C, and SpMV (x of 1M fp32)."""
    import torch
    from segtaco_gb300 import synth
    A = synth.power_law(s=1.922, seed=0)
    Ad = ops.DeviceCSR.from_host(A, "cuda")
    N = Bd.shape[1]
    byts = algorithmic_bytes(A.M, A.K, A.nnz, N)
    mx = int(A.row_lengths().max())
    out = {"M": A.M, "K": A.K, "nnz": A.nnz, "N": N, "zipf_s": 1.922, "max_row": mx,
           "bytes": byts, "schedules": {}}
    for s in ("rb_sr", "rb_pr", "eb_sr", "eb_pr"):
        c = N_.Config.make(schedule=N_.SCHEDULES[s])
        N_.check(N_.lib().segtaco_autotune_heuristic(A.M, A.K, A.nnz, N, N_.F32, mx, c))
        w = torch.empty(max(256, ops.spmm_workspace_size(Ad, N, N_.F32, c)), dtype=torch.uint8,
                        device="cuda")
        st, kt = time_spmm(ops, N_, Ad, Bd, Cd, c, w, stream, max(3, args.steps // 2), 2)
        out["schedules"][s] = {"config": {k: v for k, v in c.as_dict().items() if v},
                               "ms_per_step": round(st, 4), "kernel_ms": round(kt, 4),
                               "GBps": round(byts / st / 1e6, 1),
                               "roofline_frac": round(byts / kt / 1e6 / peak, 4)}
        del w
    x = torch.from_numpy(synth.dense(A.K, 1, seed=3).ravel()).cuda()
    y = torch.empty(A.M, dtype=torch.float32, device="cuda")
    ws = torch.empty(max(256, ops.spmv_workspace_size(Ad)), dtype=torch.uint8, device="cuda")
    ms = _time_events(lambda: ops.spmv(Ad, x, y, workspace=ws, stream=stream), stream,
                      max(5, args.steps // 2))
    vb = A.nnz * 8 + (A.M + 1) * 4 + A.K * 4 + A.M * 4
    out["spmv"] = {"ms": round(ms, 4), "GBps": round(vb / ms / 1e6, 1),
                   "roofline_frac": round(vb / ms / 1e6 / peak, 4), "bytes": vb}
    del Ad
    return out


def run_batched(args, N_, ops, stream, count=256):
    """Uneven-size stream: `count` pool matrices (M = K log-uniform in [1e3, 2e5],
    lognormal row lengths of mean 12, four structures, N in {16, 32, 64, 128},
    FP32).  Per-call launches (one segtaco_spmm per matrix, each with the
    library's tuned config) against the batched persistent launch, direct and
    replayed from its CUDA graph."""
    import numpy as np
    import torch
    from segtaco_gb300 import synth

    items, byts, nnz = [], 0, 0
    for m in range(count):
        A, n, _ = synth.pool_matrix(m)
        B = torch.from_numpy(synth.dense(A.K, n, seed=1000 + m)).cuda()
        C = torch.empty((A.M, n), dtype=torch.float32, device="cuda")
        items.append((ops.DeviceCSR.from_host(A, "cuda"), B, C))
        byts += algorithmic_bytes(A.M, A.K, A.nnz, n)
        nnz += A.nnz
    batch = ops.Batch(items, stream=stream)
    groups, nitems, cfgs = batch.info()
    wsz = max(max(256, ops.spmm_workspace_size(Ad, B.shape[1], N_.F32, c))
              for (Ad, B, _), c in zip(items, cfgs))
    ws = torch.empty(wsz, dtype=torch.uint8, device="cuda")

    def per_call():
        for (Ad, B, C), c in zip(items, cfgs):
            ops.spmm(Ad, B, C_out=C, config=c, workspace=ws, stream=stream)

    def timed(fn, reps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    reps = max(3, args.steps // 4)
    t_call = timed(per_call, reps)
    # the same per-call launches (partition + product per matrix) captured
    # once into a CUDA graph and replayed: no host issue cost in the loop
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        per_call()

    def replay():
        with torch.cuda.stream(stream):  # the graph runs on the timed stream
            g.replay()
    t_call_graph = timed(replay, reps)
    del g
    t_batch = timed(lambda: batch.run(stream=stream), reps)
    t_graph = timed(lambda: batch.run(stream=stream, graph=True), reps)
    # measured error of a sample of the batched products against FP64
    torch.cuda.synchronize()
    worst = 0.0
    for m in range(0, count, max(1, count // 8)):
        Ad, B, C = items[m]
        A_h, _, _ = synth.pool_matrix(m)
        Bh = B.cpu().numpy()
        worst = max(worst, rows_err(A_h, Bh, C, sample_rows(A_h, 512)))
    launches_call = sum(2 if c.schedule in (N_.EB_SR, N_.EB_PR) else 1 for c in cfgs)
    batch.close()
    scheds = {}
    for c in cfgs:
        k = {v: k for k, v in N_.SCHEDULES.items()}[c.schedule]
        scheds[k] = scheds.get(k, 0) + 1
    return {
        "workload": "%d uneven matrices, M=K log-uniform [1e3, 2e5], row lengths lognormal "
                    "mean 12, N in {16,32,64,128}, FP32; %d nnz in all" % (count, nnz),
        "metric": "SpMMs/s", "per_call_ms": round(t_call, 3),
        "per_call_graph_ms": round(t_call_graph, 3),
        "batched_ms": round(t_batch, 3),
        "batched_graph_ms": round(t_graph, 3),
        "per_call_spmms_per_s": round(count / t_call_graph * 1e3, 1),
        "batched_spmms_per_s": round(count / t_graph * 1e3, 1),
        # against the per-call launches replayed from a graph (no host in the loop)
        "speedup_vs_per_call": round(t_call_graph / t_graph, 3),
        "speedup_vs_per_call_python_loop": round(t_call / t_graph, 3),
        "max_err_vs_fp64": worst, "err_sample": "512 rows (incl. the 16 longest) of every "
                                                "%d-th product" % max(1, count // 8),
        "batched_GBps": round(byts / t_graph / 1e6, 1),
        "per_call_launches": launches_call, "batched_launches": groups + 1,
        "batch_groups": groups, "queue_items": nitems, "schedules": scheds,
        "timing": "CUDA events on one stream, mean of %d repetitions after 2" % reps,
    }


def _time_graph(fn, stream, reps, warm=3):
    """Device time (ms) per call of `fn` (stream-ordered work on `stream`)
    captured once into a CUDA graph and replayed `reps` times: no host work
    between the launches, for operations shorter than the host's issue time."""
    import torch
    with torch.cuda.stream(stream):
        for _ in range(warm):
            fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        fn()
    with torch.cuda.stream(stream):
        for _ in range(warm):
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            g.replay()
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _time_events(fn, stream, reps, warm=3):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_side_ops(args, N_, ops, stream, A_pl, peak, A_host=None):
    """The other hot-path operations at their configurations: SpMV on the
    power-law matrix (x of 1M fp32), the bf16-B SpMM on it (N = 128, B beyond
    L2), SpMSpV on the same matrix stored by
    columns (x with 10 % of K nonzero, distinct random indices, as segTACO's
    spmspv_csr_gpu.h:53-72 draws them), SDDMM with fp32 and bf16 factors of width
    64 and SpMM with fp32 and bf16 B (N = 64) on the banded-plus-random matrix
    (262,144^2, ~19.1M nonzeros).  bf16 error: max over 4,096 sampled rows of
    |c - c64| / sum |a b| against an FP64 product of the same bf16 values."""
    import numpy as np
    import torch
    from segtaco_gb300 import synth
    reps = max(5, args.steps // 2)
    out = {}
    # SpMV, power-law matrix (already resident)
    Ad = A_pl
    x = torch.from_numpy(synth.dense(Ad.K, 1, seed=3).ravel()).cuda()
    y = torch.empty(Ad.M, dtype=torch.float32, device="cuda")
    ws = torch.empty(max(256, ops.spmv_workspace_size(Ad)), dtype=torch.uint8, device="cuda")
    spmv = lambda: ops.spmv(Ad, x, y, workspace=ws, stream=stream)
    ms_ev = _time_events(spmv, stream, reps)
    ms = _time_graph(spmv, stream, reps)
    byts = Ad.nnz * 8 + (Ad.M + 1) * 4 + Ad.K * 4 + Ad.M * 4
    out["spmv_power_law"] = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
                             "roofline_frac": round(byts / ms / 1e6 / peak, 4),
                             "bytes": byts, "ms_events_per_call": round(ms_ev, 4),
                             "timing": "partition + product replayed from a CUDA graph"}
    if A_host is not None:
        out["spmv_power_law"]["max_err_vs_fp64"] = vec_err(A_host, x.cpu().numpy(), y)
    # bf16-B SpMM on the power-law matrix (N = 128, B 256 MB: beyond L2)
    bits = synth.to_bf16_bits(synth.dense(Ad.K, 128, seed=12))
    Bb = torch.from_numpy(bits.view(np.int16)).cuda().view(torch.bfloat16)
    Cb = torch.empty((Ad.M, 128), dtype=torch.float32, device="cuda")
    cfg = N_.Config.make(schedule=N_.AUTO)
    mx = int(A_host.row_lengths().max()) if A_host is not None else -1
    N_.check(N_.lib().segtaco_autotune_heuristic(Ad.M, Ad.K, Ad.nnz, 128, N_.BF16, mx, cfg))
    wsb = torch.empty(max(256, ops.spmm_workspace_size(Ad, 128, N_.BF16, cfg)), dtype=torch.uint8,
                      device="cuda")
    ms = _time_events(lambda: ops.spmm(Ad, Bb, C_out=Cb, config=cfg, workspace=wsb,
                                       stream=stream), stream, reps)
    byts = algorithmic_bytes(Ad.M, Ad.K, Ad.nnz, 128, 2)
    out["spmm_power_law_bf16"] = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
                                  "roofline_frac": round(byts / ms / 1e6 / peak, 4),
                                  "bytes": byts,
                                  "config": {k: v for k, v in cfg.as_dict().items() if v}}
    del Bb, Cb, wsb
    # SpMSpV, power-law matrix by columns (CSR of A^T), nx = K / 10
    if A_host is not None:
        At = A_host.transpose()
        Atd = ops.DeviceCSR.from_host(At, "cuda")
        rng = np.random.default_rng(0)
        nx = A_host.K // 10
        xi_h = np.sort(rng.permutation(A_host.K)[:nx]).astype(np.int32)
        xi = torch.from_numpy(xi_h).cuda()
        xv = torch.from_numpy(rng.uniform(-1, 1, nx).astype(np.float32)).cuda()
        ys = torch.empty(A_host.M, dtype=torch.float32, device="cuda")
        spmspv = lambda: ops.spmspv(Atd, xi, xv, A_host.M, ys, stream=stream)
        ms_ev = _time_events(spmspv, stream, reps)
        ms = _time_graph(spmspv, stream, reps)
        xd = np.zeros(A_host.K, np.float32)
        xd[xi_h] = xv.cpu().numpy()
        spmspv_err = vec_err(A_host, xd, ys)
        colnnz = np.diff(At.row_ptr)[xi_h].astype(np.int64)
        byts = int(nx * 8 + (8 * nx + 8 * colnnz.sum()) + A_host.M * 4)
        out["spmspv_power_law"] = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
                                   "roofline_frac": round(byts / ms / 1e6 / peak, 4),
                                   "bytes": byts, "nx": nx, "max_err_vs_fp64": spmspv_err,
                                   "ms_events_per_call": round(ms_ev, 4),
                                   "timing": "clear y + push replayed from a CUDA graph"}
        del Atd
    # banded-plus-random: SDDMM and SpMM, fp32 and bf16 dense operands
    A = synth.banded_plus_random(seed=0)
    Bd = ops.DeviceCSR.from_host(A, "cuda")
    D = 64
    X32 = synth.dense(A.M, D, seed=4)
    Y32 = synth.dense(A.K, D, seed=5)
    o = torch.empty(A.nnz, dtype=torch.float32, device="cuda")
    for name, conv, esz in (("f32", lambda a: torch.from_numpy(a).cuda(), 4),
                            ("bf16", lambda a: torch.from_numpy(synth.to_bf16_bits(a).view(np.int16))
                             .cuda().view(torch.bfloat16), 2)):
        X, Y = conv(X32), conv(Y32)
        # the library's choice from device statistics (nonzeros near the
        # diagonal: the band kernel)
        scfg = ops.sddmm_autotune(Bd, D, N_.F32 if esz == 4 else N_.BF16)
        ms = _time_events(lambda: ops.sddmm(Bd, X, Y, o, stream=stream, config=scfg), stream,
                          reps)
        byts = A.nnz * 12 + (A.M + 1) * 4 + (A.M + A.K) * D * esz
        out["sddmm_banded_" + name] = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
                                       "roofline_frac": round(byts / ms / 1e6 / peak, 4),
                                       "bytes": byts, "kernel": int(scfg.kernel),
                                       "max_err_vs_fp64": sddmm_err(A, X, Y, o, esz)}
        Bm = conv(synth.dense(A.K, D, seed=6))
        Cm = torch.empty((A.M, D), dtype=torch.float32, device="cuda")
        # the library's choice from device statistics (row lengths, nonzeros
        # near the diagonal: the staged B window for this banded matrix)
        cfg = ops.autotune(Bd, D, N_.F32 if esz == 4 else N_.BF16)
        wsz = max(256, ops.spmm_workspace_size(Bd, D, N_.F32 if esz == 4 else N_.BF16, cfg))
        w = torch.empty(wsz, dtype=torch.uint8, device="cuda")
        ms = _time_events(lambda: ops.spmm(Bd, Bm, C_out=Cm, config=cfg, workspace=w,
                                           stream=stream), stream, reps)
        byts = algorithmic_bytes(A.M, A.K, A.nnz, D, esz)
        ent = {"ms": round(ms, 4), "GBps": round(byts / ms / 1e6, 1),
               "roofline_frac": round(byts / ms / 1e6 / peak, 4), "bytes": byts,
               "schedule": {v: k for k, v in N_.SCHEDULES.items()}[cfg.schedule],
               "plan": ops.plan_name(Bd, Bm, cfg)}
        # error against FP64 over sampled rows (bf16: of the same bf16 values)
        torch.cuda.synchronize()
        rows = sample_rows(A, 4096)
        if esz == 2:
            Bh = Bm.view(torch.int16).cpu().numpy().view(np.uint16)
            Bf = synth.bf16_bits_to_f32(Bh).astype(np.float64)
            ent["max_err_vs_fp64_bf16_values"] = rows_err(A, Bf, Cm, rows)
        else:
            ent["max_err_vs_fp64"] = rows_err(A, Bm.cpu().numpy(), Cm, rows)
        ent["tolerance"] = 1e-5
        out["spmm_banded_" + name] = ent
    out["config"] = ("SpMV and SpMSpV (x 10%% nonzero): power-law 1Mx1M (%d nnz); "
                     "banded-plus-random %dx%d, %d nnz, D=N=64" % (Ad.nnz, A.M, A.K, A.nnz))
    return out


def run_gather_ceiling(ops, stream, reps=5):
    """Random-row gather throughput of this GPU (segtaco_probe_gather) over
    buffers that fit in L2 and buffers that do not: the ceilings that bound
    SpMM with scattered columns (each nonzero gathers one dense row slice)."""
    import torch
    big = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")
    out = {}
    for mb in (32, 64, 96, 128, 256, 1024):
        buf = big[:mb << 20]
        for rb in (64, 128, 512):
            n = (6 << 30) // rb
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            for _ in range(2):
                ops.probe_gather(buf, rb, n, 0, stream=stream)
            ev[0].record(stream)
            for i in range(reps):
                ops.probe_gather(buf, rb, n, 0, seed=i, stream=stream)
            ev[1].record(stream)
            torch.cuda.synchronize()
            sec = ev[0].elapsed_time(ev[1]) / reps / 1e3
            out["%dMB_%dB" % (mb, rb)] = {"GBps": round(n * rb / sec / 1e9, 1),
                                          "Glines_per_s": round(n * max(rb, 128) / 128 / sec / 1e9, 2)}
    del big
    return out


def run_link_probe(stream, gb=1):
    """Host<->device bandwidth over the Grace-Blackwell link: copy-engine
    copies of pinned memory (one direction, then both at once) and the
    SM-driven copy kernel the serving loop can use (segtaco_probe_copy)."""
    import ctypes as C
    import time
    import torch
    from segtaco_gb300 import native as N_
    n = gb << 30
    h = torch.empty(n, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(n, dtype=torch.uint8).pin_memory()
    d = torch.empty(n, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(n, dtype=torch.uint8, device="cuda")
    desc = torch.empty(256, dtype=torch.uint8, device="cuda")
    s2 = torch.cuda.Stream()
    sms = torch.cuda.get_device_properties(0).multi_processor_count

    def rate(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return round(n / ((time.perf_counter() - t) / reps) / 1e9, 1)

    def both():
        with torch.cuda.stream(stream):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    def sm(dst, src):
        N_.check(N_.lib().segtaco_probe_copy(C.c_void_p(dst.data_ptr()), C.c_void_p(src.data_ptr()),
                                             n, C.c_void_p(desc.data_ptr()), sms * 4, None))
    out = {"ce_h2d_GBps": rate(lambda: d.copy_(h, non_blocking=True)),
           "ce_d2h_GBps": rate(lambda: h.copy_(d, non_blocking=True)),
           "ce_both_directions_GBps_each": rate(both),
           "sm_copy_h2d_GBps": rate(lambda: sm(d, h)),
           "sm_copy_d2h_GBps": rate(lambda: sm(h, d)),
           "bytes_per_copy": n}
    del h, h2, d, d2
    return out


def serving_stream(n_req, pool_size=1024, lam=20000.0, recent=8, p_repeat=0.8, seed=0):
    """Request stream of the serving workload: Poisson arrivals at `lam` per
    second, op SpMM or SDDMM 50/50, matrix id one of the `recent` most recently
    used ids with probability p_repeat, else a uniform draw from the pool."""
    import numpy as np
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1e6 / lam, size=n_req))
    is_spmm = rng.random(n_req) < 0.5
    ids, last = [], []
    for _ in range(n_req):
        if last and rng.random() < p_repeat:
            m = last[int(rng.integers(0, len(last)))]
        else:
            m = int(rng.integers(0, pool_size))
        ids.append(m)
        if m in last:
            last.remove(m)
        last.append(m)
        del last[:-recent]
    return arrivals, is_spmm, ids


_POOL_CACHE = {}  # pool matrices of a request stream, shared by the fp32 and bf16 runs


def served_err(args, N_, mats, ids, is_spmm, count=32):
    """Bound-normalised error against FP64 of served results: the stream's
    first `count` requests (SpMM and SDDMM, device-resident fp32 operands),
    submitted at once to a fresh server so that they batch together."""
    import numpy as np
    import torch
    from segtaco_gb300 import synth
    from segtaco_gb300.serving import Server
    worst, keep = 0.0, []
    with Server(slots=args.serve_slots, max_batch=args.serve_max_batch) as srv:
        for m in sorted(set(ids[:count])):
            srv.add_matrix(m, mats[m][0], pin=True)
        tickets = []
        for k in range(count):
            A, n, _ = mats[ids[k]]
            X = torch.from_numpy(synth.dense(A.M if not is_spmm[k] else A.K, n, seed=90 + k)).cuda()
            if is_spmm[k]:
                out = torch.empty((A.M, n), dtype=torch.float32, device="cuda")
                tickets.append(srv.spmm(ids[k], X, out, device=True))
                keep.append((k, X, None, out))
            else:
                Y = torch.from_numpy(synth.dense(A.K, n, seed=190 + k)).cuda()
                out = torch.empty(A.nnz, dtype=torch.float32, device="cuda")
                tickets.append(srv.sddmm(ids[k], X, Y, out, device=True))
                keep.append((k, X, Y, out))
        bad = sum(1 for t in tickets if srv.wait(t, -1) != N_.OK)
        if bad:
            return float("inf")
    for k, X, Y, out in keep:
        A = mats[ids[k]][0]
        if Y is None:
            worst = max(worst, rows_err(A, X.cpu().numpy(), out, sample_rows(A, 1024)))
        else:
            worst = max(worst, sddmm_err(A, X, Y, out, 4, n=50_000))
    return worst


def run_serving(args, N_, n_req=2000, bf16=False, device=False):
    """Served SpMM/SDDMM stream through segtaco_server (continuous batching over
    a device CSR cache), against the same stream in per-call mode (one request
    per launch).  Dense operands come from pinned host memory and results go
    back to pinned host memory, so every request pays its copies; with
    device=True they are device-resident (SEGTACO_REQ_DEVICE_DENSE) and no
    request crosses the link."""
    import numpy as np
    import torch
    from segtaco_gb300 import synth
    from segtaco_gb300.serving import Server

    arrivals, is_spmm, ids = serving_stream(n_req)
    mats = _POOL_CACHE.setdefault(n_req, {m: synth.pool_matrix(m) for m in sorted(set(ids))})
    maxK = max(A.K for A, _, _ in mats.values())
    maxM = max(A.M for A, _, _ in mats.values())
    bank_t = torch.from_numpy(synth.dense(max(maxK, maxM), 128, seed=5).ravel()).pin_memory()
    if bf16:
        bank_t = torch.from_numpy(synth.to_bf16_bits(bank_t.numpy())).pin_memory()
    if device:  # the same operands resident on the device
        bank = bank_t.cuda()
        if bf16:
            bank = bank.view(torch.int16).view(torch.bfloat16)
        arena = torch.empty(1 << 30, dtype=torch.float32, device="cuda")  # 4 GB of results
    else:
        bank = bank_t.numpy()
        arena_t = torch.empty(1 << 30, dtype=torch.float32).pin_memory()  # 4 GB of results
        arena = arena_t.numpy()
    arena_cap = arena.numel() if device else arena.size
    keep, reqs, in_b, out_b, cursor = [], [], 0, 0, 0
    for k in range(n_req):
        A, n, _ = mats[ids[k]]
        if is_spmm[k]:
            B = bank[:A.K * n].reshape(A.K, n)
            size = A.M * n
        else:
            B = bank[:A.M * n].reshape(A.M, n)
            Y = bank[:A.K * n].reshape(A.K, n)
            size = A.nnz
        if cursor + size > arena_cap:
            cursor = 0
        out = arena[cursor:cursor + size]
        cursor += (size + 63) // 64 * 64
        if is_spmm[k]:
            reqs.append(Server.request(N_.OP_SPMM, ids[k], B, out.reshape(A.M, n), device=device))
            in_b += 0 if device else B.nbytes
        else:
            reqs.append(Server.request(N_.OP_SDDMM, ids[k], B, out, Y=Y, device=device))
            in_b += 0 if device else B.nbytes + Y.nbytes
        out_b += 0 if device else size * 4
    result = {"workload": "%d requests, Poisson arrivals at 20k/s, SpMM or SDDMM 50/50, matrix "
                          "ids from a 1024-matrix pool (%d distinct used; recent-id repeats "
                          "p=0.8 over the last 8 ids), dense operands %s %s"
                          % (n_req, len(mats), "bf16" if bf16 else "fp32",
                             "resident on the device" if device else "from pinned host memory"),
              "h2d_bytes": in_b, "d2h_bytes": out_b}
    for mode, flags in (("batched", 0), ("per_call", N_.SERVER_PER_CALL)):
        with Server(flags=flags, slots=1 if flags else args.serve_slots,
                    max_batch=args.serve_max_batch) as srv:
            for m, (A, _, _) in mats.items():
                srv.add_matrix(m, A, pin=True)
            srv.wait(srv.replay(reqs, arrivals)[-1], -1)  # cold pass: fills the cache
            srv.drain(-1)
            srv.stats(reset=True)
            tickets = srv.replay(reqs, arrivals)
            srv.drain(-1)
            st = srv.stats(reset=True)
            bad = sum(1 for t in tickets if srv.wait(t, 0) != N_.OK)
            # capacity: the same requests all arriving at once
            burst = srv.replay(reqs, np.zeros(len(reqs)))
            srv.drain(-1)
            sb = srv.stats()
            bad += sum(1 for t in burst if srv.wait(t, 0) != N_.OK)
        result[mode] = {"requests_per_s": round(st["completed"] / st["span_s"], 1),
                        "p50_us": round(st["p50_us"], 1), "p99_us": round(st["p99_us"], 1),
                        "max_us": round(st["max_us"], 1), "mean_batch": round(st["mean_batch"], 2),
                        "batches": st["batches"], "span_ms": round(st["span_s"] * 1e3, 2),
                        "burst_requests_per_s": round(sb["completed"] / sb["span_s"], 1),
                        "failed": bad}
    if device and not bf16:
        result["max_err_vs_fp64"] = served_err(args, N_, mats, ids, is_spmm)
        result["err_sample"] = ("the first 32 requests of the stream, submitted together to a "
                                "fresh server (batched in the mix), each to its own output")
    result["throughput_vs_per_call"] = round(result["batched"]["requests_per_s"] /
                                             result["per_call"]["requests_per_s"], 3)
    result["p99_vs_per_call"] = round(result["per_call"]["p99_us"] /
                                      max(result["batched"]["p99_us"], 1e-9), 3)
    result["capacity_vs_per_call"] = round(result["batched"]["burst_requests_per_s"] /
                                           result["per_call"]["burst_requests_per_s"], 3)
    return result


def launches_per_step(eb, ws_need, plan):
    """Launches of one timed step (partition + product) for the plan named by
    segtaco_spmm_plan_name."""
    if eb:
        return 2
    if " pieces " in plan:
        return 3 if not plan.endswith(" parts=1") else 2
    return 3 if ws_need else 1


RESULT_KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
               "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
               "roofline", "gpu_launches", "e2e", "cpu_baseline", "clocks")


def result_line(detail):
    """The result line (printed last): the contract's keys and a compact
    summary, well inside a 3 KB tail; the gather and flop figures, the clock
    sample counts and the CPU baseline's one-thread sample live in the detail
    line."""
    line = {k: detail[k] for k in RESULT_KEYS}
    if isinstance(line["roofline"], dict):
        line["roofline"] = {k: v for k, v in line["roofline"].items()
                            if k not in ("gathered_bytes", "gather_GBps", "flops", "tflops")}
    if isinstance(line["clocks"], dict):
        line["clocks"] = {k: v for k, v in line["clocks"].items()
                          if k not in ("samples", "interval_ms", "nvml_samples")}
    if isinstance(line["cpu_baseline"], dict) and "one_thread" in line["cpu_baseline"]:
        line["cpu_baseline"] = dict(line["cpu_baseline"])
        line["cpu_baseline"]["one_thread"] = {
            "value": line["cpu_baseline"]["one_thread"].get("value")}
    line["summary"] = compact_summary(detail)
    return line


def compact_summary(d):
    """The headline's context in a few hundred bytes: per-schedule kernel ms,
    roofline fraction and error vs FP64; segTACO's own GPU kernels and
    cuSPARSE on the same operands; batched and served ratios; side ops."""
    def r(x, n=4):
        return None if x is None else round(x, n)
    out = {}
    if d.get("schedules"):
        out["schedules"] = {k: [v["kernel_ms"], v["roofline_frac"], float("%.2g" % v["max_err_vs_fp64"])]
                            for k, v in d["schedules"].items()}
        out["schedules_fields"] = ["kernel_ms", "frac", "err_vs_fp64"]
    v = d.get("power_law_10m")
    if v:
        out["power_law_10m_ms"] = {k: x["kernel_ms"] for k, x in v["schedules"].items()}
        out["power_law_10m_ms"]["spmv"] = v["spmv"]["ms"]
    rg = d.get("reference_gpu")
    if rg:
        if "unavailable" in rg:
            out["segtaco_gpu"] = rg["unavailable"]
        for w in ("power_law", "uniform16"):
            e = rg.get(w)
            if e and "segtaco" in e:
                out["segtaco_gpu_ms_vs_ours_" + w] = {
                    k: [e["segtaco"][k]["ms"], e["ours"][k]["ms"]] for k in e["segtaco"]}
                if w == "uniform16":
                    out["uniform16_max_err_vs_fp64"] = float("%.2g" % e.get("max_err_vs_fp64", 0))
            elif e:
                out["segtaco_gpu_" + w] = e
    if d.get("vendor") and "ms_per_step" in d["vendor"]:
        out["cusparse_ms"] = d["vendor"]["ms_per_step"]
    b = d.get("batched")
    if b:
        out["batched"] = {"speedup_vs_per_call_graph": b["speedup_vs_per_call"],
                          "per_call_graph_ms": b["per_call_graph_ms"],
                          "batched_graph_ms": b["batched_graph_ms"],
                          "max_err_vs_fp64": float("%.2g" % b["max_err_vs_fp64"])}
    sv = d.get("served")
    if sv:
        def one(x):
            return [round(x["batched"]["requests_per_s"]), round(x["per_call"]["requests_per_s"]),
                    round(x["batched"]["p50_us"]), round(x["batched"]["p99_us"]),
                    round(x["per_call"]["p99_us"]), round(x["capacity_vs_per_call"], 2)]
        out["served_fields"] = ["rps", "per_call_rps", "p50_us", "p99_us", "per_call_p99_us",
                                "capacity_x"]
        out["served"] = {"fp32_host": one(sv)}
        for k, n in (("bf16_operands", "bf16_host"), ("device_operands", "fp32_device")):
            if sv.get(k):
                out["served"][n] = one(sv[k])
                if "max_err_vs_fp64" in sv[k]:
                    out["served_max_err_vs_fp64"] = float("%.2g" % sv[k]["max_err_vs_fp64"])
    so = d.get("side_ops")
    if so:
        out["side_ops"] = {}
        for k, x in so.items():
            if isinstance(x, dict) and "ms" in x:
                err = x.get("max_err_vs_fp64", x.get("max_err_vs_fp64_bf16_values"))
                out["side_ops"][k] = [x["ms"], x["roofline_frac"]] + (
                    [float("%.2g" % err)] if err is not None else [])
        out["side_ops_fields"] = ["ms", "frac", "err_vs_fp64"]
    return out


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    from segtaco_gb300 import native as N_
    from segtaco_gb300 import ops, taco

    torch.cuda.set_device(local)
    A, B, N, desc = make_workload(args.workload)
    byts = algorithmic_bytes(A.M, A.K, A.nnz, N)
    Ad = ops.DeviceCSR.from_host(A, "cuda")
    Bd = torch.from_numpy(B).cuda()
    Cd = torch.empty((A.M, N), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    peak, peak_kind = peak_hbm()

    max_len = int(A.row_lengths().max())

    def tuned(schedule):
        """The library's choice for this shape (schedule -1 = let it pick), from
        the row and band statistics of the matrix on the device."""
        return ops.autotune(Ad, N, N_.F32, schedule=schedule, max_row_len=max_len)

    cfg = tuned(N_.AUTO if args.schedule == "auto" else N_.SCHEDULES[args.schedule])
    if args.col_tile:
        cfg.col_tile = args.col_tile
    if args.items:
        cfg.items_per_unit = args.items
    if args.l2_hints:
        cfg.flags |= N_.FLAG_L2_HINTS
    if args.row_walk:
        cfg.flags |= N_.FLAG_ROW_WALK
    if args.flat_walk:
        cfg.flags |= N_.FLAG_FLAT_WALK
    if args.depth:
        cfg.depth = args.depth
    if args.vec:
        cfg.vec = args.vec
    ws_need = ops.spmm_workspace_size(Ad, N, N_.F32, cfg)
    ws_bytes = max(256, ws_need)
    plan = ops.plan_name(Ad, Bd, cfg)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")

    # per-schedule sweep (context for the headline; same workload)
    schedules = {}
    err_rows = sample_rows(A, 4096)  # 4,096 random rows and the 16 longest
    if args.all_schedules:
        for s in ("rb_sr", "rb_pr", "eb_sr", "eb_pr"):
            c = tuned(N_.SCHEDULES[s])
            c.flags |= cfg.flags & (N_.FLAG_L2_HINTS | N_.FLAG_ROW_WALK | N_.FLAG_FLAT_WALK)
            wsz = max(256, ops.spmm_workspace_size(Ad, N, N_.F32, c))
            w = torch.empty(wsz, dtype=torch.uint8, device="cuda")
            st, kt = time_spmm(ops, N_, Ad, Bd, Cd, c, w, stream, max(3, args.steps // 2), 2)
            torch.cuda.synchronize()
            schedules[s] = {"config": {k: v for k, v in c.as_dict().items() if v},
                            "ms_per_step": round(st, 4), "kernel_ms": round(kt, 4),
                            "GBps": round(byts / st / 1e6, 1),
                            "roofline_frac": round(byts / kt / 1e6 / peak, 4),
                            "max_err_vs_fp64": rows_err(A, B, Cd, err_rows)}
            del w

    # the same configuration at the exponent that gives ~10M nonzeros
    variant = None
    if args.all_schedules and args.workload == "power_law" and not args.no_side_ops:
        variant = run_power_law_variant(args, N_, ops, stream, Bd, Cd, peak)

    # cuSPARSE CSR_ALG2 on the same resident operands (segTACO's vendor comparator)
    vendor = None
    if not args.no_vendor:
        try:
            for _ in range(2):
                ops.vendor_spmm(Ad, Bd, Cd, stream=stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            nv = max(3, args.steps // 2)
            e0.record(stream)
            for _ in range(nv):
                ops.vendor_spmm(Ad, Bd, Cd, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            vms = e0.elapsed_time(e1) / nv
            vendor = {"library": "cuSPARSE CSR_ALG2 (row-major)", "ms_per_step": round(vms, 4),
                      "GBps": round(byts / vms / 1e6, 1),
                      "note": "includes per-call handle/descriptor setup"}
        except Exception as exc:  # the comparator is context, not the product
            vendor = {"error": str(exc)[:200]}

    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    step_ms, kern_ms = time_spmm(ops, N_, Ad, Bd, Cd, cfg, ws, stream, args.steps, args.warmup)
    barrier(world)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    step_ms = reduce_max(step_ms, world)
    kern_ms = reduce_max(kern_ms, world)
    value = world * byts / step_ms / 1e6  # GB/s over all ranks
    achieved = byts / kern_ms / 1e6
    eb = cfg.schedule in (N_.EB_SR, N_.EB_PR)
    kernel_name = {N_.RB_SR: "spmm_rb_sr_kernel", N_.RB_PR: "spmm_rb_pr_kernel",
                   N_.EB_SR: "spmm_eb_sr_kernel", N_.EB_PR: "spmm_eb_pr_kernel"}[cfg.schedule]
    traffic = committed_traffic(args.workload, kernel_name)

    # e2e through the drop-in surface with pinned host operands
    e2e = None
    if not args.no_e2e:
        name = {N_.RB_SR: "spmm_rb_sr", N_.RB_PR: "spmm_rb_pr", N_.EB_SR: "spmm_eb_sr",
                N_.EB_PR: "spmm_eb_pr"}[cfg.schedule]

        def pinned(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            return t, t.numpy()
        keep = [pinned(x) for x in (A.row_ptr, A.col, A.val, B)]
        Ch_t = torch.empty((A.M, N), dtype=torch.float32).pin_memory()
        Ch = Ch_t.numpy()
        tA, hA = taco.csr(keep[0][1], keep[1][1], keep[2][1], A.M, A.K)
        tB, hB = taco.dense(keep[3][1])
        tC, hC = taco.dense(Ch)
        for _ in range(2):
            taco.call(name, tC, tA, tB)
        torch.cuda.synchronize()
        n_e2e = max(3, min(args.steps, 10))
        barrier(world)
        # each drop-in call returns with C on the host: time them one by one
        # and take the median (one slow call of the host link does not move it)
        call_s = []
        for _ in range(n_e2e):
            t0 = time.perf_counter()
            taco.call(name, tC, tA, tB)
            call_s.append(time.perf_counter() - t0)
        t_e2e = reduce_max(statistics.median(call_s), world)
        t_e2e_mean = reduce_max(sum(call_s) / len(call_s), world)
        N_.lib().segtaco_taco_release()
        h2d = (A.M + 1) * 4 + A.nnz * 8 + A.K * N * 4
        e2e = {"value": round(world * byts / t_e2e / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": A.M * N * 4,
               "ms_per_step": round(t_e2e * 1e3, 3), "entry_point": name,
               "statistic": "median of %d calls (mean %.3f ms)" % (n_e2e, t_e2e_mean * 1e3)}

    batched = None
    if not args.no_batched:
        batched = run_batched(args, N_, ops, stream, count=args.batch_count)
    served = None
    if not args.no_serving:
        served = run_serving(args, N_)
        served["bf16_operands"] = run_serving(args, N_, bf16=True)
        served["device_operands"] = run_serving(args, N_, device=True)
    side = None
    if not args.no_side_ops:
        side = run_side_ops(args, N_, ops, stream, Ad, peak, A)
    ceiling = link = None
    if not args.no_probe:
        ceiling = run_gather_ceiling(ops, stream)
        link = run_link_probe(stream)
    ref_gpu = None
    if not args.no_ref_gpu and args.workload == "power_law":
        ref_gpu = run_reference_gpu(args, N_, ops, stream, peak, A, B)

    cpu = None  # the CPU baseline runs at N = 1 only (rank 0 of a single rank)
    if rank == 0 and world == 1 and not args.no_cpu:
        # about 10 s of host time: the full product repeated, median taken
        t1, _, _, _ = cpu_spmm_timed(A, B, 1)
        reps = int(min(60, max(2, round(10.0 / max(t1, 1e-3)))))
        sec, Ms, nnzs, threads = cpu_spmm_timed(A, B, reps)
        # one thread on the first rows (about 3 s), scaled by the nonzeros it covers
        frac1 = min(1.0, max(0.01, 3.0 / max(t1 * threads, 1e-3)))
        sec1, M1, nnz1, _ = cpu_spmm_timed(A, B, 1, threads=1, frac=frac1)
        cpu = {"value": round(byts * (nnzs / A.nnz) / sec / 1e9, 3), "unit": UNIT,
               "cores": threads, "kind": "port", "cpu_model": cpu_model(),
               "sample": "full workload, median of %d runs after warm-up (%.3f s each, %.1f s "
                         "in all)" % (reps, sec, reps * sec),
               "one_thread": {"value": round(byts * (nnz1 / A.nnz) / sec1 / 1e9, 3),
                              "sample": "rows [0, %d) (%.1f%% of nonzeros), one run after "
                                        "warm-up" % (M1, 100.0 * nnz1 / A.nnz)},
               "build": cpu_baseline_build()}

    if rank == 0:
        detail = {
            "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy PCG64)",
            "config": {"workload": desc, "M": A.M, "K": A.K, "nnz": A.nnz, "N": N,
                       "schedule": {v: k for k, v in N_.SCHEDULES.items()}[cfg.schedule],
                       "col_tile": cfg.col_tile, "items_per_unit": cfg.items_per_unit,
                       "l2_hints": bool(cfg.flags & N_.FLAG_L2_HINTS),
                       "l2": "no flush: A %.0f MB, B %.0f MB, C %.0f MB each exceed the %.0f MB L2"
                             % (Ad.nbytes() / 1e6, B.nbytes / 1e6, A.M * N * 4 / 1e6, L2_BYTES / 1e6),
                       "parallelism": "replicas x%d" % world},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "kernel": kernel_name,
                         "gathered_bytes": A.nnz * N * 4,
                         "gather_GBps": round(A.nnz * N * 4 / kern_ms / 1e6, 1),
                         "flops": 2 * A.nnz * N,
                         "tflops": round(2 * A.nnz * N / kern_ms / 1e9, 3),
                         "kernel_ms": round(kern_ms, 4), "peak_source": peak_kind + " hbm_gbs",
                         # the DRAM bytes ncu measured per launch over the live kernel time:
                         # how close the kernel runs to HBM for the traffic it causes
                         "traffic_GBps": (round(traffic / kern_ms / 1e6, 1) if traffic else None),
                         "traffic_frac": (round(traffic / kern_ms / 1e6 / peak, 4)
                                          if traffic else None)},
            # per step: eb = merge path + product; rb_sr's long rows = the list
            # + long-row CTAs + row-block kernel; rb_pr's pieces = the list +
            # the row-block kernel (+ the pieces' passes with k_parts > 1);
            # rb = product
            "gpu_launches": args.steps * launches_per_step(eb, ws_need, plan),
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks, "schedules": schedules,
            "power_law_10m": variant,
            "vendor": vendor, "batched": batched, "served": served,
            "gather_ceiling": ceiling, "link": link, "side_ops": side,
            "reference_gpu": ref_gpu,
        }
        # Everything measured, on one line that is not the result line ...
        print("# detail " + json.dumps(detail), flush=True)
        # ... then the result line last and compact, so that a reader of the
        # last few KB of output sees it whole.
        print(json.dumps(result_line(detail), separators=(",", ":")), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="power_law", choices=["power_law", "power_law_10m", "power_law_quarter", "uniform16",
                             "banded"])
    ap.add_argument("--schedule", default="auto", choices=["auto", "rb_sr", "rb_pr", "eb_sr", "eb_pr"])
    ap.add_argument("--col-tile", type=int, default=0)
    ap.add_argument("--items", type=int, default=0)
    ap.add_argument("--l2-hints", action="store_true")
    ap.add_argument("--row-walk", action="store_true")
    ap.add_argument("--flat-walk", action="store_true")
    ap.add_argument("--vec", type=int, default=0, choices=[0, 1, 2, 4, 8],
                    help="dense elements per lane per step (0: the planner's)")
    ap.add_argument("--depth", type=int, default=0, choices=[0, 4, 8],
                    help="row walk: 16-byte loads in flight per lane (0: the planner's)")
    ap.add_argument("--all-schedules", action="store_true", default=True)
    ap.add_argument("--no-all-schedules", dest="all_schedules", action="store_false")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-vendor", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-count", type=int, default=256,
                    help="batched: matrices of the pool (256: the benchmark's; fewer for profiling)")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-slots", type=int, default=4, help="serving: batches in flight")
    ap.add_argument("--serve-max-batch", type=int, default=64, help="serving: requests per batch")
    ap.add_argument("--no-probe", action="store_true")
    ap.add_argument("--no-side-ops", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip timing segTACO's own GPU kernels (baseline/ref_gpu.py)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
