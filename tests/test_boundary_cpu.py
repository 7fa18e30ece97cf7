"""The C-ABI library: loads, exports every symbol include/*.h declares, and
validates arguments on the host (no device work happens in these tests)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from segtaco_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _header(name):
    with open(os.path.join(INCLUDE, name)) as f:
        return f.read()


def c_abi_names():
    names = set()
    for h in ("segtaco.h", "segtaco_taco.h"):
        txt = re.sub(r"/\*.*?\*/", "", _header(h), flags=re.S)
        names |= set(re.findall(r"\b(segtaco_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def cxx_names():
    txt = _header("segtaco_taco.h")
    spmm = re.findall(r"^SEGTACO_SPMM_DECL\((\w+)\)", txt, flags=re.M)
    side = ["spmv_csr_gpu_taco", "sddmm_csr_gpu_taco", "sddmm_csr_gpu_warp", "spmspv_csr_gpu_taco",
            "get_gpu_timer_result"]
    return spmm, side


def test_library_loads(native_lib):
    assert N.version().startswith("segtaco-gb300")


@pytest.mark.parametrize("name", c_abi_names())
def test_c_symbol_exported(native_lib, name):
    assert hasattr(native_lib, name), name
    assert name in N.SIGNATURES, "ctypes signature missing for " + name


def test_cxx_dropin_symbols_exported(native_lib):
    spmm, side = cxx_names()
    # gpu_kernels.cuh:11-93 declares 79 SpMM names; two more are defined there.
    assert len(spmm) == 81
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", N.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(\w+)\(taco_tensor_t\*", out))
    exported |= set(re.findall(r"\b(get_gpu_timer_result)\(\)", out))
    for name in spmm + side:
        assert name in exported, name
    # and the names are the C++ (mangled) ones a segTACO driver links against
    raw = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    assert "_Z10spmm_rb_srP13taco_tensor_tS0_S0_" in raw
    assert "_Z20get_gpu_timer_resultv" in raw


def test_taco_name_table_covers_every_declared_name(native_lib):
    spmm, side = cxx_names()
    table = N.taco_names()
    assert set(spmm) | set(side[:4]) == set(table)


def test_struct_layouts_match_the_c_headers(tmp_path):
    """ctypes mirrors of segtaco_config and taco_tensor_t have the C layout."""
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stddef.h>
#include <stdio.h>
#include "segtaco.h"
#include "segtaco_taco.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\\n", sizeof(segtaco_config), sizeof(struct taco_tensor_t),
         offsetof(struct taco_tensor_t, indices), offsetof(struct taco_tensor_t, vals),
         offsetof(struct taco_tensor_t, vals_size));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [C.sizeof(N.Config), C.sizeof(N.TacoTensor), N.TacoTensor.indices.offset,
                   N.TacoTensor.vals.offset, N.TacoTensor.vals_size.offset]


def test_argument_errors_without_device(native_lib):
    L = native_lib
    # negative sizes are rejected before any CUDA call
    st = L.segtaco_spmm(-1, 4, 0, None, None, None, None, N.F32, 4, None, 4, 4, None, None, 0, None)
    assert st == N.EINVAL and "negative" in N.last_error()
    # empty problem: nothing to do, success
    assert L.segtaco_spmm(0, 4, 0, None, None, None, None, N.F32, 4, None, 4, 4, None, None, 0,
                          None) == N.OK
    st = L.segtaco_spmm(4, 4, 3, C.c_void_p(16), None, None, None, N.F32, 4, None, 4, 4, None,
                        None, 0, None)
    assert st == N.EINVAL and "col is NULL" in N.last_error()
    st = L.segtaco_spmm(4, 4, 0, C.c_void_p(16), C.c_void_p(16), None, C.c_void_p(16), 7, 4,
                        C.c_void_p(16), 4, 4, None, None, 0, None)
    assert st == N.EINVAL and "dtype" in N.last_error()
    st = L.segtaco_spmm(4, 4, 0, C.c_void_p(16), C.c_void_p(16), None, C.c_void_p(16), N.F32, 2,
                        C.c_void_p(16), 4, 4, None, None, 0, None)
    assert st == N.EINVAL and "ldb" in N.last_error()
    bad = N.Config.make(schedule=9)
    st = L.segtaco_spmm(4, 4, 0, C.c_void_p(256), C.c_void_p(256), None, C.c_void_p(256), N.F32,
                        4, C.c_void_p(256), 4, 4, C.byref(bad), None, 0, None)
    assert st == N.EINVAL and "schedule" in N.last_error()
    both = N.Config.make(flags=N.FLAG_ROW_WALK | N.FLAG_FLAT_WALK)
    st = L.segtaco_spmm(4, 4, 0, C.c_void_p(256), C.c_void_p(256), None, C.c_void_p(256), N.F32,
                        4, C.c_void_p(256), 4, 4, C.byref(both), None, 0, None)
    assert st == N.EINVAL and "exclusive" in N.last_error()
    assert L.segtaco_taco_call(b"no_such_kernel", None, None, None, None) == N.EINVAL


def test_batch_argument_errors_without_device(native_lib):
    L = native_lib
    h = C.c_void_p()
    assert L.segtaco_batch_create(-1, None, None, None, C.byref(h)) == N.EINVAL
    assert L.segtaco_batch_create(1, None, None, None, C.byref(h)) == N.EINVAL
    probs = (N.SpmmProblem * 2)()
    probs[0].M, probs[0].K, probs[0].N, probs[0].nnz = 4, 4, 4, 0
    probs[0].row_ptr = probs[0].B = probs[0].C = 256
    probs[0].ldb = probs[0].ldc = 4
    probs[1] = probs[0]
    probs[1].ldc = 2  # ldc < N
    cfgs = (N.Config * 2)(N.Config.make(), N.Config.make())
    st = L.segtaco_batch_create(2, probs, cfgs, None, C.byref(h))
    assert st == N.EINVAL and "problem 1" in N.last_error() and not h.value
    probs[1].ldc, probs[1].b_dtype = 4, 5
    assert L.segtaco_batch_create(2, probs, cfgs, None, C.byref(h)) == N.EINVAL
    assert L.segtaco_batch_run(None, None) == N.EINVAL
    assert L.segtaco_batch_run_graph(None, None) == N.EINVAL
    assert L.segtaco_batch_info(None, None, None, None) == N.EINVAL
    assert L.segtaco_batch_destroy(None) == N.OK
    st = (C.c_int64 * 4)()
    assert L.segtaco_row_stats(-1, None, st, None) == N.EINVAL


def test_workspace_and_heuristic(native_lib):
    L = native_lib
    out = C.c_size_t()
    cfg = N.Config.make(schedule="eb_sr", items_per_unit=256)
    assert L.segtaco_spmm_workspace_size(1000, 1000, 20000, 128, N.F32, C.byref(cfg),
                                         C.byref(out)) == N.OK
    nch = (1000 + 20000 + 255) // 256
    assert out.value >= 2 * (nch + 1) * 4
    cfg = N.Config.make(schedule="rb_sr")
    assert L.segtaco_spmm_workspace_size(1000, 1000, 20000, 128, N.F32, C.byref(cfg),
                                         C.byref(out)) == N.OK
    assert out.value == 0
    # rb with LONG_ROWS from 1M nonzeros: the list of rows of >= items_per_unit
    # (2048) nonzeros in two parts (rows of >= 8 * 2048: at most nnz / 16384;
    # the others: at most nnz / 2048) and the counters; none without the flag
    # or when N is not a multiple of the 16-byte chunk
    def ws(n, **kw):
        c = N.Config.make(schedule="rb_sr", **kw)
        assert L.segtaco_spmm_workspace_size(10**6, 10**6, 2 * 10**7, n, N.F32, C.byref(c),
                                             C.byref(out)) == N.OK
        return out.value

    def want(T):
        entries = 2 * 10**7 // (8 * T) + 1 + 2 * 10**7 // T + 1
        return (entries * 4 + 255) // 256 * 256 + 256
    LR = N.FLAG_LONG_ROWS
    assert ws(128, flags=LR) == want(2048)
    assert ws(128, items_per_unit=512, flags=LR) == want(512)
    assert ws(128) == 0
    assert ws(126, flags=LR) == 0
    # rb_pr: pieces of 4096 nonzeros, at most 2 nnz / 4096 + 1 of rows of
    # several pieces (each with a counter per column slab and a partial row)
    # and nnz / T + 1 one-piece rows; W = 32 columns per slab here, 4 slabs
    multi = 2 * 2 * 10**7 // 4096 + 1
    cap = multi + 2 * 10**7 // 512 + 1  # default threshold for rb_pr: 512
    part = (2 * cap + 4 * multi + 63) // 64 * 64
    c = N.Config.make(schedule="rb_pr", flags=LR, k_parts=1)
    assert L.segtaco_spmm_workspace_size(10**6, 10**6, 2 * 10**7, 128, N.F32, C.byref(c),
                                         C.byref(out)) == N.OK
    assert out.value == ((part + multi * 128) * 4 + 255) // 256 * 256 + 256
    c = N.Config.make(schedule="rb_pr", flags=LR)  # one pass by default
    assert L.segtaco_spmm_workspace_size(10**6, 10**6, 2 * 10**7, 128, N.F32, C.byref(c),
                                         C.byref(out)) == N.OK
    assert out.value == ((part + multi * 128) * 4 + 255) // 256 * 256 + 256
    # two passes over B's rows: pieces of 2048, every entry with counters and
    # two partial rows
    multi = 2 * 2 * 10**7 // 2048 + 1
    cap = multi + 2 * 10**7 // 512 + 1
    part = (2 * cap + 4 * cap + 63) // 64 * 64
    c = N.Config.make(schedule="rb_pr", flags=LR, k_parts=2)
    assert L.segtaco_spmm_workspace_size(10**6, 10**6, 2 * 10**7, 128, N.F32, C.byref(c),
                                         C.byref(out)) == N.OK
    assert out.value == ((part + cap * 2 * 128) * 4 + 255) // 256 * 256 + 256
    name = C.create_string_buffer(256)
    for k, want_parts in ((0, 1), (2, 2), (9, 8)):
        c = N.Config.make(schedule="rb_pr", flags=LR, k_parts=k)
        assert L.segtaco_spmm_plan_name(10**6, 10**6, 2 * 10**7, 128, N.F32, None, 128,
                                        C.byref(c), name, 256) == N.OK
        assert name.value.decode().endswith(" parts=%d" % want_parts)
    c = N.Config.make(schedule="rb_pr", flags=LR, col_tile=32, vec=4)
    name = C.create_string_buffer(256)
    assert L.segtaco_spmm_plan_name(10**6, 10**6, 2 * 10**7, 128, N.F32, None, 128, C.byref(c),
                                    name, 256) == N.OK
    assert name.value.decode().startswith("rb_pr pieces ")
    h = N.Config()
    h.schedule = -1
    assert L.segtaco_autotune_heuristic(16384, 16384, 262144, 32, N.F32, 16, C.byref(h)) == N.OK
    assert h.schedule == N.RB_PR
    h.schedule = -1
    assert L.segtaco_autotune_heuristic(10**6, 10**6, 2 * 10**7, 128, N.F32, 48679,
                                        C.byref(h)) == N.OK
    assert h.schedule == N.EB_PR
    assert (h.col_tile, h.vec) == (32, 8)  # B beyond L2, skewed rows: 8 columns per lane
    assert h.flags == N.FLAG_L2_HINTS  # ... and the gathered B rows evict_last
    assert h.items_per_unit == 512
    h.schedule = -1
    assert L.segtaco_autotune_heuristic(262144, 262144, 19135456, 64, N.F32, 73,
                                        C.byref(h)) == N.OK
    assert h.schedule == N.RB_PR and h.vec == 8  # B beyond L2: 8 columns per lane
    h.schedule = -1
    assert L.segtaco_autotune_heuristic(20000, 20000, 240000, 64, N.F32, 30,
                                        C.byref(h)) == N.OK
    assert h.vec == 0  # B in L2: the planner's 16-byte lanes
    h.schedule = -1
    assert L.segtaco_autotune_heuristic(10**6, 10**6, 2 * 10**7, 128, N.BF16, 48679,
                                        C.byref(h)) == N.OK
    assert (h.col_tile, h.vec) == (64, 16)  # bf16 B beyond L2, skewed: 16 columns per lane
    for sched, tile, items, flags in ((N.RB_SR, 128, 2048, N.FLAG_LONG_ROWS),
                                      (N.EB_SR, 128, 512, 0)):
        h.schedule = sched  # sequential: 16-byte lanes; rb_sr: long rows from 2048
        assert L.segtaco_autotune_heuristic(10**6, 10**6, 2 * 10**7, 128, N.F32, 48679,
                                            C.byref(h)) == N.OK
        assert h.schedule == sched and h.col_tile == tile and h.vec == 0
        assert h.items_per_unit == items and h.flags == flags
    # rb_pr: long rows (pieces) from 512 nonzeros, then 64 short rows per warp
    # (32 while 64 would leave fewer than 8192 warps); rows known short or
    # unknown: none (unknown: not skewed, no L2 hints)
    H, LR = N.FLAG_L2_HINTS, N.FLAG_LONG_ROWS
    for m, max_len, flags, rows, items in ((10**6, 511, H, 4, 2048),
                                           (10**6, 512, LR | H, 64, 512),
                                           (10**6, 48679, LR | H, 64, 512),
                                           (10**6, -1, 0, 4, 2048),
                                           (300_000, 48679, LR | H, 32, 512)):
        h.schedule = N.RB_PR
        assert L.segtaco_autotune_heuristic(m, 10**6, m * 20, 128, N.F32, max_len,
                                            C.byref(h)) == N.OK
        assert (h.flags, h.rows_per_unit, h.items_per_unit) == (flags, rows, items), (m, max_len)
    h.schedule = N.RB_PR  # long rows under a mean of 73 nonzeros per row: 4 rows per warp
    assert L.segtaco_autotune_heuristic(262144, 262144, 19135456, 64, N.F32, 580,
                                        C.byref(h)) == N.OK
    assert h.flags == N.FLAG_LONG_ROWS and h.rows_per_unit == 4
    # small products: merge-path chunks shrink until the grid holds 4,096 of
    # them (16,384 rows + 262,144 nonzeros: 64 items); rb_sr 2 rows per warp
    for sched, items, rows in ((N.EB_PR, 64, 1), (N.EB_SR, 64, 1), (N.RB_SR, 2048, 2)):
        h.schedule = sched
        assert L.segtaco_autotune_heuristic(16384, 16384, 262144, 32, N.F32, 16,
                                            C.byref(h)) == N.OK
        assert (h.items_per_unit, h.rows_per_unit) == (items, rows), sched
    h.schedule = N.RB_SR  # bf16 too: 128-column slabs (8-byte lanes) from 1M nonzeros
    assert L.segtaco_autotune_heuristic(10**6, 10**6, 2 * 10**7, 128, N.BF16, 48679,
                                        C.byref(h)) == N.OK
    assert h.col_tile == 128
    for n, tile in ((32, 32), (16, 32), (64, 64), (33, 64), (100, 128)):
        for sched in (N.RB_SR, N.EB_SR):  # sequential: the narrowest lanes covering N
            h.schedule = sched
            assert L.segtaco_autotune_heuristic(16384, 16384, 262144, n, N.F32, 16,
                                                C.byref(h)) == N.OK
            assert h.col_tile == tile, (sched, n, h.col_tile)


def test_autotune_from_a_host_csr(native_lib):
    """ops.autotune on a host CSR: the longest row from its row_ptr."""
    from segtaco_gb300 import ops, synth
    A = synth.power_law(60_000, 50_000, 1.8, 40_000, 0.02, seed=35)  # 1.09M nonzeros
    assert A.nnz >= 10**6 and A.row_lengths().max() >= 2048
    c = ops.autotune(A, 128)
    assert c.schedule == N.EB_PR and c.flags == 0  # skewed: merge path
    c = ops.autotune(A, 128, schedule=N.RB_SR)
    assert c.schedule == N.RB_SR and c.flags == N.FLAG_LONG_ROWS and c.items_per_unit == 2048
    c = ops.autotune(A, 128, schedule=N.RB_PR, max_row_len=100)
    assert c.flags == 0  # rows known to be short: every row in the row-block kernel
    U = synth.uniform_rows(seed=0)
    assert ops.autotune(U, 32).schedule == N.RB_PR  # even rows: row-balanced


def test_flag_constants_match_the_header():
    """Every SEGTACO_FLAG_* of include/segtaco.h has the same value in native.py."""
    text = open(os.path.join(ROOT, "include", "segtaco.h")).read()
    flags = dict(re.findall(r"#define SEGTACO_(FLAG_[A-Z0-9_]+)\s+(\d+)u", text))
    assert len(flags) >= 7
    for name, value in flags.items():
        assert getattr(N, name) == int(value), name
    kernels = dict(re.findall(r"#define SEGTACO_(SDDMM_[A-Z]+)\s+(\d+)", text))
    assert set(kernels) == {"SDDMM_AUTO", "SDDMM_FIXED", "SDDMM_GENERAL", "SDDMM_BAND"}
    for name, value in kernels.items():
        assert getattr(N, name) == int(value), name


def test_sddmm_autotune_band(native_lib):
    """segtaco_sddmm_autotune keeps SEGTACO_SDDMM_BAND (rows near the diagonal)
    for D = 64 only; the Python autotuner sets it from the band statistics."""
    from segtaco_gb300 import ops, synth
    for D, dt, want in ((64, N.F32, N.SDDMM_BAND), (32, N.F32, N.SDDMM_AUTO),
                        (128, N.F32, N.SDDMM_AUTO), (64, N.BF16, N.SDDMM_BAND)):
        c = N.SddmmConfig.make(N.SDDMM_BAND)
        assert native_lib.segtaco_sddmm_autotune(262144, 262144, 19135456, D, dt, 73,
                                                 C.byref(c)) == N.OK
        assert c.kernel == want and c.block_nnz == 256
    assert ops.sddmm_autotune(synth.banded_plus_random(2000, 32, 8, seed=3), 64).kernel == \
        N.SDDMM_BAND
    assert ops.sddmm_autotune(synth.random_csr(2000, 2000, 0.01, seed=4), 64).kernel == \
        N.SDDMM_AUTO


def test_device_available_is_a_query(native_lib):
    # never raises; 0 on a host without a GPU, 1 on the GB300
    assert native_lib.segtaco_device_available() in (0, 1)


def test_window_plan(native_lib):
    """SEGTACO_FLAG_WINDOW plans rb_pr's band kernel where it applies (N >= 64
    and a multiple of 16, B and C 16-byte aligned, B's row pitch a multiple of
    16 bytes, ldc a multiple of 4, 32 + 2H <= 256 window rows), else the
    TMA-staged row-block kernel where that tensor copy is legal (window of at
    most 256 rows and 60 KB), and only for row-block schedules."""
    L = native_lib
    buf = C.create_string_buffer(256)

    def plan(n, dt, ldb, cfg, B=0x10000000):
        assert L.segtaco_spmm_plan_name(3000, 3000, 200000, n, dt, C.c_void_p(B), ldb,
                                        C.byref(cfg), buf, 256) == N.OK
        return buf.value.decode()
    mk = lambda sched, **k: N.Config.make(schedule=sched, flags=N.FLAG_WINDOW,
                                          rows_per_unit=k.get("rpu", 16),
                                          items_per_unit=k.get("halo", 32),
                                          col_tile=k.get("tile", 64), vec=k.get("vec", 8))
    assert " band " in plan(64, N.F32, 64, mk(N.RB_PR))
    assert " band " in plan(128, N.BF16, 128, mk(N.RB_PR, vec=16))
    assert " band " in plan(80, N.F32, 80, mk(N.RB_PR))
    assert " band " in plan(64, N.F32, 64, mk(N.RB_PR, halo=112))       # 256 window rows
    assert " band " not in plan(64, N.F32, 64, mk(N.RB_PR, halo=113))   # 258
    assert " window V=8 G=4 " in plan(48, N.F32, 48, mk(N.RB_PR, tile=48))  # N < 64: window
    assert " window V=2 G=32 " in plan(64, N.F32, 64, mk(N.RB_SR, vec=0))   # rb_sr: window
    assert " window V=16 G=4 " in plan(48, N.BF16, 48, mk(N.RB_PR, vec=16))
    for name in (plan(64, N.F32, 64, mk(N.EB_PR)),                      # rb only
                 plan(64, N.F32, 66, mk(N.RB_PR, vec=2)),               # pitch 264 B
                 plan(64, N.F32, 64, mk(N.RB_PR), B=0x10000008)):       # 8-byte aligned
        assert " window " not in name and " band " not in name, name
    assert " window " not in plan(48, N.F32, 48, mk(N.RB_PR, rpu=32, halo=96, tile=48))  # 320 rows
    # the heuristic reads the bit as band statistics: rb_pr keeps it (the band
    # kernel, halo 32); without it a B that fits L2 under a large product gets
    # one 64-column slab of 8-column lanes
    for flags, want in ((N.FLAG_WINDOW, N.FLAG_WINDOW), (0, 0)):
        h = N.Config.make(schedule=N.AUTO, flags=flags)
        assert L.segtaco_autotune_heuristic(262144, 262144, 19135456, 64, N.F32, 73,
                                            C.byref(h)) == N.OK
        assert (h.schedule, h.flags, h.col_tile, h.vec) == (N.RB_PR, want, 64, 8)
    h = N.Config.make(schedule=N.RB_SR, flags=N.FLAG_WINDOW)  # rb_sr: not chosen
    assert L.segtaco_autotune_heuristic(262144, 262144, 19135456, 64, N.F32, 73,
                                        C.byref(h)) == N.OK
    assert not h.flags & N.FLAG_WINDOW
    h = N.Config.make(schedule=N.AUTO)  # B of 512 MB: 32-column slabs
    assert L.segtaco_autotune_heuristic(10**6, 10**6, 2 * 10**7, 128, N.F32, 48679,
                                        C.byref(h)) == N.OK
    assert h.col_tile == 32


def test_band_fraction_host():
    from segtaco_gb300 import ops, synth
    A = synth.banded_plus_random(2000, 32, 8, seed=3)
    f = ops.in_band_fraction_host(A, 32)
    assert abs(f - 65.0 / 73.0) < 0.01
    P = synth.power_law(3000, 3000, 1.8, 1000, 0.02, seed=4)
    assert ops.in_band_fraction_host(P, 32) < 0.1
