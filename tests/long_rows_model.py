"""A CPU restatement of the long-row CTA schedule of
segtaco_gb300/csrc/spmm_long.cu, used by test_long_rows_model_cpu.py to check
its index arithmetic without a GPU: which thread copies which 16-byte chunk of
which B row into which ring slot, which slots each stage and the final fold
use, the order of copies, waits and barriers, and the work list (front part:
rows of >= 8 * threshold nonzeros; back part: the other long rows).

The constants are read from the CUDA source, so the model follows it."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "segtaco_gb300", "csrc", "spmm_long.cu")


def constants():
    text = open(SRC).read()
    out = {}
    for name in ("kLongCta", "kLongStage", "kLongRing"):
        m = re.search(r"constexpr int %s = (\d+);" % name, text)
        assert m, name
        out[name] = int(m.group(1))
    return out


def long_list_caps(nnz, T):
    """Capacities of the two list parts (internal.h long_list_caps)."""
    return nnz // (8 * T) + 1, nnz // T + 1


def list_rows(lengths, T, nnz):
    """The rows the list kernel appends: (front part, back part, caps)."""
    hi_cap, lo_cap = long_list_caps(nnz, T)
    front = [r for r, n in enumerate(lengths) if n >= 8 * T]
    back = [r for r, n in enumerate(lengths) if T <= n < 8 * T]
    return front, back, hi_cap, lo_cap


def items(front, back, hi_cap, slabs):
    """(row, slab) of every queue item, in queue order, and the list slot read."""
    n_hi, n_lo = len(front), len(back)
    lst = {}
    for i, r in enumerate(front):
        lst[i] = r
    for i, r in enumerate(back):
        lst[hi_cap + i] = r
    out = []
    for item in range((n_hi + n_lo) * slabs):
        if item < n_hi * slabs:  # front part: row by row, every slab of a row
            li, slab = divmod(item, slabs)
        else:  # back part: slab by slab
            slab, lo = divmod(item - n_hi * slabs, n_lo)
            li = n_hi + lo
        idx = li if li < n_hi else hi_cap + (li - n_hi)
        out.append((lst[idx], slab, idx))
    return out


def copies(W, esz, N, col0, cnt, C):
    """(row in stage, chunk) pairs the CTA copies for a stage of `cnt` nonzeros."""
    EPC = 16 // esz
    CH = W // EPC
    RP = C["kLongCta"] // CH
    RPT = C["kLongStage"] // RP
    done = []
    for t in range(C["kLongCta"]):
        c, rr = t % CH, t // CH
        for i in range(RPT):
            row = rr + RP * i
            if row < cnt and col0 + c * EPC < N:
                done.append((row, c))
    return done, EPC


def reads(W, esz, cnt, pr, C):
    """(row in stage, column in slab) pairs the threads read from the ring."""
    out = []
    if not pr:
        for t in range(min(W, C["kLongCta"])):
            for i in range(cnt):
                out.append((i, t))
    else:
        CPL = W // 32
        RW = C["kLongStage"] // 4
        for warp in range(4):
            for lane in range(32):
                for i in range(warp * RW, min(warp * RW + RW, cnt)):
                    for u in range(CPL):
                        out.append((i, lane * CPL + u))
    return out


def pipeline_events(nst, C):
    """Program order of one item: ('issue', stage, slot), ('commit', group),
    ('wait', groups allowed pending), ('sync',), ('consume', stage, slot)."""
    NS = C["kLongRing"]
    ev = []
    g = 0
    for st in range(NS - 1):
        if st < nst:
            ev.append(("issue", st, st % NS))
        ev.append(("commit", g))
        g += 1
    for st in range(nst):
        ev.append(("wait", NS - 2))
        ev.append(("sync",))
        sn = st + NS - 1
        if sn < nst:
            ev.append(("issue", sn, sn % NS))
        ev.append(("commit", g))
        g += 1
        ev.append(("consume", st, st % NS))
    return ev


def check_pipeline(nst, C):
    """Replays pipeline_events: every consumed stage sits in its slot and its
    copy group has completed before the barrier that precedes the read; a
    slot is rewritten only after a barrier that follows its last read."""
    NS = C["kLongRing"]
    slot_stage = {}
    issued_group = {}      # stage -> commit group that carries its copies
    pending_stages = []    # stages issued but not yet in a committed group
    committed = 0
    completed_upto = -1    # groups 0 .. completed_upto have landed
    last_read = {}         # slot -> event index of its last consume
    last_sync = -1
    for k, e in enumerate(pipeline_events(nst, C)):
        if e[0] == "issue":
            _, st, slot = e
            if slot in last_read:
                assert last_sync > last_read[slot], ("slot rewritten before a barrier", st)
            slot_stage[slot] = st
            pending_stages.append(st)
        elif e[0] == "commit":
            for st in pending_stages:
                issued_group[st] = e[1]
            pending_stages = []
            committed = e[1] + 1
        elif e[0] == "wait":
            completed_upto = max(completed_upto, committed - 1 - e[1])
        elif e[0] == "sync":
            last_sync = k
        elif e[0] == "consume":
            _, st, slot = e
            assert slot_stage.get(slot) == st, ("stage not in its slot", st)
            assert issued_group[st] <= completed_upto, ("stage read before it landed", st)
            last_read[slot] = k
    return True
