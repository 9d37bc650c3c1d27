"""The barrier protocol of the warp-specialised row pass (k_row_ws in
csrc/ocean_kernels.cu), replayed on the CPU under many warp schedules.

Every wait of a CTA has to end; a named barrier that never completes hangs the
GPU.  Each warp's sequence of `bar.sync` / `bar.arrive` (id, thread count) is
written out here as the kernel issues it, for the job counts and sample counts
a CTA can get. A scheduler then runs the warps in random orders and checks
four things:
  - every warp finishes (no deadlock);
  - no warp arrives twice in one generation of a barrier (an early arrival for
    a later job would complete the wrong generation on the hardware);
  - all participants of a generation give the same thread count;
  - no generation is left half-arrived when the CTA exits.
The copy-wait time-outs do not change the sequence: after a time-out the
kernel skips copies, never barriers.
"""
import random

import pytest

LINE_FOR = {512: (16, 16, 2), 1024: (16, 16, 4), 2048: (16, 16, 8)}   # LineFor<N> (R1, R2, R3)
BAR_SYNC0, BAR_FULL, BAR_EMPTY, BAR_PRE, BAR_TW = 0, 4, 6, 8, 9       # RowWsCfg; lines use 1..3


def row_ws_warps(N, n_jobs, nsmp, tail_sync=False, sets=2, radices=None):
    """Per-warp barrier sequences of one k_row_ws CTA with n_jobs jobs (items x
    samples, nsmp samples per item).  tail_sync: line_fft ends on a line
    barrier (the other callers of line_fft) or not (k_row_ws).  sets: line
    buffer sets (RowWsCfg::SETS; 1 for the 32 x 32 lines at three CTAs per
    SM).  radices: the line decomposition (default LineFor<N>)."""
    R1, R2, R3 = radices or LINE_FOR[N]
    G = N // R1
    fft_threads = 3 * G
    pre_threads = 256 if N >= 2048 else 128
    threads = fft_threads + pre_threads
    prologue = [("sync", BAR_SYNC0, threads)] * 3     # set-up, rows in, job 0's inputs complete
    # line_fft: stockham pass 1 (write, sync, read, sync) and, with R3 > 1, pass 2
    # (write, sync, read, [sync]); the final read's barrier only with tail_sync
    def line_ops(li):
        ops = [("sync", 1 + li, G)]                   # line_sync after loading the inputs
        ops += [("sync", 1 + li, G)]
        if R3 > 1 or tail_sync:
            ops += [("sync", 1 + li, G)]
        if R3 > 1:
            ops += [("sync", 1 + li, G)]
            if tail_sync:
                ops += [("sync", 1 + li, G)]
        return ops
    warps = []
    for w in range(fft_threads // 32):
        li = (w * 32) // G
        ops = list(prologue) + [("sync", BAR_TW, fft_threads)]
        for j in range(n_jobs):
            b = j % sets
            if j > 0:
                ops.append(("sync", BAR_FULL + b, threads))
            ops += line_ops(li)
            ops.append(("arrive", BAR_EMPTY + b, threads))
        warps.append(ops)
    for w in range(pre_threads // 32):
        ops = list(prologue)
        for j in range(1, n_jobs):
            b, smp = j % sets, j % nsmp
            if smp == 0:
                ops.append(("sync", BAR_PRE, pre_threads))       # the item's rows are in
            if j >= sets:
                ops.append(("sync", BAR_EMPTY + b, threads))     # set b's previous job is transformed
            ops.append(("arrive", BAR_FULL + b, threads))
            if smp == nsmp - 1:
                ops.append(("sync", BAR_PRE, pre_threads))       # done with the stage: refill it
        for j in range(max(n_jobs - sets, 0), n_jobs):           # the transform side's last arrivals
            ops.append(("sync", BAR_EMPTY + j % sets, threads))
        warps.append(ops)
    return warps


class ProtocolError(AssertionError):
    pass


def run(warps, seed):
    """Execute the sequences in a random interleaving; raise ProtocolError on
    a deadlock, a double arrival, a count mismatch or a half-arrived barrier."""
    rng = random.Random(seed)
    pc = [0] * len(warps)
    blocked = [False] * len(warps)
    gens = {}
    while True:
        ready = [w for w in range(len(warps)) if pc[w] < len(warps[w]) and not blocked[w]]
        if not ready:
            if any(pc[w] < len(warps[w]) for w in range(len(warps))):
                raise ProtocolError(f"deadlock: warps {[w for w in range(len(warps)) if blocked[w]]} wait")
            break
        w = rng.choice(ready)
        kind, bid, count = warps[w][pc[w]]
        g = gens.setdefault(bid, {"count": count, "arrived": 0, "who": set(), "waiting": []})
        if g["count"] != count:
            raise ProtocolError(f"barrier {bid}: thread count {count} against {g['count']}")
        if w in g["who"]:
            raise ProtocolError(f"barrier {bid}: warp {w} arrives twice in one generation")
        g["who"].add(w)
        g["arrived"] += 32
        pc[w] += 1
        if kind == "sync":
            blocked[w] = True
            g["waiting"].append(w)
        if g["arrived"] > count:
            raise ProtocolError(f"barrier {bid}: {g['arrived']} arrivals for {count}")
        if g["arrived"] == count:
            for x in g["waiting"]:
                blocked[x] = False
            del gens[bid]
    if gens:
        raise ProtocolError(f"half-arrived barriers at exit: {sorted(gens)}")


@pytest.mark.parametrize("N", sorted(LINE_FOR))
@pytest.mark.parametrize("n_items,nsmp", [(1, 1), (2, 1), (3, 1), (7, 1), (1, 8), (2, 8), (3, 3)])
def test_row_ws_protocol_terminates(N, n_items, nsmp):
    warps = row_ws_warps(N, n_items * nsmp, nsmp)
    for seed in range(40):
        run(warps, seed)


@pytest.mark.parametrize("n_items,nsmp", [(1, 1), (2, 1), (3, 1), (7, 1), (2, 8), (3, 3)])
def test_one_set_32x32_protocol_terminates(n_items, nsmp):
    """row_variant 5: 32 x 32 lines (one warp each), one line-buffer set."""
    warps = row_ws_warps(1024, n_items * nsmp, nsmp, sets=1, radices=(32, 32, 1))
    for seed in range(40):
        run(warps, seed)


def test_tail_sync_variant_terminates():
    """line_fft with its final line barrier (the default for the other kernels)."""
    for seed in range(20):
        run(row_ws_warps(1024, 4, 1, tail_sync=True), seed)


def test_checker_finds_a_missing_empty_wait():
    """Planted mistake: the prepass does not wait on EMPTY before refilling a
    set.  The transform warps' arrivals for jobs j and j+2 then meet in one
    generation, which the checker reports."""
    warps = row_ws_warps(1024, 6, 1)
    broken = [[op for op in ops if not (op[0] == "sync" and op[1] in (BAR_EMPTY, BAR_EMPTY + 1))]
              if i >= 3 * 64 // 32 else ops for i, ops in enumerate(warps)]
    with pytest.raises(ProtocolError):
        for seed in range(40):
            run(broken, seed)


def test_checker_finds_a_missing_final_wait():
    """Planted mistake: the prepass leaves without consuming the last two
    EMPTY arrivals; those generations stay half-arrived."""
    warps = row_ws_warps(1024, 3, 1)
    n_fft = 3 * 64 // 32
    broken = [ops if i < n_fft else ops[:-2] for i, ops in enumerate(warps)]
    with pytest.raises(ProtocolError):
        run(broken, 0)
