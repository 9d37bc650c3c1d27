"""Autotuner of the per-N launch configuration (ocean_tuning in include/ocean.h).

Run on a GB300 (it times kernels):

    python fft-ocean-waves_gb300/tune.py [--out DIR] [--sizes 512,1024] [--reps 5]

For every N it times steady back-to-back frames through ocean_update over a
ring of tiles (each frame's spectrum comes from HBM, as in bench.py), for each
candidate of
    row_overlap      0 / 1   (the row pass starts under the previous frame's
                              output stage, or waits for it first)
    row_ctas_per_sm  0 (as many as fit), 1, 2, 3, 4, 6, 8 (persistent row-pass
                              grid; caps above the occupancy limit give its grid)
    row_variant      0 .. 5 (N >= 512: warp-specialised row pass, every warp
                              running the prepass and then its line FFT,
                              warp-specialised with 8-point-first lines, or
                              (N = 1024) warp-specialised or every warp with
                              32 x 32 lines, or warp-specialised with 32 x 32
                              lines at three CTAs per SM)
    col_fused        0 / 2 / 4 (N = 512, 1024: the column side as column FFT +
                              output kernels, or as one fused kernel with 2 or 4
                              column pairs per CTA)
and keeps the fastest (median of `reps` runs).  Then it times the 64-tile,
8-sample batch (workloads.batched_tiles) for each wave budget and keeps the
fastest.  It writes DIR/tuning_table.inc -- the table the library compiles
in (copy it to fft-ocean-waves_gb300/csrc/ and rebuild) -- and
DIR/tuning_sweep.json with every measurement.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

SIZES = (32, 64, 128, 256, 512, 1024, 2048)
RING = 8


def time_frames(torch, og, ring, outs, stream, K=40, reps=5):
    """Median ms per frame of K back-to-back frames over the ring."""
    res = []
    for r in range(reps + 1):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda._sleep(2_000_000)
        for i in range(2):                                # lead-in frames (pipeline fill), untimed
            ring[(len(ring) - 2 + i) % len(ring)].update((r * K - 2 + i) / 60.0, *outs[(len(ring) - 2 + i) % len(ring)],
                                                         stream=stream)
        a.record(stream)
        for i in range(K):
            j = i % len(ring)
            ring[j].update((r * K + i) / 60.0, *outs[j], stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        if r:
            res.append(a.elapsed_time(b) / K)
    return statistics.median(res)


def tune_size(torch, og, workloads, N, reps, log):
    dev = torch.device("cuda")
    stream = torch.cuda.Stream()
    p = workloads.plain(N)
    ring = [og.Ocean(p, seed=1) for _ in range(RING)]
    outs = [(torch.empty((N, N), device=dev), torch.empty((N, N), device=dev), torch.empty((N, N), device=dev),
             torch.empty((N, N, 4), device=dev)) for _ in range(RING)]
    base = og.get_tuning(N)
    results = []
    with torch.cuda.stream(stream):
        for i in range(2 * RING):                         # warm-up (first-launch set-up of every kernel)
            ring[i % RING].update(i / 60.0, *outs[i % RING], stream=stream)
        torch.cuda.synchronize()
        fused_opts = (0, 2, 4) if N in (512, 1024) else (0,)
        variants = ((0, 1, 2, 3, 4, 5) if N == 1024 else (0, 1, 2)) if N >= 512 else (1,)
        for variant in variants:                          # row pass: warp-specialised or every warp
            for fused in fused_opts:                      # the fused column kernel exists for 512 and 1024
                for cap in (0, 1, 2, 3, 4, 6, 8):         # 0: as many CTAs per SM as fit
                    for overlap in (0, 1):
                        og.set_tuning(N, row_overlap=overlap, row_ctas_per_sm=cap, col_fused=fused,
                                      row_variant=variant)
                        ms = time_frames(torch, og, ring, outs, stream, reps=reps)
                        results.append({"row_overlap": overlap, "row_ctas_per_sm": cap, "col_fused": fused,
                                        "row_variant": variant, "ms_per_frame": round(ms, 6)})
                        log(f"N={N} variant={variant} fused={fused} overlap={overlap} ctas/SM={cap}: "
                            f"{ms * 1e3:.2f} us")
    for oc in ring:
        oc.close()
    best = min(results, key=lambda r: r["ms_per_frame"])
    og.set_tuning(N, **base)
    return best, results


def tune_batch(torch, og, workloads, reps, log, budgets=(32, 48, 64, 96)):
    dev = torch.device("cuda")
    stream = torch.cuda.Stream()
    S = 8
    tiles, seeds, times = workloads.batched_tiles(samples=S)
    outs = []
    keep = []
    for p in tiles:
        b3 = torch.empty((S, 3, p.N, p.N), device=dev)
        b4 = torch.empty((S, p.N, p.N, 4), device=dev)
        keep += [b3, b4]
        outs += [(b3[s, 0], b3[s, 1], b3[s, 2], b4[s]) for s in range(S)]
    saved = {N: og.get_tuning(N) for N in SIZES}
    results = []
    with torch.cuda.stream(stream):
        for mib in budgets:
            for N in SIZES:
                og.set_tuning(N, wave_mib=mib)
            with og.OceanBatch(tiles, seeds, S) as b:
                ts = []
                for r in range(reps + 1):
                    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    b.update(times, outs, stream=stream)
                    e.record(stream)
                    torch.cuda.synchronize()
                    if r:
                        ts.append(a.elapsed_time(e))
                b.device_status()
            ms = statistics.median(ts)
            results.append({"wave_mib": mib, "batch_ms": round(ms, 4)})
            log(f"batch wave_mib={mib}: {ms:.3f} ms")
    for N in SIZES:
        og.set_tuning(N, **saved[N])
    return min(results, key=lambda r: r["batch_ms"]), results


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="tuning_out")
    ap.add_argument("--sizes", default=",".join(str(n) for n in SIZES))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--no-batch", action="store_true")
    args = ap.parse_args()
    import torch
    import build as ocean_build
    ocean_build.build()
    import ocean_gb300 as og
    import workloads
    os.makedirs(args.out, exist_ok=True)
    log = lambda m: print(m, flush=True)
    sizes = [int(x) for x in args.sizes.split(",")]
    table = {N: og.get_tuning(N) for N in SIZES}
    sweep = {"sizes": {}, "batch": None}
    for N in sizes:
        best, res = tune_size(torch, og, workloads, N, args.reps, log)
        table[N]["row_overlap"] = best["row_overlap"]
        table[N]["row_ctas_per_sm"] = best["row_ctas_per_sm"]
        table[N]["col_fused"] = best.get("col_fused", 0)
        table[N]["row_variant"] = best.get("row_variant", table[N]["row_variant"])
        sweep["sizes"][N] = {"best": best, "all": res}
    for N in SIZES:                                       # the batch is timed with the winners
        og.set_tuning(N, **table[N])
    if not args.no_batch:
        best, res = tune_batch(torch, og, workloads, args.reps, log)
        for N in SIZES:
            table[N]["wave_mib"] = best["wave_mib"]
        sweep["batch"] = {"best": best, "all": res}
    dev = torch.cuda.get_device_name()
    lines = ["// Launch configuration per N: {N, row_overlap, row_ctas_per_sm, wave_mib, col_fused, row_variant}.",
             "// Written by fft-ocean-waves_gb300/tune.py from measurements on a GB300",
             f"// ({dev}): steady back-to-back frames for the single-tile knobs (median of",
             f"// {args.reps} runs of 40 frames), the 64-tile batch for wave_mib."]
    lines += [f"{{{N}, {table[N]['row_overlap']}, {table[N]['row_ctas_per_sm']}, {table[N]['wave_mib']}, "
              f"{table[N]['col_fused']}, {table[N]['row_variant']}}}," for N in SIZES]
    with open(os.path.join(args.out, "tuning_table.inc"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    with open(os.path.join(args.out, "tuning_sweep.json"), "w") as fh:
        json.dump(sweep, fh, indent=1)
    print("\n".join(lines))


if __name__ == "__main__":
    main()
