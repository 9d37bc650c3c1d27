"""Benchmark of the per-frame Tessendorf ocean update (one JSON line on rank 0).

Workload (default): the plain drop-in tile at N=1024 -- L=2000 m, A=2, wind
30 m/s at 30 deg, lambda=1.3, l=0.1, seeded uniform noise (seed 1) -- advanced
frame by frame at dt = 1/60 s from t = 0 (workloads.plain).  A step is one
frame: the row pass (evolution + choppy + horizontal FFT) and the column pass
(vertical FFT + inversion + lambda + normal + Jacobian), our kernels only.

value: K frames back to back on one stream, timed by two CUDA events around
all of them.  The frames rotate over R = 8 tiles with their own spectrum,
scratch and output maps (8 x 97 MB, well above the 129 MB L2), so a frame's
spectrum was last touched 7 frames (about 600 MB of traffic) earlier and is
read from HBM, as in a renderer's frame; no L2 flush runs inside the timed
region.  A device-side sleep before the frames lets the host queue them ahead
of the GPU, so the device never waits for a launch, and two untimed lead-in
frames precede the first timed one, so that every timed frame follows a frame
(its row pass overlaps the previous frame's output stage) as in steady state.

isolated: the same frames one at a time, L2 flushed before each (a 512 MiB
buffer written, then a 512 MiB buffer read) and each frame bracketed by its own
CUDA events, so every frame also pays the launch of its first kernel.

kernel_ms: each stage launched K times back to back over the R tiles between
two events (the average launch duration on the stream); the row stage's
spectrum comes from HBM as in a frame, the column stages' inputs (which a live
frame finds in L2) come from HBM too, so theirs are upper bounds.

e2e: the same frames through the C ABI (ocean_update) with every output map
copied back to pinned host memory inside the timed region; the per-frame input
is the time value (a by-value argument).  The headline e2e pipelines the
frames (two device output sets, the copies on their own stream, so frame i+1
computes while frame i's 29 MB cross the host link; no L2 flush, the link
sets the rate); `serial_value` runs compute and copies one after the other,
L2 flushed before each frame.

--impl reference: the reference's algorithm (FP32 C++ port of the shader
passes, oracle/ocean_oracle.c port_*) on the host cores, same config/metric.

Multi-GPU (torchrun): tiles do not exchange data, so every rank advances its
own tiles (replicas, weak scaling); time = max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fft-ocean-waves_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

METRIC = "ocean frames/s (N=1024, 3 fields + normal/J)"
BYTES_PER_TEXEL = 92            # algorithmic bytes per texel per frame
# The frame's 92 B/texel split over its kernels: rows read h0 (16) and write
# the intermediate (24); columns read it (24); outputs write dx, dy, dz and
# normal_j (28); the fused column kernel does both column stages (52).
KERNEL_BYTES = {"k_row_pass": 40, "k_row_ws": 40, "k_col_fft": 24, "k_col_out": 28, "k_col_fused": 52}
# The frame's compulsory I/O: h0 in (16) and the four maps out (28); the
# intermediate round trip is left out (it can stay in L2).
COMPULSORY_BYTES_PER_TEXEL = 44


def row_kernel(N):
    """The row stage's kernel: warp-specialised where a line is whole warps
    and the tuning keeps that variant, else the every-warp pass."""
    import ocean_gb300 as og
    return "k_row_ws" if N >= 512 and og.get_tuning(N)["row_variant"] not in (1, 4) else "k_row_pass"


def c2_params(N):
    import workloads
    return workloads.plain(N)


def bench_config(N, world):
    """The workload description both arms print (identical dicts)."""
    return {"workload": f"plain tile N={N}, L=2000 m, A=2, V=30 m/s @30deg, lambda=1.3, l=0.1, "
                        f"frames at dt=1/60 s", "N": N, "fields": 3,
            "l2": "inputs larger than L2: frames rotate over 8 tiles (8 x 97 MB), no flush in the timed region",
            "steady_state": "2 untimed lead-in frames queued right before the K timed ones",
            "parallelism": f"replicas x{world}"}


def peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_table():
    """Per-launch DRAM bytes from the committed ncu summary, if present."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the GPU is busy."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(backend="nccl"):
    """One process per GPU (torchrun env).  Tiles are replicas: the ranks only
    meet in the timing barriers."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier_max(world, value, device="cuda"):
    """Barrier, then the maximum of `value` over the ranks (the job's time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(N, seconds, threads=None):
    """FP32 port of the reference algorithm (oracle/) on the host cores, on a
    time-bounded sample of consecutive frames; also the checker of the GPU
    frame against the FP64 oracle."""
    from oracle import oracle
    import numpy as np
    d = c2_params(N)
    p = oracle.Params(N=N, L=d.L, amplitude=d.amplitude, wind_speed=d.wind_speed, wind_x=d.wind_dir_x,
                      wind_y=d.wind_dir_y, choppiness=d.choppiness, suppression=d.suppression, gravity=d.gravity)
    if threads:
        oracle.set_threads(threads)
    cores = oracle.max_threads()
    nz = oracle.noise(1, N)
    port = oracle.Port(p, nz)
    port.frame(0.0)
    frames, t0 = 0, time.perf_counter()
    while True:
        port.frame(frames / 60.0)
        frames += 1
        el = time.perf_counter() - t0
        if el >= seconds and frames >= 3:
            break
    port.close()
    return {"value": frames / el, "unit": "frames/s", "cores": cores, "kind": "port",
            "sample": f"{frames} consecutive N={N} frames (dt=1/60 s) in {el:.1f} s, FP32 reference algorithm "
                      f"(2*log2N radix-2 ping-pong passes per field), OpenMP {cores} threads"}


def parity_check(N, gpu_frame, t):
    """Part of the CPU leg, after the timed region: the FP64 oracle checks one
    GPU frame (err_vs_fp64).  Nothing timed runs through the oracle."""
    from oracle import oracle
    import numpy as np
    d = c2_params(N)
    p = oracle.Params(N=N, L=d.L, amplitude=d.amplitude, wind_speed=d.wind_speed, wind_x=d.wind_dir_x,
                      wind_y=d.wind_dir_y, choppiness=d.choppiness, suppression=d.suppression, gravity=d.gravity)
    h = oracle.h0(p, oracle.noise(1, N))
    ref = oracle.update(p, h, t)
    errs = {k: oracle.rel_l2(gpu_frame[k], ref[k]) for k in ("dx", "dy", "dz")}
    errs["normal"] = oracle.rel_l2(gpu_frame["nj"][..., :3], ref["nj"][..., :3])
    errs["J"] = oracle.rel_l2(gpu_frame["nj"][..., 3], ref["nj"][..., 3])
    errs["J_max_abs"] = float(np.abs(gpu_frame["nj"][..., 3].astype(np.float64) - ref["nj"][..., 3]).max())
    errs["dy_max_abs"] = float(np.abs(gpu_frame["dy"].astype(np.float64) - ref["dy"]).max())
    return {k: float(f"{v:.3g}") for k, v in errs.items()}


RING = 8      # tiles the timed frames rotate over (8 x 97 MB: every frame's inputs come from HBM)
LEAD_IN = 2   # untimed frames queued right before the timed ones (pipeline fill)


def run_gpu(args, world, rank, local):
    import numpy as np
    import torch
    import build as ocean_build
    ocean_build.build()
    import ocean_gb300 as og

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    N = args.size
    p = c2_params(N)

    def maps():
        return (torch.empty((N, N), dtype=torch.float32, device=dev), torch.empty((N, N), dtype=torch.float32, device=dev),
                torch.empty((N, N), dtype=torch.float32, device=dev),
                torch.empty((N, N, 4), dtype=torch.float32, device=dev))

    # R tiles of the same workload (same spectrum, own state and outputs)
    ring = [og.Ocean(p, seed=1 + rank) for _ in range(RING)]
    ring_out = [maps() for _ in range(RING)]
    oc = ring[0]
    dx, dy, dz, nj = ring_out[0]
    fl_w = torch.empty(128 << 20, dtype=torch.float32, device=dev)   # 512 MiB
    fl_r = torch.ones(128 << 20, dtype=torch.float32, device=dev)
    fl_sink = torch.empty((), dtype=torch.float32, device=dev)

    def flush():
        fl_w.zero_()
        torch.sum(fl_r, dim=(0,), out=fl_sink)

    def prime():
        """Keep the device busy while the host queues the timed launches."""
        torch.cuda._sleep(4_000_000)   # ~2 ms at 2 GHz

    K = args.steps
    launches = 0
    with torch.cuda.stream(stream):
        for i in range(max(args.warmup, RING)):
            flush()
            ring[i % RING].update(i / 60.0, *ring_out[i % RING], stream=stream)
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            wall0 = time.perf_counter()
            # headline: K whole frames through ocean_update back to back (three
            # kernels each, chained by programmatic dependent launch), rotating
            # over the R tiles
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            prime()
            # two untimed lead-in frames on the stream: the first timed frame
            # then follows a frame, as every later one does (steady state)
            for i in range(LEAD_IN):
                j = (RING - LEAD_IN + i) % RING
                ring[j].update((args.warmup - LEAD_IN + i) / 60.0, *ring_out[j], stream=stream)
            per_frame = 2 if og.get_tuning(N)["col_fused"] else 3   # kernels per frame
            e0.record(stream)
            for i in range(K):
                j = i % RING
                ring[j].update((args.warmup + i) / 60.0, *ring_out[j], stream=stream)
            e1.record(stream)
            launches += per_frame * K
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
            if world > 1:
                torch.distributed.barrier()
            total_s = barrier_max(world, e0.elapsed_time(e1) / 1e3)

            # isolated frames: L2 flushed before each, each bracketed by events
            ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
            for i in range(K):
                flush()
                ev[i][0].record(stream)
                oc.update((args.warmup + i) / 60.0, dx, dy, dz, nj, stream=stream)
                ev[i][1].record(stream)
            torch.cuda.synchronize()
            iso_s = barrier_max(world, sum(ev[i][0].elapsed_time(ev[i][1]) for i in range(K)) / 1e3)

            # per-stage average launch durations: each stage K times back to
            # back over the R tiles between two events.  Every launch is a
            # programmatic dependent of the one before (its launch latency is
            # hidden, as inside a frame); the row passes are made to wait for
            # their predecessor before starting (row_overlap 0), so that their
            # work does not overlap and the average is one launch's duration.
            kernel_ms = {}
            saved = og.set_tuning(N, row_overlap=0)
            if og.get_tuning(N)["col_fused"]:                # the frame's column side is one kernel
                stages = ((row_kernel(N), lambda j, t: ring[j].update_rows(t, stream=stream)),
                          ("k_col_fused", lambda j, t: ring[j].update_columns_outputs(*ring_out[j], stream=stream)))
            else:
                stages = ((row_kernel(N), lambda j, t: ring[j].update_rows(t, stream=stream)),
                          ("k_col_fft", lambda j, t: ring[j].update_columns(stream=stream)),
                          ("k_col_out", lambda j, t: ring[j].update_outputs(*ring_out[j], stream=stream)))
            for name, call in stages:
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                prime()
                a.record(stream)
                for i in range(K):
                    call(i % RING, (args.warmup + i) / 60.0)
                b.record(stream)
                torch.cuda.synchronize()
                kernel_ms[name] = a.elapsed_time(b) / K
            og.set_tuning(N, **saved)
            # the same stages with events between them inside flushed frames
            # (each then also pays its own launch)
            kv = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(K)]
            for i in range(K):
                flush()
                t = (args.warmup + i) / 60.0
                for j, (name, call) in enumerate(stages):
                    kv[i][j].record(stream)
                    if j == 0:
                        oc.update_rows(t, stream=stream)
                    elif name == "k_col_fused":
                        oc.update_columns_outputs(dx, dy, dz, nj, stream=stream)
                    elif name == "k_col_fft":
                        oc.update_columns(stream=stream)
                    else:
                        oc.update_outputs(dx, dy, dz, nj, stream=stream)
                kv[i][len(stages)].record(stream)
            torch.cuda.synchronize()
            kernel_iso_ms = {name: sum(kv[i][j].elapsed_time(kv[i][j + 1]) for i in range(K)) / K
                             for j, (name, _) in enumerate(stages)}

            # e2e: C-ABI call + all outputs copied to pinned host memory, every frame.
            hdx, hdy, hdz = (torch.empty((N, N), dtype=torch.float32, pin_memory=True) for _ in range(3))
            hnj = torch.empty((N, N, 4), dtype=torch.float32, pin_memory=True)
            E = max(20, K // 4)
            for i in range(3):
                oc.update(i / 60.0, dx, dy, dz, nj, stream=stream)
                for hsrc, hdst in ((dx, hdx), (dy, hdy), (dz, hdz), (nj, hnj)):
                    hdst.copy_(hsrc, non_blocking=True)
            torch.cuda.synchronize()
            ee = []
            for i in range(E):
                flush()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                oc.update(i / 60.0, dx, dy, dz, nj, stream=stream)
                for hsrc, hdst in ((dx, hdx), (dy, hdy), (dz, hdz), (nj, hnj)):
                    hdst.copy_(hsrc, non_blocking=True)
                b.record(stream)
                ee.append((a, b))
            torch.cuda.synchronize()
            e2e_serial_s = barrier_max(world, sum(a.elapsed_time(b) for a, b in ee) / 1e3)

            # e2e, pipelined (the headline): the same C-ABI frames into two
            # alternating device output sets on the compute stream; each frame's
            # dx, dy, dz, normal_j go to pinned host memory on a copy stream while
            # the next frame computes.  Timed from the first frame's launch to the
            # last frame's copy.  No L2 flush here: the flush would run on the
            # compute stream inside the timed region, and the rate is set by the
            # host link (29 MB per frame) with the compute hidden under it.
            copy_stream = torch.cuda.Stream()
            dsets = [(dx, dy, dz, nj), ring_out[1]]
            hsets = [(hdx, hdy, hdz, hnj),
                     tuple(torch.empty(b.shape, dtype=torch.float32, pin_memory=True) for b in (dx, dy, dz, nj))]
            computed = [torch.cuda.Event(), torch.cuda.Event()]
            copied = [None, None]

            def e2e_frame(i):
                j = i % 2
                if copied[j] is not None:                  # set j's previous frame is on the host
                    stream.wait_event(copied[j])
                oc.update(i / 60.0, *dsets[j], stream=stream)
                computed[j].record(stream)
                copy_stream.wait_event(computed[j])
                with torch.cuda.stream(copy_stream):
                    for hsrc, hdst in zip(dsets[j], hsets[j]):
                        hdst.copy_(hsrc, non_blocking=True)
                copied[j] = torch.cuda.Event()
                copied[j].record(copy_stream)

            for i in range(3):
                e2e_frame(i)
            torch.cuda.synchronize()
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            for i in range(E):
                e2e_frame(i)
            stream.wait_event(copied[(E - 1) % 2])
            p1.record(stream)
            torch.cuda.synchronize()
            e2e_s = barrier_max(world, p0.elapsed_time(p1) / 1e3)
        clocks = clk.summary()
        # one frame at a known time for the parity check
        t_chk = 1000 / 60.0
        oc.update(t_chk, dx, dy, dz, nj, stream=stream)
        torch.cuda.synchronize()
        oc.device_status()
        frame = {"dx": dx.cpu().numpy(), "dy": dy.cpu().numpy(), "dz": dz.cpu().numpy(), "nj": nj.cpu().numpy()}
        grid_stats = None if args.no_extra else bench_grid(torch, og, dev, stream, flush, (dx, dy, dz, nj))
    for r in ring:
        r.close()
    del ring_out

    if rank != 0:
        return None
    value = world * K / total_s
    ms = 1e3 * total_s / K
    iso_ms = 1e3 * iso_s / K
    # the dominant kernel by the isolated per-kernel times (each a frame's
    # stage with its own launch, inputs as in a frame); its achieved rate uses
    # the back-to-back duration (launch hidden, as in the frame)
    dominant = max(kernel_iso_ms, key=kernel_iso_ms.get)
    dom_ms = kernel_ms[dominant]
    dom_bytes = KERNEL_BYTES[dominant] * N * N
    peak, peak_kind = peak_hbm()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = traffic_table().get(f"{dominant}@{N}")
    frame_gbs = BYTES_PER_TEXEL * N * N / (ms * 1e-3) / 1e9
    iso_gbs = BYTES_PER_TEXEL * N * N / (iso_ms * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "frames/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded splitmix64 uniform noise, seed 1)",
        "config": bench_config(N, world),
        "tuning": og.get_tuning(N),
        "kernel_ms": {k: round(v, 5) for k, v in kernel_ms.items()},
        "kernel_ms_isolated": {k: round(v, 5) for k, v in kernel_iso_ms.items()},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": dom_bytes, "traffic": traffic},
        "roofline_frame": {"bytes_per_frame": BYTES_PER_TEXEL * N * N, "achieved": round(frame_gbs, 1),
                           "frac": round(frame_gbs / peak, 4)},
        "roofline_compulsory": {"bytes_per_frame": COMPULSORY_BYTES_PER_TEXEL * N * N,
                                "achieved": round(frame_gbs * COMPULSORY_BYTES_PER_TEXEL / BYTES_PER_TEXEL, 1),
                                "frac": round(frame_gbs * COMPULSORY_BYTES_PER_TEXEL / BYTES_PER_TEXEL / peak, 4)},
        "isolated": {"value": round(world * K / iso_s, 1), "unit": "frames/s", "ms_per_frame": round(iso_ms, 5),
                     "frac": round(iso_gbs / peak, 4),
                     "how": "one frame at a time, L2 flushed before each, CUDA events around each frame"},
        "e2e": {"value": round(world * E / e2e_s, 1), "unit": "frames/s", "h2d_bytes_per_step": 8,
                "d2h_bytes_per_step": 28 * N * N,
                "path": "ocean_update (C ABI) + D2H of dx, dy, dz, normal_j to pinned host buffers; "
                        "pipelined: frame i+1 computes while frame i copies (two output sets, a copy stream)",
                "serial_value": round(world * E / e2e_serial_s, 1),
                "serial_path": "ocean_update then the four D2H copies, one frame at a time on one stream"},
        "gpu_launches": launches,
        "clocks": clocks,
        "wall_s_timed_region": round(wall, 4),
    }
    if not args.no_extra:
        out["grid"] = grid_stats
        out["adjoint"] = bench_adjoint(torch, og, dev, stream)
        out["adjoint_large"] = bench_adjoint_large(torch, og, dev, stream)
        out["batched"] = bench_batched(torch, og, dev, stream, flush)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(N, args.cpu_seconds)
        out["err_vs_fp64"] = parity_check(N, frame, t_chk)
    return out


def bench_adjoint(torch, og, dev, stream, reps=5):
    """Parameter-fit workload: N=512, T=32 frames at dt=0.1 s.  Forward = the
    32 frames into a (T, 3, N, N) buffer; backward = ocean_backward over the
    32 frames' upstream gradients (one call, no stored or recomputed frames)."""
    import workloads
    N, T = 512, 32
    times = [0.1 * j for j in range(T)]
    oc = og.Ocean(workloads.fit_params(), seed=3)
    D = torch.empty((T, 3, N, N), device=dev)
    nj = torch.empty((N, N, 4), device=dev)
    G = torch.randn((3, T, N, N), device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fw, bw = [], []
    with torch.cuda.stream(stream):
        for rep in range(reps + 2):
            ev[0].record(stream)
            for j, t in enumerate(times):
                oc.update(t, D[j, 0], D[j, 1], D[j, 2], nj, stream=stream)
            ev[1].record(stream)
            oc.backward(times, G[0], G[1], G[2], stream=stream)
            ev[2].record(stream)
            torch.cuda.synchronize()
            if rep >= 2:
                fw.append(ev[0].elapsed_time(ev[1]))
                bw.append(ev[1].elapsed_time(ev[2]))
    oc.close()
    f, b = sum(fw) / len(fw), sum(bw) / len(bw)
    return {"workload": "N=512, T=32 frames, dt=0.1 s (parameter-fit config)", "forward_ms": round(f, 4),
            "backward_ms": round(b, 4), "fwd_frames_per_s": round(T / (f * 1e-3), 1),
            "fwd_adj_frames_per_s": round(T / ((f + b) * 1e-3), 1), "adj_over_fwd": round((f + b) / f, 3),
            "gpu_launches_per_step": 3 * T + 2}


def bench_adjoint_large(torch, og, dev, stream, n_sets=16, chunk=16):
    """Full-spectrum adjoint at N=2048 (workloads.adjoint_sets): per set, the
    MSE over T=64 frames (dt=0.05 s) of the displacement maps against a target
    sequence generated on the device from the 5 %-perturbed h0, and dL/dh0 for
    every mode.

    forward: per frame, the model frame and the target frame (two
    ocean_update calls) and the squared residual summed on the device: the
    loss.  backward: frames are recomputed from h0 (only h0 is kept) in chunks
    of 16: model and target frames, residual * 2/M as the upstream gradient,
    ocean_backward accumulating dL/dh0.  Device memory is taken from
    cudaMemGetInfo at the peak of each phase, relative to before the set."""
    import workloads as W
    N, T, dt = W.ADJ_N, W.ADJ_T, W.ADJ_DT
    times = [dt * j for j in range(T)]
    M = 3.0 * T * N * N
    fwd_ms = bwd_ms = 0.0
    fwd_mem = bwd_mem = 0
    losses = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]   # forward start/end, backward start/end
    with torch.cuda.stream(stream):
        for s, (p, seed) in enumerate(W.adjoint_sets(n_sets)):
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            model = og.Ocean(p, seed=seed)
            target = og.Ocean(p, seed=seed)
            h0 = torch.empty((N, N, 4), device=dev)
            model.get_h0(h0, stream=stream)
            gen = torch.Generator(device=dev).manual_seed(W.perturb_seed(s))
            h0t = h0 * (1.0 + 0.05 * torch.randn(h0.shape, device=dev, generator=gen))
            target.set_h0(h0t, stream=stream)
            del h0, h0t
            D = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
            Tg = [torch.empty((N, N), device=dev) for _ in range(3)] + [torch.empty((N, N, 4), device=dev)]
            acc = torch.zeros((), dtype=torch.float64, device=dev)
            if s == 0:   # untimed: the first use of the residual's kernels (module load / JIT on this arch)
                for f in range(3):
                    acc += torch.sum(torch.square(D[f] - Tg[f]), dtype=torch.float64)
                acc.zero_()
            torch.cuda.synchronize()
            ev[0].record(stream)
            for t in times:
                model.update(t, *D, stream=stream)
                target.update(t, *Tg, stream=stream)
                for f in range(3):
                    acc += torch.sum(torch.square(D[f] - Tg[f]), dtype=torch.float64)
            ev[1].record(stream)
            torch.cuda.synchronize()
            fwd_mem = max(fwd_mem, free0 - torch.cuda.mem_get_info()[0])
            losses.append(acc.item() / M)
            G = torch.empty((3, chunk, N, N), device=dev)
            nj = torch.empty((N, N, 4), device=dev)
            dh0 = torch.zeros((N, N, 4), device=dev)
            model.backward(times[:1], G[0, :1], G[1, :1], G[2, :1], dh0=dh0, stream=stream)   # adjoint scratch
            torch.cuda.synchronize()
            ev[2].record(stream)
            for c0 in range(0, T, chunk):
                n = min(chunk, T - c0)
                for j in range(n):
                    model.update(times[c0 + j], G[0, j], G[1, j], G[2, j], nj, stream=stream)
                    target.update(times[c0 + j], *Tg, stream=stream)
                    for f in range(3):
                        G[f, j].sub_(Tg[f]).mul_(2.0 / M)
                model.backward(times[c0:c0 + n], G[0, :n], G[1, :n], G[2, :n], dh0=dh0, accumulate=c0 > 0,
                               stream=stream)
            ev[3].record(stream)
            torch.cuda.synchronize()
            bwd_mem = max(bwd_mem, free0 - torch.cuda.mem_get_info()[0])
            fwd_ms += ev[0].elapsed_time(ev[1])
            bwd_ms += ev[2].elapsed_time(ev[3])
            model.device_status()
            model.close()
            target.close()
            del D, Tg, G, nj, dh0
    return {"workload": f"{n_sets} parameter sets, N={N}, T={T} frames at dt={dt} s: MSE of the displacement maps "
                        f"against the target of the 5%-perturbed h0 (generated on the device), dL/dh0 per mode",
            "forward_frames_per_s": round(n_sets * T / (fwd_ms * 1e-3), 1),
            "forward_ms_per_set": round(fwd_ms / n_sets, 3),
            "backward_ms_per_set": round(bwd_ms / n_sets, 3),
            "fwd_adj_over_fwd": round((fwd_ms + bwd_ms) / fwd_ms, 3),
            "fwd_mem_bytes": int(fwd_mem), "bwd_mem_bytes": int(bwd_mem),
            "loss_mean": float(f"{sum(losses) / len(losses):.6g}"), "frames_stored": 0,
            "how": "forward = model + target frame and the squared residual per frame; backward = frames recomputed "
                   "from h0 in chunks of 16 (model + target + residual) and ocean_backward (dL/dh0 accumulated)"}


def bench_batched(torch, og, dev, stream, flush, S=8, reps=3):
    """Batched mixed-size launch vs looping the plain per-tile update over the
    same 64 tiles x 8 time samples (t ~ U(0, 600) s)."""
    import workloads
    tiles, seeds, times = workloads.batched_tiles(samples=S)
    n = len(tiles)
    outs = []
    bufs = []
    for p in tiles:
        N = p.N
        b3 = torch.empty((S, 3, N, N), device=dev)
        b4 = torch.empty((S, N, N, 4), device=dev)
        bufs += [b3, b4]
        for s in range(S):
            outs.append((b3[s, 0], b3[s, 1], b3[s, 2], b4[s]))
    texels = sum(p.N * p.N for p in tiles) * S
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    bt, lt = [], []
    with og.OceanBatch(tiles, seeds, S) as b, torch.cuda.stream(stream):
        singles = [og.Ocean(p, seed=sd) for p, sd in zip(tiles, seeds)]
        for rep in range(reps + 1):
            flush()
            ev[0].record(stream)
            b.update(times, outs, stream=stream)
            ev[1].record(stream)
            torch.cuda.synchronize()
            if rep:
                bt.append(ev[0].elapsed_time(ev[1]))
            flush()
            ev[0].record(stream)
            for i, oc in enumerate(singles):
                for s in range(S):
                    oc.update(times[i * S + s], *outs[i * S + s], stream=stream)
            ev[1].record(stream)
            torch.cuda.synchronize()
            if rep:
                lt.append(ev[0].elapsed_time(ev[1]))
        # the same loop captured in a CUDA graph (no host launch overhead)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for i, oc in enumerate(singles):
                for s in range(S):
                    oc.update(times[i * S + s], *outs[i * S + s], stream=stream)
        gt = []
        for rep in range(reps + 1):
            flush()
            ev[0].record(stream)
            g.replay()
            ev[1].record(stream)
            torch.cuda.synchronize()
            if rep:
                gt.append(ev[0].elapsed_time(ev[1]))
        del g
        b.device_status()
        for oc in singles:
            oc.close()
    bms, lms, gms = sum(bt) / len(bt), sum(lt) / len(lt), sum(gt) / len(gt)
    return {"workload": f"{n} tiles, N in {{128..2048}} (seed 2), {S} samples each, t~U(0,600) s",
            "tile_frames": n * S, "texels_per_launch": texels, "batched_ms": round(bms, 3),
            "loop_ms": round(lms, 3), "batched_tile_frames_per_s": round(n * S / (bms * 1e-3), 1),
            "loop_tile_frames_per_s": round(n * S / (lms * 1e-3), 1), "speedup_vs_loop": round(lms / bms, 3),
            "loop_graph_ms": round(gms, 3), "speedup_vs_graphed_loop": round(gms / bms, 3),
            "batched_effective_GBps": round(92 * texels / (bms * 1e-3) / 1e9, 1)}


def bench_grid(torch, og, dev, stream, flush, oc_maps, reps=20):
    """The render grid's displacement (the reference's 1024-square grid, UV
    repeat 64) over one frame's N=1024 maps, and its tessellation levels."""
    dx, dy, dz, nj = oc_maps
    g = og.grid_params()
    n = g.squares
    verts = torch.empty(((n + 1) * (n + 1), 8), device=dev)
    levels = torch.empty((2 * n * n, 4), device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    vt, lt = [], []
    with torch.cuda.stream(stream):
        for r in range(reps + 3):
            flush()
            ev[0].record(stream)
            og.displace_grid(dx, dy, dz, nj, g, verts, stream=stream)
            ev[1].record(stream)
            og.grid_tess_levels(g, levels, stream=stream)
            ev[2].record(stream)
            torch.cuda.synchronize()
            if r >= 3:
                vt.append(ev[0].elapsed_time(ev[1]))
                lt.append(ev[1].elapsed_time(ev[2]))
    v_ms, l_ms = sum(vt) / len(vt), sum(lt) / len(lt)
    nv = (n + 1) * (n + 1)
    # the sky environment cube map of render_envmap() (512 x 512 faces) on
    # seeded stand-in tables, and the shading of the grid's vertices from it
    import numpy as np
    rng = np.random.default_rng(5)
    tr = torch.from_numpy(rng.random((64, 256, 4), dtype=np.float32)).to(dev)
    ins = torch.from_numpy(rng.random((32, 128, 256, 4), dtype=np.float32) * np.float32(0.05)).to(dev)
    sky = torch.empty((6, 512, 512, 4), device=dev)
    colors = torch.empty((nv, 4), device=dev)
    cam, sun = (0.0, 10.0, 0.0), og.sky_sun_direction(-0.4)
    st, ct = [], []
    with torch.cuda.stream(stream):
        for r in range(reps + 3):
            flush()
            ev[0].record(stream)
            og.sky_envmap(cam, sun, tr, ins, sky, stream=stream)
            ev[1].record(stream)
            og.shade_grid(verts, cam, sun, (0.0, 0.2, 0.3), sky, colors, stream=stream)
            ev[2].record(stream)
            torch.cuda.synchronize()
            if r >= 3:
                st.append(ev[0].elapsed_time(ev[1]))
                ct.append(ev[1].elapsed_time(ev[2]))
    s_ms, c_ms = sum(st) / len(st), sum(ct) / len(ct)
    return {"workload": f"grid of {n} squares (UV repeat 64) over N={dy.shape[0]} maps, L2 flushed",
            "vertices": nv, "displace_ms": round(v_ms, 4), "vertices_per_s": round(nv / (v_ms * 1e-3), 1),
            "tess_levels_ms": round(l_ms, 4), "triangles_per_s": round(2 * n * n / (l_ms * 1e-3), 1),
            "sky_envmap_ms": round(s_ms, 4), "sky_texels_per_s": round(6 * 512 * 512 / (s_ms * 1e-3), 1),
            "shade_ms": round(c_ms, 4), "shaded_vertices_per_s": round(nv / (c_ms * 1e-3), 1)}


def run_reference(args, world, rank):
    """The reference's algorithm on the host cores (FP32 port, OpenMP)."""
    if rank != 0:
        return None
    from oracle import oracle
    N = args.size
    d = c2_params(N)
    p = oracle.Params(N=N, L=d.L, amplitude=d.amplitude, wind_speed=d.wind_speed, wind_x=d.wind_dir_x,
                      wind_y=d.wind_dir_y, choppiness=d.choppiness, suppression=d.suppression, gravity=d.gravity)
    cores = oracle.max_threads()
    port = oracle.Port(p, oracle.noise(1, N))
    for i in range(args.warmup):
        port.frame(i / 60.0)
    ts = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        port.frame((args.warmup + i) / 60.0)
        ts.append(time.perf_counter() - t0)
    port.close()
    total = sum(ts)
    value = args.steps / total
    return {
        "metric": METRIC, "value": round(value, 3), "unit": "frames/s", "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded splitmix64 uniform noise, seed 1)",
        "config": bench_config(N, world),
        "cpu_baseline": {"value": round(value, 3), "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} consecutive N={N} frames; FP32 port of the reference's GLSL passes "
                                   f"(the GL path itself is unavailable on this box)"},
        "e2e": {"value": round(value, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the adjoint and batched measurements")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        world, rank, local = dist_init()
        out = run_gpu(args, world, rank, local)
    if out is not None:
        print(json.dumps(out), flush=True)
    if world > 1 and args.impl != "reference":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
