"""Benchmark of the GB300 DIC hot path on the 2048x2048 / 41x41-subset workload.

A step is one target frame through FFT-CC then IC-GN (155,236 POIs) with the
reference image's precompute cached, as the reference's worker thread runs it
(TW/TW_Core/fftcctworkerthread.cpp:399-481).  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU algorithm on the host cores
instead: whole frames of the same workload through the oracle restatement
(whose outputs are pinned to the reference's own code by tests/test_ref_pin.py;
the reference sources themselves are not present where the bench runs).
Multi-GPU runs are independent replicas (the path has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "POIs/s at 2048², 41px subsets; p50/p99 frame latency vs plain FP32 GPU path"
UNIT = "POIs/s"
WORKLOAD = ("2048x2048 uint8 speckle pair (100k speckles, sinusoidal field u=3sin(2pi x/1024)+1.5, "
            "v=2cos(2pi y/768)-0.8, noise sigma 2), ROI 2046x2046 at (1,1), 41x41 subsets (r=20), step 5, "
            "margin 20 -> 155,236 POIs; FFT-CC + IC-GN (max 20 iterations, dP < 0.001) per frame, "
            "reference precompute cached")


def config_of(n_pois, world):
    """The workload's configuration, the same in both arms."""
    return {"workload": WORKLOAD, "pois": n_pois, "parallelism": f"replicas x{world}",
            "l2": "GPU arm: flushed between steps by a 256 MB write outside the timed events; CPU arm: the "
                  "frame's working set (images, gradients, 268 MB LUT) exceeds the host caches"}


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


# --------------------------------------------------------------- clocks ----
class ClockSampler:
    """nvidia-smi clock / throttle sampling every 20 ms; only the samples
    taken between mark_start() and mark_stop() (the timed region) count."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []  # (host time, csv line)
        self.t0 = self.t1 = None

    def start(self, wait_s=5.0):
        """Start sampling and wait (at most wait_s) for the first sample."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        t_end = time.perf_counter() + wait_s
        while not self.lines and time.perf_counter() < t_end:
            time.sleep(0.01)

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.perf_counter(), ln.strip()))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_stop(self):
        self.t1 = time.perf_counter()
        time.sleep(0.05)  # the sample taken at the region's end

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = self.t0 if self.t0 is not None else -1e30
        t1 = (self.t1 + 0.025) if self.t1 is not None else 1e30
        for ts, ln in self.lines:
            if ts < t0 or ts > t1:
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": 20}


# ---------------------------------------------------------- distributed ----
def dist_setup(n_gpus):
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("TWDIC_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    """Max of a per-rank time over all ranks (the job ends with its slowest rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ workloads ----
def workload():
    from tw_gb300 import synth
    return synth.scale_2048()


def params_of(g, path):
    from tw_gb300 import dic
    return dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                           g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, path)


# ------------------------------------------------------------- CPU legs ----
def cpu_rate(pair, g, poi, n_sample, nthreads=0):
    """Oracle (restated reference CPU path) throughput, extrapolated to a full
    frame: the reference recomputes the gradients and the target LUT of the
    whole ROI once per ICGN2D_Algorithm call (TW_paDIC_ICGN2D_CPU.cpp:77-132),
    timed here with an empty POI list, plus FFT-CC and IC-GN of the first
    n_sample POIs scaled to all POIs.  Returns (POIs/s, seconds spent, threads)."""
    from oracle import oracle as O
    sp = np.ascontiguousarray(poi[:n_sample])
    t0 = time.perf_counter()
    O.icgn(pair.ref, pair.tar, g, sp[:0], np.zeros(0, np.float32), np.zeros(0, np.float32), nthreads=nthreads)
    t_pre = time.perf_counter() - t0
    t1 = time.perf_counter()
    u, v, z, st = O.fftcc(pair.ref, pair.tar, sp, g.subset_r, nthreads=nthreads)
    O.icgn(pair.ref, pair.tar, g, sp, u, v, nthreads=nthreads)
    t_sample = time.perf_counter() - t1
    per_poi = max(t_sample - t_pre, 1e-9) / n_sample
    frame_s = t_pre + per_poi * len(poi)
    return len(poi) / frame_s, t_pre + t_sample, O.max_threads()


def cpu_baseline(pair, g, poi, gpu_out=None, target_s=12.0):
    rate, dt, thr = cpu_rate(pair, g, poi, 1500)
    n = int(min(len(poi), max(1500, rate * target_s)))
    rate, dt, thr = cpu_rate(pair, g, poi, n)
    line = {"value": round(rate, 1), "unit": UNIT, "cores": thr, "kind": "port",
            "sample": f"first {n} POIs (row-major) of the workload, FFT-CC + IC-GN, plus the per-frame whole-ROI "
                      f"gradient/LUT precompute, extrapolated to all {len(poi)} POIs ({dt:.1f} s of CPU work); OpenMP "
                      "over POIs; oracle = C++ restatement of the reference CPU path (MKL/FFTW/LAPACKE not available)"}
    if gpu_out is not None:
        line["accuracy_vs_oracle"] = accuracy_vs_oracle(pair, g, poi, gpu_out)
    return line


def accuracy_vs_oracle(pair, g, poi, gpu_out, stride=31):
    """The GPU frame's results against the oracle on every stride-th POI:
    FFT-CC in FP32 (integer guesses), then IC-GN in FP32 (the parity
    reference) and in FP64 from the same guesses.  Integer displacements are
    compared exactly, a difference counted as an exact tie when both shifts
    have the same exact correlation; POIs flagged Success by both sides are
    compared on u, v and the gradients; flags and iteration counts are
    compared on all sampled POIs."""
    from oracle import compare as C
    from oracle import oracle as O
    idx = np.arange(0, len(poi), stride)
    sp = np.ascontiguousarray(poi[idx])
    u, v, z, st = O.fftcc(pair.ref, pair.tar, sp, g.subset_r)
    out = {"pois": int(len(idx)), "sample": f"every {stride}-th POI of the frame"}
    if "u_int" in gpu_out:
        rep = C.fftcc_parity(pair.ref, pair.tar, sp, g.subset_r, gpu_out["u_int"][idx], gpu_out["v_int"][idx],
                             gpu_out["zncc"][idx], u, v, z, st)
        out["fftcc"] = {"compared": rep.n, "integer_equal": rep.n - rep.mismatches, "exact_ties": rep.exact_ties,
                        "rounding_ties": rep.rounding_ties, "unexplained": rep.unexplained,
                        "max_abs_zncc": rep.max_zncc_err}
    p6g, itg, flg = gpu_out["p6"][idx], gpu_out["iters"][idx], gpu_out["flags"][idx]
    for prec in ("f32", "f64"):
        p6o, ito, flo = O.icgn(pair.ref, pair.tar, g, sp, u, v, precision=prec)
        ok = (flg == 0) & (flo == 0)
        d = np.abs(p6g[ok].astype(np.float64) - p6o[ok].astype(np.float64))
        out[prec] = {"compared": int(ok.sum()), "flags_equal": float((flg == flo).mean()),
                     "iterations_equal": float((itg == ito).mean()),
                     "max_abs_u": float(d[:, 0].max()), "max_abs_v": float(d[:, 3].max()),
                     "mean_abs_uv": float(d[:, [0, 3]].mean()),
                     "max_abs_gradient": float(d[:, [1, 2, 4, 5]].max())}
    return out


def cpu_frame(pair, g, poi, nthreads=0):
    """One whole frame on the host cores, as the reference's CPU path runs it:
    FFT-CC of every POI (Fftcc2D_CPU::Algorithm_FFTCC), then IC-GN of every
    POI including the per-call whole-ROI gradient and LUT precompute
    (ICGN2D_CPU::ICGN2D_Algorithm).  Returns seconds."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    u, v, z, st = O.fftcc(pair.ref, pair.tar, poi, g.subset_r, nthreads=nthreads)
    O.icgn(pair.ref, pair.tar, g, poi, u, v, nthreads=nthreads)
    return time.perf_counter() - t0


def run_reference(args, world, rank):
    """Whole frames of the workload on the host cores, timed one per step
    (warm-up steps are bounded samples of 2000 POIs)."""
    if rank != 0:
        return 0
    pair, g = workload()
    from oracle import oracle as O
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    P = len(poi)
    for _ in range(args.warmup):
        cpu_frame(pair, g, poi[:2000])
    t_wall0 = time.perf_counter()
    secs = [cpu_frame(pair, g, poi) for _ in range(args.steps)]
    t_wall = time.perf_counter() - t_wall0
    value = P * len(secs) / sum(secs)
    lat = [1000.0 * x for x in secs]
    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sum(lat) / len(lat), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": config_of(P, 1),
            "frame_latency_ms": {"p50": round(pct(lat, 50), 1), "p99": round(pct(lat, 99), 1)},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                             "sample": f"whole frames of {P} POIs (FFT-CC + IC-GN with the per-call whole-ROI "
                                       f"gradient/LUT precompute), one per step; {sum(secs):.1f} s over "
                                       f"{args.steps} steps; OpenMP over POIs"},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0,
            "wall_s_timed_region": round(t_wall, 3)}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------- GPU legs ----
def time_frames(fr, tar_dev, outs, steps, warmup, flush, torch, clocks=None):
    """Device-timed frames with device-resident inputs; L2 flushed between
    frames outside the timed events."""
    for i in range(warmup):
        flush.fill_(i)
        fr.process(tar_dev, **outs)
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.mark_start()
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    phases = []
    for i in range(steps):
        flush.fill_(i)
        evs[i][0].record(stream)
        fr.process(tar_dev, **outs)
        evs[i][1].record(stream)
        phases.append(fr.phase_times())
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.mark_stop()
    ms = [a.elapsed_time(b) for a, b in evs]
    return ms, phases


def time_e2e(fr, tar_host, outs_host, steps, warmup, flush, torch):
    for i in range(warmup):
        flush.fill_(i)
        torch.cuda.synchronize()
        fr.process(tar_host, **outs_host)
    ms = []
    for i in range(steps):
        flush.fill_(i)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fr.process(tar_host, **outs_host)  # synchronous: host outputs
        ms.append(1000.0 * (time.perf_counter() - t0))
    return ms


def pct(xs, q):
    s = sorted(xs)
    return s[min(len(s) - 1, int(round(q / 100.0 * (len(s) - 1))))]


def run_gpu(args, world, rank, local):
    import torch
    from tw_gb300.build import build
    build()
    torch.cuda.set_device(local)
    # every launch of the run (L2 flush, frames, CUDA events) goes to one
    # non-default stream that the DIC handles are bound to
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        return _run_gpu(args, world, rank, local, torch)


def _run_gpu(args, world, rank, local, torch):
    from tw_gb300 import PATH_FAST, PATH_PLAIN, dic
    pair, g = workload()
    P = None
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    tar_dev = torch.from_numpy(pair.tar).cuda()
    ref_dev = torch.from_numpy(pair.ref).cuda()

    fr = dic.DICFrame(params_of(g, PATH_FAST))
    P = fr.n
    fr.set_stream(torch.cuda.current_stream())
    fr.set_reference(ref_dev)
    outs = fr.alloc_outputs(device="cuda")

    dist_barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t_wall0 = time.perf_counter()
    ms, phases = time_frames(fr, tar_dev, outs, args.steps, args.warmup, flush, torch, clocks)
    t_wall = time.perf_counter() - t_wall0
    torch.cuda.synchronize()
    dist_barrier(world)
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(ms), world)
    value = P * args.steps * world / (total_ms / 1000.0)

    # end-to-end through the public API with pinned host buffers
    tar_pin = torch.from_numpy(pair.tar).pin_memory()
    outs_h = {k: torch.from_numpy(v).pin_memory() for k, v in fr.alloc_outputs().items()}
    e2e_ms = time_e2e(fr, tar_pin, outs_h, args.steps, args.warmup, flush, torch)
    e2e_total = max_over_ranks(sum(e2e_ms), world)
    e2e_value = P * args.steps * world / (e2e_total / 1000.0)
    d2h = sum(int(v.numel() * v.element_size()) for v in outs_h.values())

    # accuracy of the last frame vs the imposed field
    from oracle import compare as C  # test infrastructure: truth error only
    p6 = outs["p6"].cpu().numpy()
    flags = outs["flags"].cpu().numpy()
    iters_np = outs["iters"].cpu().numpy()
    iters = outs["iters"].cpu().numpy()
    poi = fr.poi_positions()
    acc = C.truth_error(pair, poi, p6, flags)
    kbar = float(iters[flags == 0].mean())

    # roofline of the dominant phase
    ph = {k: statistics.mean(p[k] for p in phases) for k in phases[0]}
    roof = roofline(g, P, ph, kbar)

    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (IC-GN), fp16 tensor core / fp32 (FFT-CC), "
                                                            "fp64 (6x6 solve)", "data": "synthetic",
            "config": config_of(P, world),
            "path": "fast (tensor-core FFT-CC, one-POI-per-warp IC-GN on the neighbourhood table)",
            "frame_latency_ms": {"p50": round(pct(ms, 50), 4), "p99": round(pct(ms, 99), 4)},
            "phases_ms": {k: round(v, 4) for k, v in ph.items()},
            "accuracy": {"vs_imposed_field": acc, "mean_iterations": round(kbar, 3),
                         "success_fraction": float((flags == 0).mean())},
            "roofline": roof,
            "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": int(pair.tar.nbytes),
                    "d2h_bytes_per_step": d2h, "p50_ms": round(pct(e2e_ms, 50), 4),
                    "p99_ms": round(pct(e2e_ms, 99), 4)},
            # per frame: k_fftcc_tc, k_nbhd_table, k_icgn_warp
            "gpu_launches": 3 * args.steps,
            "clocks": clk,
            "wall_s_timed_region": round(t_wall, 3)}
    if not args.no_plain:
        # plain FP32 GPU path, same workload, same timing rules
        frp = dic.DICFrame(params_of(g, PATH_PLAIN))
        frp.set_stream(torch.cuda.current_stream())
        frp.set_reference(ref_dev)
        outs_p = frp.alloc_outputs(device="cuda")
        psteps = max(3, min(args.steps, 10))
        ms_p, phases_p = time_frames(frp, tar_dev, outs_p, psteps, min(args.warmup, 3), flush, torch)
        plain_value = P * psteps / (sum(ms_p) / 1000.0)
        php = {k: statistics.mean(p[k] for p in phases_p) for k in phases_p[0]}
        del frp, outs_p
        torch.cuda.empty_cache()
        line["plain_fp32"] = {"value": round(plain_value, 1), "ms_per_step": round(sum(ms_p) / psteps, 4),
                              "p50_ms": round(pct(ms_p, 50), 4), "p99_ms": round(pct(ms_p, 99), 4),
                              "phases_ms": {k: round(v, 4) for k, v in php.items()}}
        line["speedup_vs_plain_fp32"] = round(value / (plain_value * world), 3)
        # the same ratio per phase: FFT-CC (tensor-core DFT GEMMs against a
        # direct FP32 DFT), target table (neighbourhood table against the
        # float LUT), IC-GN
        line["speedup_vs_plain_fp32_by_phase"] = {k: round(php[k] / ph[k], 3) for k in ("fftcc", "prepare", "icgn")
                                                  if ph.get(k, 0) > 0}
    if rank == 0 and not args.no_serving:
        # serving (12 camera streams, Poisson arrivals) and batched uneven
        # pairs, each on its own synthetic data generated before its run
        from tw_gb300.batch_bench import run_batched
        from tw_gb300.serve_bench import make_streams, run_serving
        sdata = make_streams()
        line["serving"] = run_serving(seconds=4.0, data=sdata)
        # the same streams at twice the arrival rates (the GPU near saturation:
        # frames queue, batches form, lanes overlap) and at four times (overload:
        # the queues fill and frames are dropped)
        line["serving_saturation"] = run_serving(seconds=4.0, data=sdata, load=2.0)
        line["serving_overload"] = run_serving(seconds=4.0, data=sdata, load=4.0)
        line["batched"] = run_batched(pairs=48, steps=3)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O  # noqa: F401  (CPU baseline leg)
        # the integer FFT-CC of the same frame (one more call, outside the
        # timed regions), for the accuracy block's FFT-CC comparison
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r,
                          g.grid, g.grid, g.margin, g.margin, path=PATH_FAST)
        U, V, Z = f.InitializeFFTCC(pair.ref)
        f.ComputeFFTCC(U, V, Z, pair.tar)
        gpu_out = {"p6": p6, "iters": iters_np, "flags": flags, "u_int": U.ravel(), "v_int": V.ravel(),
                   "zncc": Z.ravel()}
        line["cpu_baseline"] = cpu_baseline(pair, g, poi, gpu_out=gpu_out)
    if rank == 0:
        print(json.dumps(line))
    return 0


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
# of each kernel on this workload, from the ncu captures summarised in
# profiles/k_icgn_warp_2048_subset41.md and profiles/k_fftcc_tc_2048_subset41.md
NCU_TRAFFIC = {"k_icgn_warp": 139.83e6 + 7.27e6, "k_fftcc_tc": 532.76e6 + 5.50e6}
# from the same IC-GN capture: L1 hit rate of its gathers and the FMA-heavy
# pipe's share of cycles (the kernel's limiter)
NCU_ICGN_L1_HIT = 0.933
NCU_ICGN_FMAHEAVY = 0.667


def fp32_peak(peaks):
    """FP32 SIMT peak: SMs x 128 FP32 lanes x 2 flops (FMA) x the measured
    maximum SM clock.  Derived, not measured: MEASURED_PEAKS.json has no FP32
    figure.  Returns (flops/s, description)."""
    sms = 152
    try:
        import torch
        if torch.cuda.is_available():
            sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    sm_mhz = peaks.get("sm_max_mhz", 2070.0)
    return sms * 128 * 2 * sm_mhz * 1e6, f"derived: {sms} SMs x 128 FP32 lanes x 2 flops x {sm_mhz:.0f} MHz"


def roofline(g, P, ph, kbar):
    """Roofline of the dominant kernel, the fast IC-GN (k_icgn_warp), timed by
    the per-phase CUDA events of the frame.

    Binding view (bound / achieved / peak / frac): FP32.  The kernel is
    limited by the SM's FP32 and integer pipes (ncu: FMA-heavy pipe busy 67 %
    of cycles, 77 % issue) with its gathers served by L1 (93 % hits); the
    credited work is k*S*64 flops per POI (k = mean iterations, S = subset
    pixels; 64 flops per sample and iteration: warp 8, bicubic Horner 30,
    mean/norm 6, residual 4, right-hand side 12, address 4), against the
    derived FP32 peak.

    Secondary views: HBM (the compulsory bytes per launch: the target's 4x4
    neighbourhood table read once, 16 B per ROI pixel; the per-reference
    gradient image, float2, 8 B per ROI pixel; the target image; per POI the
    reference cache entry -- statistics 64 B, FP64 inverse Hessian 168 B, flag
    1 B -- the POI 8 B, u/v in 8 B and out 8 B, p6 24 B, iteration count 4 B
    and flag 1 B; the subset sample table, 16 B per subset pixel); gathers
    (k*S*40 B per POI through L1/L2: table entry, gradient and sample-table
    entry of every sample); and the tensor view of the FFT-CC kernel
    (48 N^3 flops per POI) with its own HBM bytes (per POI the cached
    reference spectrum, N/2 + 1 rows of N rounded up to 4 FP16 pairs, and the
    reference window sums 8 B, the POI 8 B, u, v, ZNCC 12 B and status 1 B;
    both images once)."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    tc = peaks.get("bf16_tflops", 1900.0)
    src = "measured" if peaks else "fallback"
    fp32, fp32_src = fp32_peak(peaks)
    S = (2 * g.subset_r + 1) ** 2
    N = 2 * g.subset_r
    t_icgn = ph["icgn"] / 1000.0
    t_fftcc = ph["fftcc"] / 1000.0
    per_poi = 64 + 168 + 1 + 8 + 8 + 8 + 24 + 4 + 1
    bytes_icgn = P * per_poi + (16 + 8) * g.roi_w * g.roi_h + g.img_w * g.img_h + 16 * S
    flops_icgn = kbar * S * 64 * P
    achieved = flops_icgn / t_icgn / 1e12
    gather = kbar * S * 40 * P  # per sample: table entry 16 B, gradient 8 B, sample-table entry 16 B
    flops_fftcc = 48 * N ** 3 * P
    fft_tflops = flops_fftcc / t_fftcc / 1e12
    bytes_fftcc = fftcc_bytes(g, P)
    return {"kernel": "k_icgn_warp (IC-GN)", "bound": "fp32", "achieved": round(achieved, 3),
            "peak": round(fp32 / 1e12, 2), "unit": "TFLOP/s", "frac": round(achieved * 1e12 / fp32, 4),
            "traffic": NCU_TRAFFIC["k_icgn_warp"], "peak_source": fp32_src,
            "flops_per_launch": int(flops_icgn), "kernel_ms": round(ph["icgn"], 4),
            "ncu": {"fmaheavy_pipe_busy": NCU_ICGN_FMAHEAVY, "l1_hit_rate": NCU_ICGN_L1_HIT},
            "hbm_view": {"algorithmic_bytes_per_launch": int(bytes_icgn),
                         "achieved_gbs": round(bytes_icgn / t_icgn / 1e9, 2), "peak_gbs": hbm,
                         "frac": round(bytes_icgn / t_icgn / 1e9 / hbm, 5), "traffic": NCU_TRAFFIC["k_icgn_warp"],
                         "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs, burst)"},
            "gather_view": {"gather_bytes_per_launch": int(gather), "achieved_gbs": round(gather / t_icgn / 1e9, 1),
                            "l1_hit_rate_ncu": NCU_ICGN_L1_HIT},
            "fftcc_tensor_view": {"kernel": "k_fftcc_tc", "flops_per_launch": int(flops_fftcc),
                                  "achieved_tflops": round(fft_tflops, 2), "peak_tflops": tc,
                                  "frac": round(fft_tflops / tc, 4), "kernel_ms": round(ph["fftcc"], 4),
                                  "traffic": NCU_TRAFFIC["k_fftcc_tc"],
                                  "peak_source": f"{src} (MEASURED_PEAKS.json bf16_tflops, burst)",
                                  "hbm_bytes_per_launch": int(bytes_fftcc),
                                  "hbm_achieved_gbs": round(bytes_fftcc / t_fftcc / 1e9, 1),
                                  "hbm_frac": round(bytes_fftcc / t_fftcc / 1e9 / hbm, 4)},
            "frame_roofline": frame_roofline(g, P, ph, kbar, peaks, bytes_icgn + bytes_fftcc)}


def fftcc_bytes(g, P):
    """Algorithmic HBM bytes of one per-frame FFT-CC launch: per POI the
    cached reference spectrum and window sums, the POI and the outputs; both
    images once."""
    N = 2 * g.subset_r
    spectrum = (N // 2 + 1) * ((N + 3) // 4 * 4) * 4
    return P * (spectrum + 8 + 8 + 12 + 1) + 2 * g.img_w * g.img_h


def frame_roofline(g, P, ph, kbar, peaks, bytes_icgn):
    """Frame-level bound T_roof = P F_a / Peak_TC + max(P F_c / Peak_FP32,
    B_compulsory / Peak_HBM) with F_a = 48 N^3 (FFT-CC, credited flops only)
    and F_c = k S 64 (IC-GN); achieved = T_roof / T_measured.  B_compulsory is
    this design's: both images, the neighbourhood table and gradient image,
    the per-POI caches (IC-GN statistics and inverse Hessian, FFT-CC
    reference spectra) and the outputs.  (A 64 B/px coefficient LUT and S*28 B
    of per-POI reference data, the reference's layout, are never moved here,
    so they are not in the bound.)  Peak_FP32 is not in MEASURED_PEAKS.json:
    it is 128 FP32 lanes x 2 flops per SM and clock at the measured maximum SM
    clock."""
    N = 2 * g.subset_r
    S = (2 * g.subset_r + 1) ** 2
    peak_tc = peaks.get("bf16_tflops", 1900.0) * 1e12
    peak_fp32, fp32_src = fp32_peak(peaks)
    peak_hbm = peaks.get("hbm_gbs", 6800.0) * 1e9
    t_tc = P * 48 * N ** 3 / peak_tc
    t_fp32 = P * kbar * S * 64 / peak_fp32
    b_comp = bytes_icgn  # IC-GN's and FFT-CC's bytes
    t_hbm = b_comp / peak_hbm
    t_roof = t_tc + max(t_fp32, t_hbm)
    t_meas = (ph["fftcc"] + ph["prepare"] + ph["icgn"]) / 1000.0
    return {"t_roof_ms": round(t_roof * 1e3, 4), "t_measured_ms": round(t_meas * 1e3, 4),
            "achieved": round(t_roof / t_meas, 4),
            "terms_ms": {"fftcc_tensor": round(t_tc * 1e3, 4), "icgn_fp32": round(t_fp32 * 1e3, 4),
                         "hbm_compulsory": round(t_hbm * 1e3, 4)},
            "peaks": {"tensor_tflops": peak_tc / 1e12, "fp32_tflops": round(peak_fp32 / 1e12, 1),
                      "hbm_gbs": peak_hbm / 1e9,
                      "fp32_source": fp32_src}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving and batched legs")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparator leg")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    else:
        rc = run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
