"""Batched benchmark: image pairs and POI sets of uneven sizes through one
batched call (twdic_batch_*), replayed as a CUDA graph, against the same
frames processed one call each.

    python -m tw_gb300.batch_bench [--pairs 48] [--steps 5]

Workload: `pairs` image pairs with sizes drawn from {512x384, 1024x768,
1280x1024, 2048x1536, 4096x3072}, subset radius r ~ U[10, 30] and POI step
~ U[3, 12], margin 20, all seeded.  Pairs of one size share their image
content (one synthetic reference/target per size: strain ramp plus drift).
Prints one JSON line with POIs/s of the batched graph replay and of the
one-call-per-frame loop (device-resident inputs and outputs, CUDA events), the
batched call's per-phase device times and the roofline fractions of its
FFT-CC and IC-GN phases."""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SIZES = [(512, 384), (1024, 768), (1280, 1024), (2048, 1536), (4096, 3072)]


def run_batched(pairs=48, steps=5, warmup=3, seed=3, data=None):
    import numpy as np
    import torch
    from tw_gb300 import dic, synth

    rng = np.random.default_rng(seed)
    if data is None:
        data = {sz: synth.camera_sequence(sz[0], sz[1], frames=1, seed=seed + i) for i, sz in enumerate(SIZES)}
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        frames, tars, outs, jobs = [], [], [], []
        for _ in range(pairs):
            sz = SIZES[int(rng.integers(0, len(SIZES)))]
            r = int(rng.integers(10, 31))
            step = int(rng.integers(3, 13))
            ref, ts, g = data[sz]
            p = dic.make_params(g.img_w, g.img_h, 1, 1, g.img_w - 2, g.img_h - 2, r, r, step, step, 20, 20)
            f = dic.DICFrame(p)
            f.set_stream(stream)
            f.set_reference(torch.from_numpy(ref).cuda())
            frames.append(f)
            tars.append(torch.from_numpy(ts[0]).cuda())
            outs.append(f.alloc_outputs(device="cuda"))
            jobs.append(dict(size=f"{sz[0]}x{sz[1]}", r=r, step=step, pois=f.n))
        total = sum(j["pois"] for j in jobs)
        b = dic.DICBatch(graph=True)
        b.set_stream(stream)

        def timed(fn, n):
            evs = []
            for _ in range(n):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                evs.append((e0, e1))
            torch.cuda.synchronize()
            return [a.elapsed_time(c) for a, c in evs]

        for _ in range(warmup):
            b.process(frames, tars, outs)
        ms_batch = timed(lambda: b.process(frames, tars, outs), steps)
        replayed = b.replayed

        def one_by_one():
            for f, t, o in zip(frames, tars, outs):
                f.process(t, **o)

        for _ in range(warmup):
            one_by_one()
        ms_loop = timed(one_by_one, steps)
        # per-phase device times of the batched call, from calls run without
        # a graph (the same launches), and the mean IC-GN iterations per frame
        eager = dic.DICBatch(graph=False)
        eager.set_stream(stream)
        phases = []
        for _ in range(steps):
            eager.process(frames, tars, outs)
            phases.append(eager.phase_times())
        kbar = []
        for o in outs:
            fl = o["flags"].cpu().numpy()
            it = o["iters"].cpu().numpy()
            kbar.append(float(it[fl == 0].mean()) if (fl == 0).any() else 0.0)
    ph = {k: float(np.median([p[k] for p in phases])) for k in phases[0]}
    flops_fft = sum(j["pois"] * 48.0 * (2 * j["r"]) ** 3 for j in jobs)
    flops_icgn = sum(j["pois"] * k * (2 * j["r"] + 1) ** 2 * 64.0 for j, k in zip(jobs, kbar))
    peaks = _peaks()
    sizes = {}
    for j in jobs:
        sizes[j["size"]] = sizes.get(j["size"], 0) + 1
    return {"workload": f"{pairs} pairs, sizes {sizes}, r ~ U[10, 30], step ~ U[3, 12], margin 20",
            "pois": total, "radii": len(set(j["r"] for j in jobs)),
            "batched": {"ms": round(float(np.median(ms_batch)), 3),
                        "pois_per_s": round(total / (float(np.median(ms_batch)) / 1000.0), 1),
                        "graph_replay": bool(replayed)},
            "one_call_per_frame": {"ms": round(float(np.median(ms_loop)), 3),
                                   "pois_per_s": round(total / (float(np.median(ms_loop)) / 1000.0), 1)},
            "kernel_launches": "preparation (every frame's table and zeroed outputs), tensor-core FFT-CC (every "
                               "window size), IC-GN (every frame): 3",
            "phases_ms": {k: round(v, 3) for k, v in ph.items()},
            "roofline": {"fftcc": {"flops": flops_fft,
                                   "achieved_tflops": round(flops_fft / (ph["fftcc"] / 1e3) / 1e12, 1),
                                   "peak_tflops": peaks["tensor"], "frac": round(
                                       flops_fft / (ph["fftcc"] / 1e3) / 1e12 / peaks["tensor"], 4),
                                   "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)"},
                         "icgn": {"flops": flops_icgn,
                                  "achieved_tflops": round(flops_icgn / (ph["icgn"] / 1e3) / 1e12, 1),
                                  "peak_tflops": peaks["fp32"], "frac": round(
                                      flops_icgn / (ph["icgn"] / 1e3) / 1e12 / peaks["fp32"], 4),
                                  "peak_source": "derived: SMs x 128 FP32 lanes x 2 flops x max SM clock"},
                         "note": "48 N^3 flops per POI for FFT-CC (N = 2r), k S 64 for IC-GN (k the frame's mean "
                                 "iterations, S = (2r + 1)^2)"}}


def _peaks():
    """Tensor (bf16 burst) and FP32 peaks in TFLOP/s: MEASURED_PEAKS.json where
    present, else the fallback figures; FP32 is derived from the SM count and
    the maximum SM clock."""
    import torch
    tensor, mhz = 1900.0, 2070.0
    try:
        m = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        tensor, mhz = m.get("bf16_tflops", tensor), m.get("sm_max_mhz", mhz)
    except Exception:
        pass
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return {"tensor": tensor, "fp32": round(sms * 128 * 2 * mhz * 1e6 / 1e12, 2)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=48)
    ap.add_argument("--steps", type=int, default=5)
    args = ap.parse_args(argv)
    from tw_gb300.build import build
    build()
    print(json.dumps(run_batched(args.pairs, args.steps)))


if __name__ == "__main__":
    main()
