"""Serving benchmark: simulated camera streams of several resolutions with
Poisson frame arrivals, through the native server (twdic_server_*).

    python -m tw_gb300.serve_bench [--seconds 4] [--lanes 4] [--max-batch 32] [--load 1]

Default workload: 12 streams -- 4 x 640x480, 4 x 1280x1024, 4 x 2048x2048 --
31x31 subsets (r = 15) at step 8, margin 20; each stream's arrival rate is
drawn from U[30, 120] frames/s times the load factor.  Every stream has its own
speckle content (a per-stream circular shift of one speckle field per
resolution) and its own evolving deformation over a 300-frame sequence: a
linear ramp to 1 % strain plus a rigid drift that oscillates with a speed of
at most 0.5 px/frame; 20 frames sampled evenly from that sequence are
rendered per stream (bicubic warp on the GPU) and submitted in turn.  Prints
one JSON line per run: per resolution the submit-to-result latency p50/p99
(ms), frames done and dropped, the whole-server throughput in POIs/s and
frames/s, and the batching and device-overlap counters of the server."""
import argparse
import json
import os
import sys
import threading
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RESOLUTIONS = [(640, 480), (1280, 1024), (2048, 2048)]


SEQUENCE = 300  # frames of each stream's deformation history
FRAMES = 20     # frames rendered per stream, evenly spaced in the sequence


def _render_stream(intensity, shift, frames, seed, phase):
    """One stream: the speckle field rolled by `shift` (its own content), the
    reference and `frames` targets sampled evenly from a SEQUENCE-frame
    history (strain ramp to 1 %, oscillating drift of at most 0.5 px/frame),
    rendered by a Catmull-Rom warp on the GPU with noise sigma 2."""
    import numpy as np
    import torch
    h, w = intensity.shape
    dev = "cuda"
    img = torch.from_numpy(np.roll(intensity, shift, axis=(0, 1)).astype(np.float32)).to(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    ref = torch.clamp(torch.round(img), 0, 255).to(torch.uint8).cpu().numpy()
    yp, xp = torch.meshgrid(torch.arange(h, device=dev, dtype=torch.float32),
                            torch.arange(w, device=dev, dtype=torch.float32), indexing="ij")
    cx, cy = w / 2.0, h / 2.0
    amp, period = 8.0, 2.0 * np.pi * 8.0 / 0.5  # drift amplitude 8 px, speed at most 0.5 px/frame

    def cr(t):
        t2, t3 = t * t, t * t * t
        return (-0.5 * t3 + t2 - 0.5 * t, 1.5 * t3 - 2.5 * t2 + 1.0, -1.5 * t3 + 2.0 * t2 + 0.5 * t,
                0.5 * t3 - 0.5 * t2)

    tars = []
    for i in range(frames):
        k = (i + 1) * SEQUENCE // frames
        s = 0.01 * k / SEQUENCE
        u0 = amp * np.sin(2 * np.pi * k / period + phase)
        v0 = -0.7 * amp * np.sin(2 * np.pi * k / period + 2 * phase)
        # inverse of the affine map X + u(X) = x'
        X = cx + (xp - cx - u0) / (1.0 + s)
        Y = cy + (yp - cy - v0) / (1.0 - 0.6 * s)
        x0, y0 = torch.floor(X), torch.floor(Y)
        wx, wy = cr(X - x0), cr(Y - y0)
        x0, y0 = x0.long(), y0.long()
        acc = torch.zeros_like(X)
        for a in range(4):
            yy = torch.clamp(y0 + a - 1, 0, h - 1)
            row = torch.zeros_like(X)
            for b in range(4):
                xx = torch.clamp(x0 + b - 1, 0, w - 1)
                row += wx[b] * img[yy, xx]
            acc += wy[a] * row
        acc += 2.0 * torch.randn(acc.shape, generator=gen, device=dev)
        tars.append(torch.clamp(torch.round(acc), 0, 255).to(torch.uint8).cpu().numpy())
    return ref, tars


def make_streams(streams_per_res=4, seed=5, frames=FRAMES):
    """Per resolution: the geometry and, per stream, (reference, targets)."""
    import numpy as np
    from tw_gb300 import synth
    data = {}
    rng = np.random.default_rng(seed)
    for i, (w, h) in enumerate(RESOLUTIONS):
        field = synth.speckle_intensity(h, w, int(6000 * h * w / (512 * 512)), np.random.default_rng(seed + i))
        g = synth.Geometry(w, h, 1, 1, w - 2, h - 2, 15, 8, 20)
        per = []
        for j in range(streams_per_res):
            shift = (int(rng.integers(h // 8, h - h // 8)), int(rng.integers(w // 8, w - w // 8)))
            per.append(_render_stream(field, shift, frames, seed * 100 + 10 * i + j, float(rng.uniform(0, 6.28))))
        data[(w, h)] = (g, per)
    return data


def run_serving(seconds=4.0, streams_per_res=4, lanes=4, max_batch=32, queue_depth=4, seed=5, data=None,
                use_graph=True, guesses=False, load=1.0, mix_sizes=False):
    """guesses: every stream starts each frame's IC-GN from its last
    displacements (twdic_server_set_stream_guess) instead of FFT-CC.
    load: factor on every stream's arrival rate."""
    import numpy as np
    from tw_gb300 import dic
    from tw_gb300.serve import DICServer

    if data is None:
        data = make_streams(streams_per_res, seed)
    rng = np.random.default_rng(seed)
    srv = DICServer(max_batch=max_batch, queue_depth=queue_depth, lanes=lanes, use_graph=use_graph,
                    mix_sizes=mix_sizes)
    streams = []
    for res in RESOLUTIONS:
        g, per = data[res]
        p = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                            g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p)
        nx, ny = dic.num_pois(p)
        for ref, tars in per[:streams_per_res]:
            sid = srv.add_stream(p)
            if guesses:
                srv.set_stream_guess(sid, 1)
            srv.set_reference(sid, ref)
            streams.append(dict(sid=sid, res=res, tars=tars, n=nx * ny, fps=load * float(rng.uniform(30, 120))))
    # warm-up: one frame per stream (reference precompute, first tables)
    for s in streams:
        srv.poll(s["sid"], srv.submit(s["sid"], s["tars"][0]))
    base = srv.stats()
    # Poisson arrivals, merged over streams; a stream's k-th frame is its
    # (k mod FRAMES)-th rendered target
    events = []
    for s in streams:
        t = float(rng.exponential(1.0 / s["fps"]))
        k = 0
        while t < seconds:
            events.append((t, s, k))
            t += float(rng.exponential(1.0 / s["fps"]))
            k += 1
    events.sort(key=lambda e: e[0])
    pending = []
    lock = threading.Condition()
    results = []
    done_submitting = [False]

    def poller():
        while True:
            with lock:
                while not pending and not done_submitting[0]:
                    lock.wait()
                if not pending and done_submitting[0]:
                    return
                s, t = pending.pop(0)
            out = srv.poll(s["sid"], t)
            results.append((s, out["latency_ms"]))

    th = threading.Thread(target=poller)
    th.start()
    t0 = time.perf_counter()
    dropped = {res: 0 for res in RESOLUTIONS}
    for when, s, k in events:
        delay = t0 + when - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        t = srv.submit(s["sid"], s["tars"][k % len(s["tars"])])
        if t is None:
            dropped[s["res"]] += 1
            continue
        with lock:
            pending.append((s, t))
            lock.notify()
    with lock:
        done_submitting[0] = True
        lock.notify()
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    out = {"workload": f"{len(streams)} streams: " + ", ".join(f"{streams_per_res} x {w}x{h}" for w, h in
                                                               RESOLUTIONS)
                       + f"; 31x31 subsets (r = 15), step 8, margin 20; Poisson arrivals, rates {load:g} x "
                         f"U[30, 120] fps; own content and {FRAMES} frames of a {SEQUENCE}-frame evolving "
                         f"deformation per stream",
           "load": load, "offered_fps": round(sum(s["fps"] for s in streams), 1),
           "seconds": round(wall, 3), "lanes": lanes, "max_batch": max_batch, "queue_depth": queue_depth,
           "graph": use_graph, "batching": "any sizes" if mix_sizes else "sizes within 2x",
           "initial_guesses": "last frame" if guesses else "FFT-CC", "per_resolution": {}}
    pois = 0
    for res in RESOLUTIONS:
        lat = sorted(l for s, l in results if s["res"] == res)
        n_res = [s for s in streams if s["res"] == res][0]["n"]
        pois += n_res * len(lat)
        q = (lambda f: lat[min(len(lat) - 1, int(round(f * (len(lat) - 1))))]) if lat else (lambda f: None)
        out["per_resolution"][f"{res[0]}x{res[1]}"] = {
            "pois_per_frame": n_res, "frames": len(lat), "dropped": dropped[res],
            "p50_ms": round(q(0.5), 3) if lat else None, "p99_ms": round(q(0.99), 3) if lat else None}
    out["pois_per_s"] = round(pois / wall, 1)
    out["frames_per_s"] = round(len(results) / wall, 1)
    out["batches"] = st["batches"] - base["batches"]
    out["mean_batch"] = round((st["batched_frames"] - base["batched_frames"]) / max(1, out["batches"]), 2)
    out["max_batch_formed"] = st["max_batch_formed"]
    out["graph_replays"] = st["graph_replays"] - base["graph_replays"]
    # device view (CUDA events on the lanes, warm-up included): busy time and
    # the time with two or more batches running at once
    busy = st["device_busy_ms"] - base["device_busy_ms"]
    out["device"] = {"busy_fraction": round(busy / (1000.0 * wall), 3),
                     "overlap_ms": round(st["device_overlap_ms"] - base["device_overlap_ms"], 2),
                     "overlap_fraction_of_busy": round((st["device_overlap_ms"] - base["device_overlap_ms"]) /
                                                       max(busy, 1e-9), 3),
                     "peak_batches_running": st["peak_device_batches"],
                     "peak_lanes_in_flight": st["peak_lanes_in_flight"]}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=4.0)
    ap.add_argument("--lanes", type=int, default=4)
    ap.add_argument("--max-batch", type=int, default=32)
    ap.add_argument("--queue-depth", type=int, default=4)
    ap.add_argument("--load", type=float, default=1.0, help="factor on every stream's arrival rate")
    ap.add_argument("--mix-sizes", action="store_true", help="batch frames of any size together")
    ap.add_argument("--no-graph", action="store_true")
    args = ap.parse_args(argv)
    from tw_gb300.build import build
    build()
    print(json.dumps(run_serving(args.seconds, lanes=args.lanes, max_batch=args.max_batch,
                                 queue_depth=args.queue_depth, use_graph=not args.no_graph, load=args.load,
                                 mix_sizes=args.mix_sizes)))


if __name__ == "__main__":
    main()
