"""Serving benchmark: simulated camera streams of several resolutions with
Poisson frame arrivals, through the native server (twdic_server_*).

    python -m tw_gb300.serve_bench [--seconds 4] [--lanes 2] [--max-batch 32]

Default workload: 12 streams -- 4 x 640x480, 4 x 1280x1024, 4 x 2048x2048 --
31x31 subsets (r = 15) at step 8, margin 20; each stream's arrival rate is
drawn from U[30, 120] frames/s; every stream cycles through three synthetic
targets (strain ramp to 1 % plus 0.5 px/frame drift).  Streams of one
resolution share their image content.  Prints one JSON line: per resolution
the submit-to-result latency p50/p99 (ms), frames done and dropped, and the
whole-server throughput in POIs/s and frames/s."""
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


def run_serving(seconds=4.0, streams_per_res=4, lanes=2, max_batch=32, queue_depth=4, seed=5, data=None,
                use_graph=True, guesses=False):
    """guesses: every stream starts each frame's IC-GN from its last
    displacements (twdic_server_set_stream_guess) instead of FFT-CC."""
    import numpy as np
    from tw_gb300 import dic, synth
    from tw_gb300.serve import DICServer

    if data is None:
        data = {res: synth.camera_sequence(res[0], res[1], frames=3, seed=seed + i)
                for i, res in enumerate(RESOLUTIONS)}
    rng = np.random.default_rng(seed)
    srv = DICServer(max_batch=max_batch, queue_depth=queue_depth, lanes=lanes, use_graph=use_graph)
    streams = []
    for res in RESOLUTIONS:
        ref, tars, g = data[res]
        p = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                            g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p)
        nx, ny = dic.num_pois(p)
        for _ in range(streams_per_res):
            sid = srv.add_stream(p)
            if guesses:
                srv.set_stream_guess(sid, 1)
            srv.set_reference(sid, ref)
            streams.append(dict(sid=sid, res=res, tars=tars, n=nx * ny, fps=float(rng.uniform(30, 120))))
    # warm-up: one frame per stream (reference precompute, first tables)
    for s in streams:
        srv.poll(s["sid"], srv.submit(s["sid"], s["tars"][0]))
    base = srv.stats()
    # Poisson arrivals, merged over streams
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
                       + "; 31x31 subsets (r = 15), step 8, margin 20; Poisson arrivals, rates U[30, 120] fps",
           "seconds": round(wall, 3), "lanes": lanes, "max_batch": max_batch, "queue_depth": queue_depth,
           "graph": use_graph, "initial_guesses": "last frame" if guesses else "FFT-CC", "per_resolution": {}}
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
    out["graph_replays"] = st["graph_replays"] - base["graph_replays"]
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=4.0)
    ap.add_argument("--lanes", type=int, default=2)
    ap.add_argument("--max-batch", type=int, default=32)
    ap.add_argument("--queue-depth", type=int, default=4)
    ap.add_argument("--no-graph", action="store_true")
    args = ap.parse_args(argv)
    from tw_gb300.build import build
    build()
    print(json.dumps(run_serving(args.seconds, lanes=args.lanes, max_batch=args.max_batch,
                                 queue_depth=args.queue_depth, use_graph=not args.no_graph)))


if __name__ == "__main__":
    main()
