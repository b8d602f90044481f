"""Run a few frames of the 2048x2048 / 41x41-subset workload for profilers.

    python -m tw_gb300.profile_frame [--frames 3] [--path fast|plain]
        [--icgn THREADS:SAMPLER:CHUNK] [--interp bicubic|bspline]

Sets the reference once (per-reference precompute), then processes `frames`
target frames with device-resident buffers and prints the phase times of the
last one.  Small launch count and device footprint (fast path: under 0.1 GB),
so an ncu capture of one launch ends quickly.
"""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main(argv=None):
    import torch
    from tw_gb300 import INTERP_BICUBIC, INTERP_BSPLINE, PATH_FAST, PATH_PLAIN, dic, synth

    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--path", default="fast", choices=["fast", "plain"])
    ap.add_argument("--workload", default="2048", choices=["2048", "512"])
    ap.add_argument("--icgn", default=None, help="IC-GN launch shape threads:sampler:chunk (default: the frame's)")
    ap.add_argument("--interp", default="bicubic", choices=["bicubic", "bspline"], help="IC-GN interpolation")
    args = ap.parse_args(argv)
    pair, g = synth.scale_2048() if args.workload == "2048" else synth.plain_512()
    path = PATH_FAST if args.path == "fast" else PATH_PLAIN
    prm = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                          g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, path)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        fr = dic.DICFrame(prm)
        fr.set_stream(s)
        fr.set_interpolation(INTERP_BSPLINE if args.interp == "bspline" else INTERP_BICUBIC)
        if args.icgn:
            th, sa, ch = (int(x) for x in args.icgn.split(":"))
            fr.set_tuning(th, 0, sa, 1)
            fr.set_icgn_layout(ch)
        fr.set_reference(torch.from_numpy(pair.ref).cuda())
        tar = torch.from_numpy(pair.tar).cuda()
        outs = fr.alloc_outputs("cuda")
        for _ in range(args.frames):
            fr.process(tar, **outs)
        torch.cuda.synchronize()
        print(json.dumps({"pois": fr.n, "path": args.path, "interp": args.interp, "phases_ms": fr.phase_times()}))


if __name__ == "__main__":
    main()
