"""Generate tests/golden/small_case.npz: a seeded synthetic speckle pair, its POI
grid and the oracle's FFT-CC and IC-GN outputs on it; and
tests/golden/small_case_bspline.npz: the oracle's IC-GN outputs on the same
inputs with the B-spline interpolation (BicubicSplineCoefficients_s).

This fixture is a regression record of the oracle itself: tests/test_oracle.py
re-runs the oracle on the stored inputs and requires the stored outputs.  The
oracle's pin to the reference's own code is a separate set of fixtures
(make_ref_golden.py, tests/test_ref_pin.py).  Re-run this script only when the
oracle's arithmetic is changed on purpose.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tw_gb300 import synth  # noqa: E402


def main():
    pair, g = synth.small_case()
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u, v, z, st = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    p6, it, fl = O.icgn(pair.ref, pair.tar, g, poi, u, v)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_case.npz")
    geom = np.array([g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin,
                     g.max_iter], np.int32)
    np.savez_compressed(out, ref=pair.ref, tar=pair.tar, poi=poi, geom=geom, delta_p=np.float32(g.delta_p),
                        fftcc_u=u, fftcc_v=v, fftcc_zncc=z, icgn_p6=p6, icgn_iters=it, icgn_flags=fl)
    print(out, os.path.getsize(out), "bytes;", len(poi), "POIs; flags", np.bincount(fl))
    bp6, bit, bfl = O.icgn(pair.ref, pair.tar, g, poi, u, v, interp="bspline")
    out_b = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_case_bspline.npz")
    np.savez_compressed(out_b, icgn_p6=bp6, icgn_iters=bit, icgn_flags=bfl)
    print(out_b, os.path.getsize(out_b), "bytes; flags", np.bincount(bfl))


if __name__ == "__main__":
    main()
