"""Generate tests/golden/ref_<case>.npz: outputs of the REFERENCE'S OWN CPU
code (Fftcc2D_CPU and ICGN2D_CPU compiled from the reference sources by
oracle/build_ref.py, with FFTW / LAPACKE / OpenCV / Qt stand-ins) on seeded
synthetic inputs.  These fixtures pin both the oracle restatement
(tests/test_ref_pin.py) and the CUDA path (tests/test_gpu_parity.py) to the
reference's behaviour; they travel where the reference checkout does not.

Each file holds the input images (so no generator has to reproduce them
bit for bit elsewhere), the geometry, the POIs, the reference's FFT-CC
outputs where the case runs FFT-CC, the IC-GN guesses, and the reference's
IC-GN outputs (u, v, iteration counts and the per-POI flags that
ICGN2D_Compute returns) for bicubic and, where listed, B-spline
interpolation.  The reference's IC-GN keeps the displacement gradients in a
local variable (TW_paDIC_ICGN2D_CPU.cpp:499), so no gradient is stored.

    python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_ref as R  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tw_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def flags_case():
    """The small case with a zero (dark) reference patch and a patch of
    vertical stripes (R_y = 0, singular Hessian); POIs whose subsets stay in
    the ROI, with guesses that keep, or push outside the ROI, the warped
    subset."""
    pair, g = synth.small_case()
    ref = pair.ref.copy()
    r = g.subset_r
    ref[25:56, 135:166] = 0                       # dark around (40, 150)
    cols = np.arange(60 - r - 2, 60 + r + 3)      # stripes around (60, 60)
    ref[60 - r - 2:60 + r + 3, cols] = (37 * cols % 200 + 20).astype(np.uint8)[None, :]
    # Success; OutofROI in the first (integer) pass; DarkSubset; SingularHessian;
    # Success; OutofROI after the first solve moves the subset past the last
    # ROI column, and past the first ROI row; Success
    poi = np.array([[80, 96], [80, 96], [40, 150], [60, 60], [100, 120], [60, 180], [11, 100], [117, 60]],
                   np.int32)
    gu = np.array([1.6, 200.0, 1.6, 1.6, 1.6, 0.0, 1.6, 1.6], np.float32)
    gv = np.array([-2.4, 0.0, -2.4, -2.4, -2.4, -2.4, 0.0, -2.4], np.float32)
    return ref, pair.tar, g, poi, gu, gv


def grid_case(pair, g):
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    return O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)


def geom_array(g):
    return np.array([g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r,
                     getattr(g, "subset_ry", 0) or g.subset_r, g.grid, g.margin, g.max_iter], np.int32)


def save(name, ref, tar, g, poi, gu, gv, fft=None, interps=("bicubic",)):
    out = dict(ref=ref, tar=tar, geom=geom_array(g), delta_p=np.float32(g.delta_p), poi=poi, guess_u=gu,
               guess_v=gv)
    if fft is not None:
        out.update(fftcc_u=fft[0], fftcc_v=fft[1], fftcc_zncc=fft[2])
    for interp in interps:
        u, v, it, fl = R.icgn(ref, tar, g, poi, gu, gv, interp=interp)
        out.update({f"{interp}_u": u, f"{interp}_v": v, f"{interp}_iters": it, f"{interp}_flags": fl})
        print(f"  {interp}: flags {np.bincount(fl, minlength=5)}, mean iterations {it[fl == 0].mean():.3f}")
    path = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes;", len(poi), "POIs")


def main():
    R.build()
    # the stored small case (inputs of small_case.npz) and config 0 (512^2)
    for name, make in [("small", synth.small_case), ("plain512", synth.plain_512)]:
        pair, g = make()
        rp, u, v, z = R.fftcc(pair.ref, pair.tar, g)
        assert np.array_equal(rp, grid_case(pair, g))
        save(name, pair.ref, pair.tar, g, rp, u, v, fft=(u, v, z), interps=("bicubic", "bspline"))
    # subset radii at both ends of the tensor-core FFT-CC range
    for r in (8, 31):
        pair, g = synth.small_case(h=150, w=170, r=r, grid=9, seed=100 + r)
        rp, u, v, z = R.fftcc(pair.ref, pair.tar, g)
        save(f"r{r}", pair.ref, pair.tar, g, rp, u, v, fft=(u, v, z))
    # non-square subsets: the reference's IC-GN handles them; its FFT-CC plans
    # the window with the dimensions swapped (TW_paDIC_FFTCC2D_CPU.cpp:62-73),
    # so the guesses are the oracle's FFT-CC of the [2ry][2rx] window
    rx, ry = 12, 8
    pair, _ = synth.small_case(h=150, w=170, r=rx, grid=9, seed=77)
    g = synth.Geometry(170, 150, 1, 1, 168, 148, rx, 9, 12, subset_ry=ry)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, rx, g.grid, g.margin, ry=ry)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, rx, g.grid, ry=ry)
    u, v, _, _ = O.fftcc(pair.ref, pair.tar, poi, rx, ry=ry)
    save("nonsquare", pair.ref, pair.tar, g, poi, u, v)
    # every flag the reference raises
    ref, tar, g, poi, gu, gv = flags_case()
    save("flags", ref, tar, g, poi, gu, gv, interps=("bicubic", "bspline"))


if __name__ == "__main__":
    main()
