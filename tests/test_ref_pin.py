"""The oracle pinned to the reference's own code.

tests/golden/ref_<case>.npz hold outputs of the reference's Fftcc2D_CPU and
ICGN2D_CPU, compiled from the reference sources with stand-ins for FFTW,
LAPACKE, OpenCV and Qt (oracle/build_ref.py; the fixtures are made by
tests/golden/make_ref_golden.py).  Here the oracle (tw_oracle.cpp, the C++
restatement every GPU parity test uses) is run on the stored inputs and must
give the reference's results:

* FFT-CC: integer u, v equal (peaks tied in exact integers, or within FP32
  rounding, are counted and allowed), ZNCC within 1e-6;
* IC-GN from the stored guesses: flags equal on every POI, iteration counts
  equal (a POI stopping on the other side of the convergence threshold is a
  tie, at most 1 % + 1), u and v within 1e-4 px on every POI.  The two differ
  only by the FFT and Cholesky arithmetic (FFTW / LAPACK against their
  restatements): the largest difference measured is 5.3e-5 px.

When the reference checkout is present, a second test rebuilds the reference
and requires that it reproduces the fixtures exactly.
"""
import glob
import os

import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "ref_*.npz")))
UV_PIN = 1e-4
ZNCC_PIN = 1e-6


def load(case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    gm = [int(x) for x in d["geom"]]
    g = synth.Geometry(gm[0], gm[1], gm[2], gm[3], gm[4], gm[5], gm[6], gm[8], gm[9], gm[10],
                       float(d["delta_p"]), subset_ry=gm[7])
    return d, g


def interps_of(d):
    return [i for i in ("bicubic", "bspline") if f"{i}_u" in d]


def test_fixture_set_is_complete():
    assert set(CASES) >= {"small", "plain512", "r8", "r31", "nonsquare", "flags"}
    d, _ = load("flags")
    # every flag the reference raises on the CPU path, OutofROI before and after the first solve
    fl, it = d["bicubic_flags"], d["bicubic_iters"]
    assert {0, 1, 2, 4} <= set(fl.tolist())
    assert ((fl == 4) & (it == 0)).any() and ((fl == 4) & (it > 0)).any()


@pytest.mark.parametrize("case", CASES)
def test_oracle_fftcc_equals_reference(case):
    d, g = load(case)
    if "fftcc_u" not in d:
        pytest.skip("no FFT-CC in this case")
    u, v, z, st = O.fftcc(d["ref"], d["tar"], d["poi"], g.subset_r, ry=g.subset_ry)
    rep = C.fftcc_parity(d["ref"], d["tar"], d["poi"], g.subset_r, u, v, z, d["fftcc_u"], d["fftcc_v"],
                         d["fftcc_zncc"], st)
    assert rep.unexplained == 0, rep
    assert rep.max_zncc_err <= ZNCC_PIN, rep
    # dark subsets keep the zero the reference's calloc gave them
    np.testing.assert_array_equal(u[st != 0], d["fftcc_u"][st != 0])


@pytest.mark.parametrize("case", CASES)
def test_oracle_icgn_equals_reference(case):
    d, g = load(case)
    for interp in interps_of(d):
        p6, it, fl = O.icgn(d["ref"], d["tar"], g, d["poi"], d["guess_u"], d["guess_v"], interp=interp)
        np.testing.assert_array_equal(fl, d[f"{interp}_flags"], err_msg=interp)
        ties = int((it != d[f"{interp}_iters"]).sum())
        assert ties <= int(0.01 * len(it)) + 1, (interp, ties)
        du = np.abs(p6[:, 0] - d[f"{interp}_u"]).max()
        dv = np.abs(p6[:, 3] - d[f"{interp}_v"]).max()
        assert du <= UV_PIN and dv <= UV_PIN, (interp, du, dv)


@pytest.mark.parametrize("case", CASES)
def test_reference_build_reproduces_fixtures(case):
    """The reference sources, rebuilt here, give the stored outputs exactly."""
    from oracle import build_ref as R
    if not R.available():
        pytest.skip("reference checkout not present")
    d, g = load(case)
    if "fftcc_u" in d:
        poi, u, v, z = R.fftcc(d["ref"], d["tar"], g)
        np.testing.assert_array_equal(poi, d["poi"])
        np.testing.assert_array_equal(u, d["fftcc_u"])
        np.testing.assert_array_equal(v, d["fftcc_v"])
        np.testing.assert_array_equal(z, d["fftcc_zncc"])
    for interp in interps_of(d):
        u, v, it, fl = R.icgn(d["ref"], d["tar"], g, d["poi"], d["guess_u"], d["guess_v"], interp=interp)
        for k, a in (("u", u), ("v", v), ("iters", it), ("flags", fl)):
            np.testing.assert_array_equal(a, d[f"{interp}_{k}"], err_msg=f"{interp}_{k}")
