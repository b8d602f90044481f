"""Bicubic B-spline interpolation (ICGN2DInterpolationFLag::BicubicSpline,
BicubicSplineCoefficients_s, TW/TW_Engine/TW_utils.cpp:521-602): the
oracle's LUT against an independent float64 evaluation and a known answer,
and the GPU IC-GN with the B-spline LUT against the oracle."""
import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import INTERP_BSPLINE, PATH_FAST, PATH_PLAIN, dic, synth

CP = np.array([[71, -19, 5, -1], [-19, 95, -25, 5], [5, -25, 95, -19], [-1, 5, -19, 71]]) / 56.0
BASE = np.array([[-1, 3, -3, 1], [3, -6, 3, 0], [-3, 0, 3, 0], [1, 4, 1, 0]]) / 6.0


def _lut64(tar, sx, sy, rw, rh):
    """float64: Base CP Omega CP Base^T per pixel, both indices reversed."""
    H, W = tar.shape
    pad = np.zeros((H + 4, W + 4))
    pad[1:H + 1, 1:W + 1] = tar
    out = np.zeros((rh, rw, 16))
    M = BASE @ CP
    for i in range(rh):
        for j in range(rw):
            om = pad[i + sy:i + sy + 4, j + sx:j + sx + 4]  # rows y-1..y+2, columns x-1..x+2
            bs = M @ om @ M.T
            out[i, j] = bs[::-1, ::-1].ravel()
    return out


def test_oracle_bspline_lut_matches_float64():
    pair, g = synth.small_case(h=40, w=48)
    rw, rh = 30, 24
    lut = O.bspline_lut(pair.tar, 2, 3, rw, rh)
    want = _lut64(pair.tar, 2, 3, rw, rh)
    np.testing.assert_allclose(lut, want, rtol=0, atol=2e-4 * max(1.0, np.abs(want).max()))


def test_bspline_reproduces_constants():
    tar = np.full((20, 24), 137, np.uint8)
    lut = O.bspline_lut(tar, 2, 2, 16, 12).astype(np.float64).reshape(12, 16, 4, 4)
    for fx, fy in [(0.0, 0.0), (0.3, 0.7), (0.99, 0.01)]:
        val = np.einsum("ijkl,k,l->ij", lut, fy ** np.arange(4), fx ** np.arange(4))
        np.testing.assert_allclose(val, 137.0, atol=2e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("path", [PATH_PLAIN, PATH_FAST])
@pytest.mark.parametrize("case", ["small", "plain512"])
def test_bspline_icgn_parity(case, path):
    pair, g = synth.small_case() if case == "small" else synth.plain_512()
    p = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, g.grid,
                        g.grid, g.margin, g.margin, g.max_iter, g.delta_p, path)
    poi = dic.poi_positions(p)
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    p6_or, it_or, fl_or = O.icgn(pair.ref, pair.tar, g, poi, u_or, v_or, interp="bspline")
    fr = dic.DICFrame(p)
    fr.set_interpolation(INTERP_BSPLINE)
    fr.set_reference(pair.ref)
    out = fr.alloc_outputs()
    fr.process(pair.tar, **out)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=path)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    same = (U.ravel() == u_or) & (V.ravel() == v_or)
    rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same, r=g.subset_r)
    assert rep.ok(), rep
    assert (out["flags"] == 0).mean() > 0.9
    err = C.truth_error(pair, poi, out["p6"], out["flags"])
    assert err["max_abs_u"] < 0.1 and err["max_abs_v"] < 0.1, err
    # the handle entry point (cuICGN2D with Iflag) agrees with the frame
    ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, len(poi), 1,
                      g.max_iter, g.delta_p, path=path, Iflag=INTERP_BSPLINE)
    ic.ResetRefImg(pair.ref)
    it = np.zeros(len(poi), np.int32)
    p6h, flh = ic.ICGN2D_Algorithm(U.ravel().copy(), V.ravel().copy(), it, poi, pair.tar)
    np.testing.assert_array_equal(p6h, out["p6"])
