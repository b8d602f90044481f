"""Bicubic B-spline interpolation (ICGN2DInterpolationFLag::BicubicSpline,
BicubicSplineCoefficients_s, TW/TW_Engine/TW_utils.cpp:521-602): the
oracle's LUT against an independent float64 evaluation and a known answer,
the separable 4-tap form the fast IC-GN evaluates from the neighbourhood
table against the oracle's LUT, and the GPU IC-GN with either sampler
against the oracle."""
import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import INTERP_BSPLINE, PATH_FAST, PATH_PLAIN, SAMPLER_LUT, SAMPLER_NBHD, dic, synth

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


# Rows of Base CP with the powers of the fraction in increasing order, as
# the fast IC-GN evaluates them: tap weights (0, 1, 0, 0), (3/56) E1,
# (3/56) E2 and (1/7) E3 (integer taps, one DP4A each on the GPU).
E1 = np.array([-11, -1, 15, -3])
E2 = np.array([19, -39, 25, -5])
E3 = np.array([-3, 8, -8, 3])


def _row(v, t):
    """h(t) = v1 + (3/56) t (e1 + t (e2 + (8/3) t e3)) along the last axis."""
    return v[..., 1] + (3 / 56) * t * (v @ E1 + t * (v @ E2 + (8 / 3) * t * (v @ E3)))


def test_separable_form_is_the_bspline_lut():
    """(R Base CP) rows are the weights above, so the tensor product of _row
    in x then y equals the LUT polynomial at every ROI pixel, the last row
    and column (whose neighbourhood leaves the image) included."""
    M = BASE[::-1] @ CP * 336
    np.testing.assert_allclose(M, np.stack([[0, 336, 0, 0], 18 * E1, 18 * E2, 48 * E3]), atol=1e-9)
    pair, g = synth.small_case(h=40, w=48)
    sx, sy, rw, rh = 1, 1, 46, 38
    lut = O.bspline_lut(pair.tar, sx, sy, rw, rh).astype(np.float64).reshape(rh, rw, 4, 4)
    pad = np.zeros((44, 52))
    pad[2:42, 2:50] = pair.tar
    rng = np.random.default_rng(3)
    for k in range(300):
        # the first 40 on the last two ROI rows, then anywhere
        i = rh - 1 - k % 2 if k < 40 else rng.integers(0, rh)
        j = rng.integers(0, rw)
        fx, fy = rng.random(2)
        want = np.einsum("kl,k,l->", lut[i, j], fy ** np.arange(4), fx ** np.arange(4))
        om = pad[i + sy + 1:i + sy + 5, j + sx + 1:j + sx + 5]
        got = _row(_row(om, fx), fy)
        assert abs(got - want) < 1e-3, (i, j, got, want)


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


def _bspline_frame(g, pair, threads=1024, chunk=32, sampler=SAMPLER_NBHD, unroll=8):
    p = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, g.grid,
                        g.grid, g.margin, g.margin, g.max_iter, g.delta_p, PATH_FAST)
    fr = dic.DICFrame(p)
    fr.set_interpolation(INTERP_BSPLINE)
    fr.set_tuning(threads, 0, sampler, 1, icgn_chunk=chunk)
    fr.set_icgn_unroll(unroll)
    fr.set_reference(pair.ref)
    out = fr.alloc_outputs()
    fr.process(pair.tar, **out)
    return out


@pytest.mark.gpu
def test_bspline_table_and_lut_samplers_agree():
    """The neighbourhood table (separable form) and the B-spline LUT (Horner
    on the reference's coefficients) are two FP32 evaluations of the same
    interpolant: same flags, displacements within a small fraction of the
    1e-3 px parity bar."""
    pair, g = synth.plain_512()
    a = _bspline_frame(g, pair, sampler=SAMPLER_NBHD)
    b = _bspline_frame(g, pair, sampler=SAMPLER_LUT)
    np.testing.assert_array_equal(a["flags"], b["flags"])
    ok = a["flags"] == 0
    assert ok.mean() > 0.9
    d = np.abs(a["p6"][ok] - b["p6"][ok])
    assert d[:, [0, 3]].max() < 2e-4, d[:, [0, 3]].max()
    assert d[:, [1, 2, 4, 5]].max() < 1e-5, d[:, [1, 2, 4, 5]].max()
    assert (a["iters"] != b["iters"]).mean() < 0.01


@pytest.mark.gpu
def test_bspline_table_layouts_bit_identical():
    """One POI per warp (CTAs of 1024 and 256 threads, unrolled by 8, 2 or 4)
    and the one-warp CTA run the same per-POI arithmetic on the B-spline
    table: identical outputs."""
    pair, g = synth.plain_512()
    outs = [_bspline_frame(g, pair, threads=t, chunk=c, unroll=u)
            for t, c, u in [(32, 0, 4), (1024, 32, 8), (1024, 32, 2), (256, 3, 4)]]
    for o in outs[1:]:
        for k in ("p6", "iters", "flags"):
            np.testing.assert_array_equal(o[k], outs[0][k])


@pytest.mark.gpu
@pytest.mark.parametrize("max_iter", [20, 1])
@pytest.mark.parametrize("sampler", [SAMPLER_NBHD, SAMPLER_LUT])
def test_bspline_subsets_touching_the_roi_edge(sampler, max_iter):
    """Margin 0 with a one-pixel border: the last POIs' subsets end on the
    ROI's last row and column, where the B-spline LUT is written (unlike the
    bicubic one) from neighbourhoods that leave the image."""
    h, w = 156, 191
    field, grad = synth.affine_field(0.3, 0.25, 0.002, -0.001, 0.001, -0.0015, w / 2, h / 2)
    pair = synth.make_pair(h, w, int(6000 * h * w / (512 * 512)), field, grad, 77, description="ROI-edge case")
    g = synth.Geometry(w, h, 1, 1, w - 2, h - 2, 10, 7, 0, max_iter=max_iter)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    assert poi[:, 0].max() + g.subset_r == g.start_y + g.roi_h - 1
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    p6_or, it_or, fl_or = O.icgn(pair.ref, pair.tar, g, poi, u_or, v_or, interp="bspline")
    out = _bspline_frame(g, pair, sampler=sampler)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=PATH_FAST)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    same = (U.ravel() == u_or) & (V.ravel() == v_or)
    rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same, r=g.subset_r)
    assert rep.ok(), (sampler, rep)
