"""GPU parity of the C-ABI paths against the oracle (the FP32 restatement of
the reference CPU path), at sizes the oracle finishes in seconds, plus
size-independent properties at the full 2048x2048 workload."""
import glob
import os

import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import (INTERP_BICUBIC, INTERP_BSPLINE, PATH_FAST, PATH_PLAIN, SAMPLER_LUT, SAMPLER_NBHD,
                      SAMPLER_WINDOW, synth)
from tw_gb300 import dic

pytestmark = pytest.mark.gpu

PATHS = [PATH_PLAIN, PATH_FAST]
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def params_of(g, path):
    return dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                           g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, path)


def oracle_run(pair, g, poi):
    u, v, z, st = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    p6, it, fl = O.icgn(pair.ref, pair.tar, g, poi, u, v)
    return u, v, z, st, p6, it, fl


@pytest.fixture(scope="module")
def small():
    pair, g = synth.small_case()
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    return pair, g, poi, oracle_run(pair, g, poi)


@pytest.fixture(scope="module")
def plain512():
    pair, g = synth.plain_512()
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    return pair, g, poi, oracle_run(pair, g, poi)


@pytest.mark.parametrize("path", PATHS)
def test_fftcc_parity(small, path):
    pair, g, poi, (u_or, v_or, z_or, st_or, *_rest) = small
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=path)
    np.testing.assert_array_equal(f.POIPositions(), poi)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    st = np.zeros(f.GetNumPOIs(), np.uint8)
    f.ComputeFFTCC(U, V, Z, pair.tar, status=st)
    rep = C.fftcc_parity(pair.ref, pair.tar, poi, g.subset_r, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or,
                         st_or)
    assert (st == st_or).all()
    assert rep.ok(), rep


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("case", ["small", "plain512"])
def test_frame_parity(request, case, path):
    pair, g, poi, (u_or, v_or, z_or, st_or, p6_or, it_or, fl_or) = request.getfixturevalue(case)
    fr = dic.DICFrame(params_of(g, path))
    np.testing.assert_array_equal(fr.poi_positions(), poi)
    fr.set_reference(pair.ref)
    out = fr.alloc_outputs()
    fr.process(pair.tar, **out)
    # compare IC-GN where the GPU's FFT-CC guess equals the oracle's (ties
    # excepted by the FFT-CC parity test)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=path)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    rep_f = C.fftcc_parity(pair.ref, pair.tar, poi, g.subset_r, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or,
                           st_or)
    assert rep_f.ok(), rep_f
    same_start = (U.ravel() == u_or) & (V.ravel() == v_or)
    rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same_start,
                        r=g.subset_r)
    print(case, path, rep_f, rep)
    assert rep.ok(), rep
    np.testing.assert_array_equal(out["u"], out["p6"][:, 0])
    np.testing.assert_array_equal(out["v"], out["p6"][:, 3])
    err = C.truth_error(pair, poi, out["p6"], out["flags"])
    assert err["max_abs_u"] < 0.05 and err["max_abs_v"] < 0.05, err
    # second frame with the cached reference gives identical results
    out2 = fr.alloc_outputs()
    fr.process(pair.tar, **out2)
    for k in out:
        np.testing.assert_array_equal(out[k], out2[k])


# (threads per CTA, chunk): one POI per CTA (chunk 0), or one POI per warp
# over runs of `chunk` consecutive POIs
ICGN_SHAPES = [(32, 0), (64, 0), (128, 0), (256, 0), (1024, 32), (512, 16), (128, 4)]


@pytest.mark.parametrize("shape", ICGN_SHAPES, ids=lambda s: f"t{s[0]}c{s[1]}")
@pytest.mark.parametrize("sampler", [SAMPLER_WINDOW, SAMPLER_LUT, SAMPLER_NBHD])
def test_fast_icgn_samplers(plain512, sampler, shape):
    """Every launch shape and target sampler of the fast IC-GN meets the
    parity bar against the oracle (staged window and neighbourhood table
    evaluate the Catmull-Rom form, the LUT sampler the reference's Hermite
    coefficients)."""
    threads, chunk = shape  # with the window sampler a one-POI-per-warp shape runs one-POI-per-CTA kernels
    pair, g, poi, (u_or, v_or, z_or, st_or, p6_or, it_or, fl_or) = plain512
    fr = dic.DICFrame(params_of(g, PATH_FAST))
    fr.set_tuning(threads, 0, sampler, 1, icgn_chunk=chunk)
    fr.set_reference(pair.ref)
    out = fr.alloc_outputs()
    fr.process(pair.tar, **out)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=PATH_FAST)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    same_start = (U.ravel() == u_or) & (V.ravel() == v_or)
    rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same_start,
                        r=g.subset_r)
    assert rep.ok(), (sampler, shape, rep)


@pytest.mark.parametrize("max_iter", [20, 1])
@pytest.mark.parametrize("sampler", [SAMPLER_NBHD, SAMPLER_LUT, SAMPLER_WINDOW])
def test_icgn_subsets_touching_the_roi_edge(sampler, max_iter):
    """Margin 0: the last POIs' subsets end on the ROI's last row and column.
    The first (integer) pass reads those pixels from the image, while the
    reference's LUT, and so the table samplers, are zero there; with one
    iteration the result is the first pass's update alone."""
    h, w = 156, 191
    field, grad = synth.affine_field(0.3, 0.25, 0.002, -0.001, 0.001, -0.0015, w / 2, h / 2)
    pair = synth.make_pair(h, w, int(6000 * h * w / (512 * 512)), field, grad, 77, description="ROI-edge case")
    g = synth.Geometry(w, h, 1, 1, w - 2, h - 2, 10, 7, 0, max_iter=max_iter)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    assert poi[:, 0].max() + g.subset_r == g.start_y + g.roi_h - 1
    assert poi[:, 1].max() + g.subset_r == g.start_x + g.roi_w - 1
    u_or, v_or, z_or, st_or, p6_or, it_or, fl_or = oracle_run(pair, g, poi)
    fr = dic.DICFrame(params_of(g, PATH_FAST))
    fr.set_tuning(1024, 0, sampler, 1, icgn_chunk=32)
    fr.set_reference(pair.ref)
    out = fr.alloc_outputs()
    fr.process(pair.tar, **out)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=PATH_FAST)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    same_start = (U.ravel() == u_or) & (V.ravel() == v_or)
    rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same_start,
                        r=g.subset_r)
    assert rep.ok(), (sampler, rep)


@pytest.mark.parametrize("sampler", [SAMPLER_LUT, SAMPLER_NBHD])
def test_warp_layout_matches_one_warp_cta(plain512, sampler):
    """One POI per warp (per-reference gradient image, runs of consecutive
    POIs) does per POI exactly the arithmetic of the one-warp CTA: same
    sample order per lane, sums, solve and update, so every output is
    bit-identical, whatever the run length, CTA size and loop unrolling."""
    pair, g, poi, _ = plain512
    outs = []
    for threads, chunk, unroll in [(32, 0, 4), (1024, 32, 4), (1024, 32, 2), (1024, 32, 8), (512, 7, 4),
                                   (128, 1, 4)]:
        fr = dic.DICFrame(params_of(g, PATH_FAST))
        fr.set_tuning(threads, 0, sampler, 1, icgn_chunk=chunk)
        fr.set_icgn_unroll(unroll)
        fr.set_reference(pair.ref)
        o = fr.alloc_outputs()
        fr.process(pair.tar, **o)
        outs.append(o)
    for o in outs[1:]:
        for k in o:
            np.testing.assert_array_equal(o[k], outs[0][k], err_msg=k)


def test_layout_rejects_bad_shapes(small):
    pair, g, poi, _ = small
    fr = dic.DICFrame(params_of(g, PATH_FAST))
    with pytest.raises(Exception):
        fr.set_icgn_layout(-1)
    with pytest.raises(Exception):
        fr.set_tuning(96, 0, SAMPLER_NBHD, 1)
    with pytest.raises(Exception):
        fr.set_icgn_unroll(3)
    # 1024 threads need the one-POI-per-warp layout: the launch is refused
    fr.set_tuning(1024, 0, SAMPLER_NBHD, 1, icgn_chunk=0)
    fr.set_reference(pair.ref)
    with pytest.raises(Exception):
        fr.process(pair.tar, **fr.alloc_outputs())


@pytest.mark.parametrize("path", PATHS)
def test_device_buffers_match_host(small, path):
    import torch
    pair, g, poi, _ = small
    fr = dic.DICFrame(params_of(g, path))
    fr.set_reference(torch.from_numpy(pair.ref).cuda())
    host = fr.alloc_outputs()
    fr.process(pair.tar, **host)
    dev = fr.alloc_outputs(device="cuda")
    fr.process(torch.from_numpy(pair.tar).cuda(), **dev)
    torch.cuda.synchronize()
    for k in host:
        np.testing.assert_array_equal(host[k], dev[k].cpu().numpy())


@pytest.mark.parametrize("path", PATHS)
def test_icgn_api_with_oracle_guesses(small, path):
    pair, g, poi, (u_or, v_or, z_or, st_or, p6_or, it_or, fl_or) = small
    n = len(poi)
    ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, n, 1,
                      g.max_iter, g.delta_p, path=path)
    ic.ResetRefImg(pair.ref)
    u, v = u_or.copy(), v_or.copy()
    iters = np.zeros(n, np.int32)
    p6, fl = ic.ICGN2D_Algorithm(u, v, iters, poi, pair.tar)
    rep = C.icgn_parity(p6, iters, fl, p6_or, it_or, fl_or, r=g.subset_r)
    assert rep.ok(), rep


@pytest.mark.parametrize("path", PATHS)
def test_icgn_flags_and_counters(small, path):
    """OutofROI before the first solve leaves the counter untouched; a dark
    reference flags DarkSubset; a subset outside the ROI is OutofROI."""
    pair, g, _, _ = small
    poi = np.array([[80, 96], [80, 96], [40, 150], [5, 5]], np.int32)
    u0 = np.array([1.6, 200.0, 1.6, 0.0], np.float32)
    v0 = np.array([-2.4, 0.0, -2.4, 0.0], np.float32)
    ref2 = pair.ref.copy()
    ref2[25:56, 135:166] = 0  # dark reference subset around POI 2
    ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, 4, 1,
                      g.max_iter, g.delta_p, path=path)
    ic.ResetRefImg(ref2)
    u, v = u0.copy(), v0.copy()
    iters = np.full(4, -1, np.int32)
    p6, fl = ic.ICGN2D_Algorithm(u, v, iters, poi, pair.tar)
    p6_or, it_or, fl_or = O.icgn(ref2, pair.tar, g, poi, u0, v0, iters_init=-1)
    np.testing.assert_array_equal(fl, fl_or)
    np.testing.assert_array_equal(iters, it_or)
    assert fl[0] == 0 and iters[0] >= 1
    assert fl[1] == 4 and iters[1] == -1 and u[1] == 200.0
    assert fl[2] == 1 and iters[2] == -1
    assert fl[3] == 4


def test_icgn_singular_hessian(small):
    """A reference subset of vertical stripes (every column constant, one
    row beyond the subset too) has R_y = 0: its Hessian is singular, so the
    factorization flags SingularHessian and the IC-GN stops after the first
    pass, as the oracle (spotrf info > 0)."""
    pair, g, _, _ = small
    poi = np.array([[80, 96], [60, 60]], np.int32)
    ref2 = pair.ref.copy()
    cols = np.arange(60 - g.subset_r - 2, 60 + g.subset_r + 3)
    ref2[60 - g.subset_r - 2:60 + g.subset_r + 3, cols] = (37 * cols % 200 + 20).astype(np.uint8)[None, :]
    u0 = np.array([1.6, 1.6], np.float32)
    v0 = np.array([-2.4, -2.4], np.float32)
    p6_or, it_or, fl_or = O.icgn(ref2, pair.tar, g, poi, u0, v0)
    assert list(fl_or) == [0, 2]
    for path in PATHS:
        ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, 2, 1,
                          g.max_iter, g.delta_p, path=path)
        ic.ResetRefImg(ref2)
        u, v = u0.copy(), v0.copy()
        iters = np.zeros(2, np.int32)
        p6, fl = ic.ICGN2D_Algorithm(u, v, iters, poi, pair.tar)
        np.testing.assert_array_equal(fl, fl_or, err_msg=str(path))
        np.testing.assert_array_equal(iters, it_or, err_msg=str(path))


@pytest.mark.parametrize("r,paths", [(6, [PATH_FAST]), (8, PATHS), (15, PATHS), (24, PATHS), (31, PATHS)])
def test_icgn_radii_parity(r, paths):
    """FFT-CC then IC-GN at subset widths below, near and above the warp
    width (13 to 63 pixels; the per-reference sums walk a subset 32 samples
    at a time with a row carry, two rows a step at r = 6), against the
    oracle.  Small subsets are ill-conditioned in FP32: on these images the
    FP32 oracle differs from its FP64 twin by up to 0.021 px at r = 4 and
    0.009 px at r = 5.  At r = 6 (13 x 13 subsets) the fast path is held to
    the flag, iteration and 1e-3 px bars with the gradient bar scaled to
    1e-4: a gradient of P is resolved over 13 pixels instead of the 41 the
    1e-5 bar was set for, and one POI differs by 2.5e-5; the plain path's
    FP32 Gauss-Jordan inverse is left out there."""
    pair, g = synth.small_case(h=150, w=170, r=r, grid=9, seed=300 + r)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u_or, v_or, z_or, st_or, p6_or, it_or, fl_or = oracle_run(pair, g, poi)
    for path in paths:
        fr = dic.DICFrame(params_of(g, path))
        fr.set_reference(pair.ref)
        out = fr.alloc_outputs()
        fr.process(pair.tar, **out)
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, r, r, g.grid, g.grid,
                          g.margin, g.margin, path=path)
        U, V, Z = f.InitializeFFTCC(pair.ref)
        f.ComputeFFTCC(U, V, Z, pair.tar)
        same_start = (U.ravel() == u_or) & (V.ravel() == v_or)
        rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same_start, r=r)
        print(r, path, rep)
        if r < 8:
            assert rep.flag_mismatch == 0 and rep.over_uv == 0 and rep.over_tie_grad == 0, (r, path, rep)
            assert rep.iter_mismatch <= rep.tie_limit and rep.max_dgrad < 1e-4, (r, path, rep)
        else:
            assert rep.ok(), (r, path, rep)


def test_non_square_subsets():
    """Half width 12, half height 8 (25 x 17 IC-GN subsets, 24 x 16 FFT-CC
    windows transformed as [2ry][2rx] arrays): POI grid, FFT-CC and IC-GN on
    both paths against the oracle."""
    rx, ry = 12, 8
    pair, _ = synth.small_case(h=150, w=170, r=rx, grid=9, seed=77)
    g = synth.Geometry(170, 150, 1, 1, 168, 148, rx, 9, 12, subset_ry=ry)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, rx, g.grid, g.margin, ry=ry)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, rx, g.grid, ry=ry)
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, rx, ry=ry)
    p6_or, it_or, fl_or = O.icgn(pair.ref, pair.tar, g, poi, u_or, v_or)
    assert (fl_or == 0).mean() > 0.9
    for path in PATHS:
        prm = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, rx, ry, g.grid, g.grid,
                              g.margin, g.margin, g.max_iter, g.delta_p, path)
        np.testing.assert_array_equal(dic.poi_positions(prm), poi)
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, rx, ry, g.grid, g.grid,
                          g.margin, g.margin, path=path)
        U, V, Z = f.InitializeFFTCC(pair.ref)
        f.ComputeFFTCC(U, V, Z, pair.tar)
        rep_f = C.fftcc_parity(pair.ref, pair.tar, poi, rx, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or, st_or,
                               ry=ry)
        assert rep_f.ok(), (path, rep_f)
        same = (U.ravel() == u_or) & (V.ravel() == v_or)
        fr = dic.DICFrame(prm)
        fr.set_reference(pair.ref)
        out = fr.alloc_outputs()
        fr.process(pair.tar, **out)
        rep = C.icgn_parity(out["p6"], out["iters"], out["flags"], p6_or, it_or, fl_or, mask=same, r=ry)
        assert rep.ok(), (path, rep)


@pytest.mark.parametrize("r", [5, 8, 10, 15, 16, 20, 24, 29, 31])
def test_fftcc_radii_parity(r):
    """FFT-CC at the subset radii of the uneven-batching workload (r in
    10..30) and the ends of the supported range, both paths."""
    pair, g = synth.small_case(h=150, w=170, r=r, grid=9, seed=100 + r)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    if nx <= 0 or ny <= 0:
        pytest.skip("no POI at this radius")
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, r)
    for path in PATHS:
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, r, r, g.grid, g.grid,
                          g.margin, g.margin, path=path)
        U, V, Z = f.InitializeFFTCC(pair.ref)
        st = np.zeros(f.GetNumPOIs(), np.uint8)
        f.ComputeFFTCC(U, V, Z, pair.tar, status=st)
        rep = C.fftcc_parity(pair.ref, pair.tar, poi, r, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or, st_or)
        print(r, path, rep)
        assert (st == st_or).all()
        assert rep.ok(), (r, path, rep)


@pytest.mark.parametrize("r", [8, 15, 20, 31])
def test_fftcc_twiddle_precisions_agree(r):
    """Single FP16 twiddles (the default) and hi + lo twiddles give the same
    integer displacements, ZNCC and everything downstream: the candidates of
    either approximate surface are re-evaluated in exact integers."""
    pair, g = synth.small_case(h=150, w=170, r=r, grid=9, seed=200 + r)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    if nx <= 0 or ny <= 0:
        pytest.skip("no POI at this radius")
    outs = []
    for hi_lo in (0, 1):
        fr = dic.DICFrame(params_of(g, PATH_FAST))
        fr.set_fftcc_twiddles(hi_lo)
        fr.set_reference(pair.ref)
        o = fr.alloc_outputs()
        fr.process(pair.tar, **o)
        outs.append(o)
    for k in outs[0]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)


def test_fftcc_dark_subset_untouched(small):
    pair, g, _, _ = small
    ref = np.full_like(pair.ref, 50)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin)
    U, V, Z = f.InitializeFFTCC(ref)
    U[:] = -3
    st = np.zeros(f.GetNumPOIs(), np.uint8)
    f.ComputeFFTCC(U, V, Z, pair.tar, status=st)
    assert (st == 1).all() and (U == -3).all()


def test_full_size_properties():
    """2048x2048, 41x41 subsets, step 5 (155,236 POIs): fast vs plain path,
    fast vs imposed field, and a POI sample against the oracle."""
    pair, g = synth.scale_2048()
    res = {}
    for path in PATHS:
        fr = dic.DICFrame(params_of(g, path))
        assert fr.n == 155236
        fr.set_reference(pair.ref)
        out = fr.alloc_outputs()
        fr.process(pair.tar, **out)
        res[path] = out
        poi = fr.poi_positions()
    a, b = res[PATH_FAST], res[PATH_PLAIN]
    both = (a["flags"] == 0) & (b["flags"] == 0)
    assert both.mean() > 0.99
    d = np.abs(a["p6"][both] - b["p6"][both])
    assert d[:, [0, 3]].max() < 1e-3
    err = C.truth_error(pair, poi, a["p6"], a["flags"])
    assert err["rms"] < 0.02, err
    # oracle on a sample of POIs: the integer FFT-CC of the whole frame on
    # both paths, then IC-GN from the oracle's guesses through the IC-GN API
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(len(poi), 3000, replace=False))
    sp = poi[idx]
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, sp, g.subset_r)
    for path in PATHS:
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                          g.grid, g.margin, g.margin, path=path)
        U, V, Z = f.InitializeFFTCC(pair.ref)
        f.ComputeFFTCC(U, V, Z, pair.tar)
        rep_f = C.fftcc_parity(pair.ref, pair.tar, sp, g.subset_r, U.ravel()[idx], V.ravel()[idx], Z.ravel()[idx],
                               u_or, v_or, z_or, st_or)
        assert rep_f.ok(), (path, rep_f)
    p6_or, it_or, fl_or = O.icgn(pair.ref, pair.tar, g, sp, u_or, v_or)
    for path in PATHS:
        ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                          len(sp), 1, g.max_iter, g.delta_p, path=path)
        ic.ResetRefImg(pair.ref)
        u, v = u_or.copy(), v_or.copy()
        iters = np.zeros(len(sp), np.int32)
        p6, fl = ic.ICGN2D_Algorithm(u, v, iters, sp, pair.tar)
        rep = C.icgn_parity(p6, iters, fl, p6_or, it_or, fl_or, r=g.subset_r)
        assert rep.ok(), (path, rep)


@pytest.mark.parametrize("y_amp,min_cand", [(1.5, 129), (8.0, 17)])
def test_fftcc_broad_surface_parity(y_amp, min_cand):
    """Low-texture stripes give a broad, periodic correlation surface: every
    POI has more candidate shifts (within 0.01 ZNCC of the approximate peak)
    than one exact-evaluation pass of a group batch holds at y_amp 1.5
    (about 200 per POI), and more than 16 at y_amp 8.  Every candidate is
    evaluated exactly, in a fixed slot order, so the integer result equals
    the oracle's and repeats bit for bit."""
    ref, tar = synth.stripe_pair(y_amp=y_amp)
    r, grid, margin = 20, 9, 12
    g = synth.Geometry(170, 150, 1, 1, 168, 148, r, grid, margin)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, r, grid, margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, margin, r, grid)
    counts = np.array([O.candidate_lower_bound(ref, tar, py, px, r) for py, px in poi])
    assert counts.min() >= min_cand, counts.min()
    u_or, v_or, z_or, st_or = O.fftcc(ref, tar, poi, r)
    for path in PATHS:
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, r, r, grid, grid, margin, margin,
                          path=path)
        runs = []
        for _ in range(2):
            U, V, Z = f.InitializeFFTCC(ref)
            st = np.zeros(f.GetNumPOIs(), np.uint8)
            f.ComputeFFTCC(U, V, Z, tar, status=st)
            runs.append((U.copy(), V.copy(), Z.copy()))
            assert (st == st_or).all()
        rep = C.fftcc_parity(ref, tar, poi, r, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or, st_or)
        print(y_amp, path, rep)
        assert rep.ok(), (y_amp, path, rep)
        for a, b in zip(runs[0], runs[1]):
            np.testing.assert_array_equal(a, b)


REF_CASES = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("case", REF_CASES)
def test_gpu_matches_reference_fixture(case, path):
    """The CUDA path against the outputs of the reference's own CPU code
    (tests/golden/ref_<case>.npz, made from the reference sources): integer
    FFT-CC equal but for counted ties, ZNCC within 3e-5; IC-GN from the
    stored guesses with the reference's flags, its iteration counts but for
    convergence-threshold ties (at most 1 % + 1), u and v within 1e-3 px."""
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    gm = [int(x) for x in d["geom"]]
    g = synth.Geometry(gm[0], gm[1], gm[2], gm[3], gm[4], gm[5], gm[6], gm[8], gm[9], gm[10],
                       float(d["delta_p"]), subset_ry=gm[7])
    ref, tar, poi = d["ref"], d["tar"], d["poi"]
    rx, ry = g.subset_r, g.subset_ry
    if "fftcc_u" in d:
        f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, rx, ry, g.grid, g.grid,
                          g.margin, g.margin, path=path)
        np.testing.assert_array_equal(f.POIPositions(), poi)
        U, V, Z = f.InitializeFFTCC(ref)
        st = np.zeros(f.GetNumPOIs(), np.uint8)
        f.ComputeFFTCC(U, V, Z, tar, status=st)
        rep = C.fftcc_parity(ref, tar, poi, rx, U.ravel(), V.ravel(), Z.ravel(), d["fftcc_u"], d["fftcc_v"],
                             d["fftcc_zncc"], st, ry=ry)
        assert rep.ok(), (case, path, rep)
    for interp in ("bicubic", "bspline"):
        if f"{interp}_u" not in d:
            continue
        n = len(poi)
        ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, rx, ry, n, 1, g.max_iter,
                          g.delta_p, path=path,
                          Iflag=INTERP_BSPLINE if interp == "bspline" else INTERP_BICUBIC)
        ic.ResetRefImg(ref)
        u, v = d["guess_u"].copy(), d["guess_v"].copy()
        iters = np.zeros(n, np.int32)
        p6, fl = ic.ICGN2D_Algorithm(u, v, iters, poi, tar)
        np.testing.assert_array_equal(fl, d[f"{interp}_flags"], err_msg=f"{case} {interp} {path}")
        ties = int((iters != d[f"{interp}_iters"]).sum())
        assert ties <= int(0.01 * n) + 1, (case, interp, path, ties)
        du = float(np.abs(u - d[f"{interp}_u"]).max())
        dv = float(np.abs(v - d[f"{interp}_v"]).max())
        print(case, interp, path, "ties", ties, "du", du, "dv", dv)
        assert du <= C.UV_TOL and dv <= C.UV_TOL, (case, interp, path, du, dv)


def test_device_pois_rewritten_in_place(small):
    """A device POI array rewritten in place between two calls (same
    address, new contents) is read afresh: the second call's results follow
    the new POIs (here the same POIs in reverse order, so a stale reference
    cache would pair every POI with another POI's Hessian)."""
    import torch
    pair, g, poi, (u_or, v_or, z_or, st_or, p6_or, it_or, fl_or) = small
    n = len(poi)
    ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, n, 1,
                      g.max_iter, g.delta_p, path=PATH_FAST)
    ic.cuInitialize(torch.from_numpy(pair.ref).cuda())
    d_tar = torch.from_numpy(pair.tar).cuda()
    d_poi = torch.from_numpy(poi).cuda()
    for order in (np.arange(n), np.arange(n)[::-1].copy()):
        d_poi.copy_(torch.from_numpy(poi[order]))
        du = torch.from_numpy(u_or[order]).cuda()
        dv = torch.from_numpy(v_or[order]).cuda()
        p6 = torch.zeros((n, 6), dtype=torch.float32, device="cuda")
        it = torch.zeros(n, dtype=torch.int32, device="cuda")
        fl = torch.zeros(n, dtype=torch.uint8, device="cuda")
        ic.cuCompute(d_tar, d_poi, du, dv, p6, it, fl)
        torch.cuda.synchronize()
        rep = C.icgn_parity(p6.cpu().numpy(), it.cpu().numpy(), fl.cpu().numpy(), p6_or[order], it_or[order],
                            fl_or[order], r=g.subset_r)
        assert rep.ok(), rep


@pytest.mark.parametrize("case", ["small", "plain512"])
def test_tables_equal_the_oracle(request, case):
    """The per-pixel tables element by element against the oracle: the
    bicubic LUT of the target (k_bicubic_lut) bit for bit, including the
    zero last ROI row and column (TW_utils.cpp:604-700); the reference
    gradients of the fast path (k_ref_grad) and of every subset in the plain
    path's per-reference cache (k_ref_precompute_plain) exactly
    (TW_utils.cpp:232-305); the B-spline LUT (k_bspline_lut) within FP32
    rounding of its products (TW_utils.cpp:521-602)."""
    pair, g, poi, _ = request.getfixturevalue(case)
    rx_o, ry_o, tx_o, ty_o, txy_o, lut_o = O.precompute_f32(pair.ref, pair.tar, g.start_x, g.start_y, g.roi_w,
                                                            g.roi_h)
    fr = dic.DICFrame(params_of(g, PATH_PLAIN))
    fr.set_reference(pair.ref)
    fr.process(pair.tar, **fr.alloc_outputs())
    lut = fr.table("bicubic_lut")
    np.testing.assert_array_equal(lut, lut_o)
    assert (lut[-1] == 0).all() and (lut[:, -1] == 0).all() and np.abs(lut[:-1, :-1]).max() > 0
    grad = fr.table("ref_gradient")
    np.testing.assert_array_equal(grad[..., 0], rx_o)
    np.testing.assert_array_equal(grad[..., 1], ry_o)
    sub = fr.table("subset_gradient")
    r = g.subset_r
    off = np.arange(-r, r + 1)
    yy = poi[:, 0, None, None] + off[None, :, None] - g.start_y
    xx = poi[:, 1, None, None] + off[None, None, :] - g.start_x
    np.testing.assert_array_equal(sub[..., 0], rx_o[yy, xx].reshape(len(poi), -1))
    np.testing.assert_array_equal(sub[..., 1], ry_o[yy, xx].reshape(len(poi), -1))
    bs = fr.table("bspline_lut").reshape(g.roi_h, g.roi_w, 16)
    bs_o = O.bspline_lut(pair.tar, g.start_x, g.start_y, g.roi_w, g.roi_h)
    print(case, "B-spline LUT: exact", float((bs == bs_o).mean()), "max diff", float(np.abs(bs - bs_o).max()))
    np.testing.assert_allclose(bs, bs_o, rtol=1e-6, atol=1e-4)


@pytest.mark.parametrize("h,w,r,grid", [
    (160, 300, 20, 5),    # batches of 6 on one POI row: the staged one-row boxes
    (170, 200, 20, 7),    # 13 POIs per row: batches across POI rows read the images
    (260, 420, 20, 60),   # a box would be wider than 256 bytes: every batch reads the images
    (200, 230, 31, 11),   # N = 62, batches of 4, rows of 16 and odd remainders
])
def test_fftcc_window_paths(h, w, r, grid):
    """The tensor-core FFT-CC's window sources: one TMA box pair per batch on
    one POI row, the images in global memory for batches across POI rows and
    for grid steps too wide for a box; strict parity with the oracle."""
    pair, g = synth.small_case(h=h, w=w, r=r, grid=grid, seed=300 + grid)
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    assert nx > 0 and ny > 0
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, r)
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, r, r, g.grid, g.grid, g.margin,
                      g.margin, path=PATH_FAST)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    st = np.zeros(f.GetNumPOIs(), np.uint8)
    f.ComputeFFTCC(U, V, Z, pair.tar, status=st)
    rep = C.fftcc_parity(pair.ref, pair.tar, poi, r, U.ravel(), V.ravel(), Z.ravel(), u_or, v_or, z_or, st_or)
    assert (st == st_or).all()
    assert rep.ok(), (nx, ny, rep)


def test_fftcc_batch_mixed_grid_steps():
    """Frames of one window size but different grid steps in one batched
    launch: the launch's window region is sized for the first frame's boxes,
    so a frame whose boxes do not fit reads its windows from the images;
    every frame equals its single-frame result and the oracle."""
    cases = [(180, 260, 20, 5, 41), (220, 330, 20, 23, 42), (200, 240, 20, 9, 43)]
    frames, tars, want, refs = [], [], [], []
    for h, w, r, grid, seed in cases:
        pair, g = synth.small_case(h=h, w=w, r=r, grid=grid, seed=seed)
        fr = dic.DICFrame(params_of(g, PATH_FAST))
        fr.set_reference(pair.ref)
        o = fr.alloc_outputs()
        fr.process(pair.tar, **o)
        frames.append(fr)
        tars.append(pair.tar)
        want.append(o)
        refs.append((pair, g))
    b = dic.DICBatch()
    outs = [fr.alloc_outputs() for fr in frames]
    b.process(frames, tars, outs)
    for i, (o, wnt, (pair, g)) in enumerate(zip(outs, want, refs)):
        for k in wnt:
            np.testing.assert_array_equal(o[k], wnt[k], err_msg=f"frame {i} {k}")
        poi = frames[i].poi_positions()
        u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
        sel = st_or == 0
        assert sel.mean() > 0.9
        np.testing.assert_allclose(o["zncc"][sel], z_or[sel], atol=3e-5)
