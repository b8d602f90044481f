"""CPU tests of the oracle (the C++ restatement of the reference CPU path).

The reference ships no golden vectors (its only active test asserts nothing,
TW/TW_EngineTester/FftccTest.cpp:14-77), so the oracle is pinned here against
(1) the third-party arithmetic it restates -- LAPACK spotrf/spotrs through
scipy's LAPACK and the DFT through numpy.fft --, (2) known answers written from
the mathematics, (3) imposed synthetic deformation fields, and (4) the
committed golden fixtures in tests/golden/ (regression of the oracle itself).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tw_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def small():
    return synth.small_case()


def test_poi_count_and_grid_match_reference_formula():
    # Fftcc2D::recomputeNumPOI (TW_paDIC_FFTCC2D.cpp:88-94)
    for roi, r, g, m in [(510, 16, 10, 20), (2046, 20, 5, 20), (100, 10, 7, 3), (40, 20, 1, 0)]:
        nx, ny, rc = O.num_pois(roi, roi, r, g, m)
        assert nx == ny == int(np.floor((roi - 2 * r - 2 * m) / np.float32(g))) + 1
        assert rc == 0
    assert O.num_pois(2046, 2046, 20, 5, 20)[:2] == (394, 394)  # 155,236 POIs
    nx, ny, rc = O.num_pois(30, 30, 20, 5, 0)
    assert rc != 0  # "Number of POIs is below 0!"
    # ComputePOIPositions_s (TW_utils.cpp:29-49): (y, x), x fastest
    yx = O.poi_positions(3, 5, 4, 2, 7, 10, 6)
    assert yx.shape == (8, 2)
    assert tuple(yx[0]) == (5 + 7 + 10, 3 + 7 + 10)
    assert tuple(yx[1]) == (22, 20 + 6)
    assert tuple(yx[4]) == (22 + 6, 20)


def test_cholesky_matches_lapack():
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(0)
    for _ in range(50):
        a = rng.normal(size=(6, 6)).astype(np.float64)
        h = (a @ a.T + 6 * np.eye(6)).astype(np.float32)
        lo = np.tril(h)
        L, info = O.potrf6(lo)
        assert info == 0
        c, info_ref = lapack.spotrf(h, lower=1)
        assert info_ref == 0
        np.testing.assert_allclose(np.tril(L), np.tril(c), rtol=2e-5, atol=2e-5)
        b = rng.normal(size=6).astype(np.float32)
        x = O.potrs6(L, b)
        x_ref, info_s = lapack.spotrs(c, b, lower=1)
        np.testing.assert_allclose(x, x_ref, rtol=1e-4, atol=1e-5)
    # not positive definite -> info > 0 (SingularHessian, TW_paDIC_ICGN2D_CPU.cpp:688-693)
    h = np.diag([1, 1, -1, 1, 1, 1]).astype(np.float32)
    _, info = O.potrf6(h)
    assert info == 3
    assert lapack.spotrf(h, lower=1)[1] == 3


@pytest.mark.parametrize("shape", [(32, 32), (40, 40), (20, 20), (58, 58), (30, 42)])
def test_dft_matches_numpy(shape):
    rng = np.random.default_rng(1)
    x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    np.testing.assert_allclose(O.dft2d(x), np.fft.fft2(x), rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(O.dft2d(x, inverse=True), np.fft.ifft2(x) * x.size, rtol=1e-10, atol=1e-9)


def test_gradients_and_lut_known_answers():
    rng = np.random.default_rng(2)
    H, W = 24, 28
    ref = rng.integers(0, 256, (H, W), dtype=np.uint8)
    tar = rng.integers(0, 256, (H, W), dtype=np.uint8)
    sx, sy, rw, rh = 2, 3, 20, 16
    Rx, Ry, Tx, Ty, Txy, lut = O.precompute_f32(ref, tar, sx, sy, rw, rh)
    r = ref.astype(np.float64)
    t = tar.astype(np.float64)
    ys, xs = np.mgrid[sy:sy + rh, sx:sx + rw]
    np.testing.assert_array_equal(Rx, 0.5 * (r[ys, xs + 1] - r[ys, xs - 1]))
    np.testing.assert_array_equal(Ry, 0.5 * (r[ys + 1, xs] - r[ys - 1, xs]))
    np.testing.assert_array_equal(Txy, 0.25 * (t[ys + 1, xs + 1] - t[ys - 1, xs + 1] - t[ys + 1, xs - 1]
                                               + t[ys - 1, xs - 1]))
    # LUT: p(fx, fy) = sum_k sum_n a[k][n] fy^k fx^n reproduces corner values and
    # derivatives of the Hermite patch (TW_utils.cpp:604-700)
    for i, j in [(0, 0), (5, 7), (rh - 2, rw - 2)]:
        a = lut[i, j].astype(np.float64)

        def p(fx, fy):
            return sum(a[k, n] * fy ** k * fx ** n for k in range(4) for n in range(4))

        def px(fx, fy):
            return sum(a[k, n] * fy ** k * n * fx ** (n - 1) for k in range(4) for n in range(1, 4))

        for dy in (0, 1):
            for dx in (0, 1):
                assert p(dx, dy) == pytest.approx(t[sy + i + dy, sx + j + dx], abs=1e-4)
                assert px(dx, dy) == pytest.approx(Tx[i + dy, j + dx], abs=1e-4)
    # never-written last row/column and the zeroed corner
    assert not lut[rh - 1].any() and not lut[:, rw - 1].any()


def test_lut_equals_catmull_rom_kernel():
    """The Hermite bicubic LUT with central differences is algebraically the
    separable Catmull-Rom kernel on the 4x4 neighbourhood; the fast IC-GN
    kernel relies on this identity."""
    rng = np.random.default_rng(3)
    H, W = 20, 20
    tar = rng.integers(0, 256, (H, W), dtype=np.uint8)
    sx = sy = 2
    rw = rh = 14
    *_, lut = O.precompute_f32(tar, tar, sx, sy, rw, rh)
    t = tar.astype(np.float64)

    def cr(x):
        x2, x3 = x * x, x * x * x
        return np.array([-0.5 * x3 + x2 - 0.5 * x, 1.5 * x3 - 2.5 * x2 + 1, -1.5 * x3 + 2 * x2 + 0.5 * x,
                         0.5 * x3 - 0.5 * x2])

    for _ in range(200):
        i, j = rng.integers(0, rh - 1), rng.integers(0, rw - 1)
        fx, fy = rng.random(2)
        a = lut[i, j].astype(np.float64)
        v_lut = sum(a[k, n] * fy ** k * fx ** n for k in range(4) for n in range(4))
        nb = t[sy + i - 1:sy + i + 3, sx + j - 1:sx + j + 3]
        v_cr = cr(fy) @ nb @ cr(fx)
        assert v_lut == pytest.approx(v_cr, abs=1e-9)


def _exact_peak(ref, tar, py, px, r):
    """Integer displacement from the exact integer correlation surface with the
    reference's first-maximum rule and wrap (TW_paDIC_FFTCC2D_CPU.cpp:300-325)."""
    c = O.exact_surface(ref, tar, py, px, r).ravel()
    k = int(np.argmax(c))  # numpy argmax returns the first maximum
    n = 2 * r
    iu, iv = k % n, k // n
    return (iu - n if iu > r else iu), (iv - n if iv > r else iv)


def test_fftcc_integer_translation_known_answer():
    """The peak is the exact correlation maximum (first-max rule).  For a
    translated speckle image it lies within one pixel of the imposed shift:
    the unpadded circular window (TW_paDIC_FFTCC2D_CPU.cpp:24-25) loses overlap
    as the shift grows, which biases broad speckle peaks towards zero."""
    rng = np.random.default_rng(4)
    inten = synth.speckle_intensity(160, 160, 700, rng)
    ref = np.clip(np.rint(inten), 0, 255).astype(np.uint8)
    poi = np.array([[y, x] for y in range(40, 121, 20) for x in range(40, 121, 20)], np.int32)
    for du, dv in [(3, -2), (-4, 4), (0, 0), (2, 3)]:
        tar = np.roll(ref, shift=(dv, du), axis=(0, 1))
        for prec in ("f32", "f64"):
            u, v, z, st = O.fftcc(ref, tar, poi, 16, precision=prec)
            assert (st == 0).all()
            for i, (py, px) in enumerate(poi):
                assert (u[i], v[i]) == _exact_peak(ref, tar, py, px, 16)
            near = (np.abs(u - du) <= 1) & (np.abs(v - dv) <= 1)
            assert near.mean() >= 0.9
            if du == dv == 0:
                assert (u == 0).all() and (v == 0).all() and (z > 0.99).all()


def test_fftcc_dark_subset_leaves_outputs_untouched():
    ref = np.full((64, 64), 40, np.uint8)
    tar = np.full((64, 64), 40, np.uint8)
    poi = np.array([[32, 32]], np.int32)
    u, v, z, st = O.fftcc(ref, tar, poi, 8, init=-7.0)
    assert st[0] == 1 and u[0] == -7 and v[0] == -7 and z[0] == -7


def test_icgn_recovers_imposed_affine_field(small):
    pair, g = small
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u, v, z, st = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    assert (st == 0).all()
    p6, it, fl = O.icgn(pair.ref, pair.tar, g, poi, u, v)
    X, Y = poi[:, 1].astype(float), poi[:, 0].astype(float)
    uu, vv = pair.field(X, Y)
    ok = fl == 0
    assert ok.mean() > 0.95
    assert np.abs(p6[ok, 0] - uu[ok]).max() < 0.05
    assert np.abs(p6[ok, 3] - vv[ok]).max() < 0.05
    gx = pair.grad(X, Y)
    assert np.abs(p6[ok, 1] - gx[0][ok]).max() < 5e-3
    assert np.abs(p6[ok, 5] - gx[3][ok]).max() < 5e-3
    assert (it[ok] >= 1).all() and (it[ok] <= g.max_iter).all()
    # FP32 restatement vs FP64 oracle
    p6d, itd, fld = O.icgn(pair.ref, pair.tar, g, poi, u, v, precision="f64")
    both = ok & (fld == 0) & (it == itd)
    assert np.abs(p6[both] - p6d[both]).max(axis=0)[[0, 3]].max() < 1e-3


def test_icgn_flags():
    # OutofROI: a POI whose warped subset leaves the ROI; DarkSubset: zero reference
    pair, g = synth.small_case()
    poi = np.array([[80, 96], [80, 96]], np.int32)
    u0 = np.array([0.0, 200.0], np.float32)
    v0 = np.zeros(2, np.float32)
    p6, it, fl = O.icgn(pair.ref, pair.tar, g, poi, u0, v0, iters_init=-1)
    assert fl[1] == 4 and it[1] == -1  # aborted in the first pass: counter untouched
    assert p6[1, 0] == 200.0
    dark = np.zeros_like(pair.ref)
    p6, it, fl = O.icgn(dark, pair.tar, g, poi[:1], u0[:1], v0[:1], iters_init=-1)
    assert fl[0] == 1 and it[0] == -1


def test_golden_fixture_regression():
    path = os.path.join(GOLDEN, "small_case.npz")
    d = np.load(path)
    g = synth.Geometry(*[int(x) for x in d["geom"][:9]], int(d["geom"][9]), float(d["delta_p"]))
    u, v, z, st = O.fftcc(d["ref"], d["tar"], d["poi"], g.subset_r)
    np.testing.assert_array_equal(u, d["fftcc_u"])
    np.testing.assert_array_equal(v, d["fftcc_v"])
    np.testing.assert_allclose(z, d["fftcc_zncc"], rtol=0, atol=2e-6)
    p6, it, fl = O.icgn(d["ref"], d["tar"], g, d["poi"], u, v)
    np.testing.assert_array_equal(fl, d["icgn_flags"])
    np.testing.assert_array_equal(it, d["icgn_iters"])
    np.testing.assert_allclose(p6, d["icgn_p6"], rtol=0, atol=1e-6)


def test_golden_fixture_regression_bspline():
    """The oracle's B-spline IC-GN on the stored inputs, from its own FFT-CC
    guesses, against tests/golden/small_case_bspline.npz."""
    d = np.load(os.path.join(GOLDEN, "small_case.npz"))
    b = np.load(os.path.join(GOLDEN, "small_case_bspline.npz"))
    g = synth.Geometry(*[int(x) for x in d["geom"][:9]], int(d["geom"][9]), float(d["delta_p"]))
    p6, it, fl = O.icgn(d["ref"], d["tar"], g, d["poi"], d["fftcc_u"], d["fftcc_v"], interp="bspline")
    np.testing.assert_array_equal(fl, b["icgn_flags"])
    np.testing.assert_array_equal(it, b["icgn_iters"])
    np.testing.assert_allclose(p6, b["icgn_p6"], rtol=0, atol=1e-6)
    # a different interpolant from the bicubic fixture's
    assert np.abs(p6 - d["icgn_p6"]).max() > 1e-5
