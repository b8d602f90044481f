"""The header-only C++ facade (include/tw_dic.hpp) compiles against the C ABI
and, on a GPU, gives the same results as the Python entry points."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tw_gb300 import dic, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp")
CUDA_INC = "/usr/local/cuda/include"


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_facade_compiles():
    r = subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Wextra", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        "-I", CUDA_INC, SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_matches_python_entry_points(tmp_path):
    lib_dir = os.path.join(ROOT, "tw_gb300")
    exe = str(tmp_path / "facade_demo")
    r = subprocess.run([_gxx(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC, SRC,
                        "-o", exe, "-L", lib_dir, "-ltwdic", f"-Wl,-rpath,{lib_dir}", "-L", "/usr/local/cuda/lib64",
                        "-lcudart"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pair, g = synth.small_case()
    (tmp_path / "ref.raw").write_bytes(pair.ref.tobytes())
    (tmp_path / "tar.raw").write_bytes(pair.tar.tobytes())
    out = str(tmp_path / "out.raw")
    r = subprocess.run([exe, str(g.img_w), str(g.img_h), str(g.subset_r), str(g.grid), str(g.margin),
                        str(tmp_path / "ref.raw"), str(tmp_path / "tar.raw"), out], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw[:4], np.int32)[0])
    o = 8
    def take(dt, cnt):
        nonlocal o
        a = np.frombuffer(raw[o:o + np.dtype(dt).itemsize * cnt], dt)
        o += np.dtype(dt).itemsize * cnt
        return a
    poi = take(np.int32, 2 * n).reshape(n, 2)
    U, V, Z = take(np.float32, n), take(np.float32, n), take(np.float32, n)
    u, v, it, fl = take(np.float32, n), take(np.float32, n), take(np.int32, n), take(np.uint8, n)
    p6 = take(np.float32, 6 * n).reshape(n, 6)
    gu, gv = take(np.float32, n), take(np.float32, n)
    # Python entry points on the same pair
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin)
    np.testing.assert_array_equal(f.POIPositions(), poi)
    PU, PV, PZ = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(PU, PV, PZ, pair.tar)
    np.testing.assert_array_equal(U, PU.ravel())
    np.testing.assert_array_equal(V, PV.ravel())
    np.testing.assert_array_equal(Z, PZ.ravel())
    fr = dic.DICFrame(dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r,
                                      g.subset_r, g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p))
    fr.set_reference(pair.ref)
    w = fr.alloc_outputs()
    fr.process(pair.tar, **w)
    np.testing.assert_array_equal(u, w["u"])
    np.testing.assert_array_equal(v, w["v"])
    np.testing.assert_array_equal(p6, w["p6"])
    np.testing.assert_array_equal(fl, w["flags"])
    np.testing.assert_array_equal(it, w["iters"])
    np.testing.assert_array_equal(gu, w["u"])
    np.testing.assert_array_equal(gv, w["v"])
    # the B-spline flag against a B-spline frame
    bu, bv, bit, bfl = take(np.float32, n), take(np.float32, n), take(np.int32, n), take(np.uint8, n)
    assert o == len(raw)
    from tw_gb300 import INTERP_BSPLINE
    fb = dic.DICFrame(dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r,
                                      g.subset_r, g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p))
    fb.set_interpolation(INTERP_BSPLINE)
    fb.set_reference(pair.ref)
    wb = fb.alloc_outputs()
    fb.process(pair.tar, **wb)
    np.testing.assert_array_equal(bu, wb["u"])
    np.testing.assert_array_equal(bv, wb["v"])
    np.testing.assert_array_equal(bit, wb["iters"])
    np.testing.assert_array_equal(bfl, wb["flags"])
    assert not np.array_equal(bu, u)  # a different interpolant
