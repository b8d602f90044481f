"""TEST INFRASTRUCTURE ONLY: ctypes loader for the C++ oracle (tw_oracle.cpp).

The oracle is a CPU restatement of the reference's CPU path (see the header of
tw_oracle.cpp for the file:line map); tests/test_ref_pin.py pins it to the
outputs of the reference's own sources (oracle/build_ref.py).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "tw_oracle.cpp")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall"]

FLAG_NAMES = ("Success", "DarkSubset", "SingularHessian", "SingularWarp", "OutofROI")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no FMA contraction, OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_pois(roi_w, roi_h, r, grid, margin, ry=None):
    """r: subset half width (and height unless ry is given)."""
    nx, ny = ctypes.c_int(), ctypes.c_int()
    rc = lib().or_num_pois(roi_w, roi_h, r, r if ry is None else ry, grid, grid, margin, margin, ctypes.byref(nx),
                           ctypes.byref(ny))
    return nx.value, ny.value, rc


def poi_positions(start_x, start_y, nx, ny, margin, r, grid, ry=None):
    yx = np.zeros((ny * nx, 2), dtype=np.int32)
    lib().or_poi_positions(start_x, start_y, nx, ny, margin, margin, r, r if ry is None else ry, grid, grid, _p(yx))
    return yx


def precompute_f32(ref, tar, sx, sy, rw, rh):
    H, W = ref.shape
    out = [np.zeros((rh, rw), np.float32) for _ in range(5)]
    lut = np.zeros((rh, rw, 4, 4), np.float32)
    rc = lib().or_precompute_f32(_p(ref), _p(tar), W, H, sx, sy, rw, rh, *[_p(o) for o in out], _p(lut))
    if rc != 0:
        raise ValueError("ROI leaves no one-pixel border")
    return (*out, lut)


def fftcc(ref, tar, poi_yx, r, precision="f32", nthreads=0, init=0.0, ry=None):
    """Integer-pixel FFT-CC.  Returns (u, v, zncc, status) where status is 0 ok,
    1 dark subset (outputs left at `init`), 2 window outside the image.
    r: window half width (and height unless ry is given)."""
    ref = np.ascontiguousarray(ref, np.uint8)
    tar = np.ascontiguousarray(tar, np.uint8)
    poi_yx = np.ascontiguousarray(poi_yx, np.int32)
    H, W = ref.shape
    n = poi_yx.shape[0]
    dt = np.float32 if precision == "f32" else np.float64
    u = np.full(n, init, dt)
    v = np.full(n, init, dt)
    z = np.full(n, init, dt)
    st = np.zeros(n, np.uint8)
    fn = lib().or_fftcc_f32 if precision == "f32" else lib().or_fftcc_f64
    fn(_p(ref), _p(tar), W, H, _p(poi_yx), n, r, r if ry is None else ry, nthreads, _p(u), _p(v), _p(z), _p(st))
    return u, v, z, st


def exact_surface(ref, tar, py, px, r, ry=None):
    """Exact integer circular correlation sum f(x) g(x + k) of the [2ry][2rx]
    windows at (py, px), indexed [ky][kx]."""
    H, W = ref.shape
    ry = r if ry is None else ry
    c = np.zeros((2 * ry, 2 * r), np.int64)
    lib().or_fftcc_exact_surface(_p(np.ascontiguousarray(ref)), _p(np.ascontiguousarray(tar)), W, int(py), int(px),
                                 int(r), int(ry), _p(c))
    return c


def candidate_lower_bound(ref, tar, py, px, r, window=0.008):
    """Number of shifts whose exact ZNCC lies within `window` of the exact
    peak.  With the tensor-core FFT-CC's surface error below 1e-3, every such
    shift is among its candidates (those within 0.01 of the approximate
    peak), so this is a lower bound on that candidate count."""
    c = exact_surface(ref, tar, py, px, r).astype(np.float64)
    f = ref[py - r:py + r, px - r:px + r].astype(np.float64)
    g = tar[py - r:py + r, px - r:px + r].astype(np.float64)
    n2 = (2 * r) ** 2
    z = (c - n2 * f.mean() * g.mean()) / np.sqrt(((f - f.mean()) ** 2).sum() * ((g - g.mean()) ** 2).sum())
    return int((z >= z.max() - window).sum())


def icgn(ref, tar, geom, poi_yx, u0, v0, precision="f32", nthreads=0, iters_init=0, interp="bicubic"):
    """IC-GN over all POIs.  Returns (p6 [n,6], iters [n], flags [n]).
    interp: "bicubic" (the Hermite LUT) or "bspline" (the B-spline LUT)."""
    ref = np.ascontiguousarray(ref, np.uint8)
    tar = np.ascontiguousarray(tar, np.uint8)
    poi_yx = np.ascontiguousarray(poi_yx, np.int32)
    H, W = ref.shape
    n = poi_yx.shape[0]
    dt = np.float32 if precision == "f32" else np.float64
    p6 = np.zeros((n, 6), dt)
    p6[:, 0] = u0
    p6[:, 3] = v0
    iters = np.full(n, iters_init, np.int32)
    flags = np.zeros(n, np.uint8)
    fn = lib().or_icgn_f32 if precision == "f32" else lib().or_icgn_f64
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 8 + [ctypes.c_void_p, ctypes.c_int,
                                                                               ctypes.c_int, ctypes.c_float,
                                                                               ctypes.c_int, ctypes.c_void_p,
                                                                               ctypes.c_void_p, ctypes.c_void_p,
                                                                               ctypes.c_int]
    mode = {"bicubic": 0, "bspline": 1}[interp]
    ry = getattr(geom, "subset_ry", 0) or geom.subset_r
    rc = fn(_p(ref), _p(tar), W, H, geom.start_x, geom.start_y, geom.roi_w, geom.roi_h, geom.subset_r,
            ry, _p(poi_yx), n, geom.max_iter, geom.delta_p, nthreads, _p(p6), _p(iters), _p(flags), mode)
    if rc != 0:
        raise ValueError("ROI leaves no one-pixel border")
    return p6, iters, flags


def potrf6(a):
    a = np.ascontiguousarray(a, np.float32).copy()
    info = lib().or_potrf6_f32(_p(a))
    return a, info


def potrs6(l, b):
    b = np.ascontiguousarray(b, np.float32).copy()
    lib().or_potrs6_f32(_p(np.ascontiguousarray(l, np.float32)), _p(b))
    return b


def dft2d(x, inverse=False):
    x = np.asarray(x, np.complex128)
    h, w = x.shape
    re = np.ascontiguousarray(x.real)
    im = np.ascontiguousarray(x.imag)
    ro = np.zeros_like(re)
    io = np.zeros_like(im)
    lib().or_dft2d_f64(_p(re), _p(im), h, w, 1 if inverse else 0, _p(ro), _p(io))
    return ro + 1j * io


def max_threads():
    return lib().or_max_threads()


def bspline_lut(tar, sx, sy, rw, rh):
    """The target's B-spline coefficient LUT, float32 [rh, rw, 16]."""
    tar = np.ascontiguousarray(tar, np.uint8)
    H, W = tar.shape
    out = np.zeros((rh, rw, 16), np.float32)
    fn = lib().or_bspline_lut_f32
    fn.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 6 + [ctypes.c_void_p]
    fn(_p(tar), W, H, sx, sy, rw, rh, _p(out))
    return out
