"""TEST INFRASTRUCTURE ONLY: compile the reference's own CPU DIC sources into
oracle/_ref/libtwref.so, a second oracle used to pin the restatement in
tw_oracle.cpp.

The reference's FFT-CC and IC-GN CPU classes are compiled from the files where
they lie in the reference checkout (never copied, never edited):

    TW/TW_Engine/TW_paDIC_FFTCC2D.cpp      Fftcc2D (POI count)
    TW/TW_Engine/TW_paDIC_FFTCC2D_CPU.cpp  Fftcc2D_CPU (FFT-CC)
    TW/TW_Engine/TW_paDIC_ICGN2D.cpp       ICGN2D
    TW/TW_Engine/TW_paDIC_ICGN2D_CPU.cpp   ICGN2D_CPU (IC-GN)
    TW/TW_Engine/TW_utils.cpp              POI grid, gradients, LUTs

together with the stand-ins in oracle/ref_shim/ for what the reference links
from outside and this machine lacks: FFTW3 (a double-precision direct DFT
rounded to float), MKL's LAPACKE (row-major wrappers over the Fortran LAPACK
that scipy links, handed over at load time), OpenCV's cv::Mat (an 8-bit image
view), Qt's qDebug (discarded) and Windows.h (one type).  The reference
includes OpenCV through Windows paths ("opencv2\\opencv.hpp"); forwarding
headers with those literal file names are written into oracle/_ref/inc.
`-fpermissive` accepts the MSVC-only extra qualification at
TW_paDIC_FFTCC2D.h:65.  The CUDA toolkit's headers supply the CUDA types that
the reference's headers name (no CUDA code is compiled or called).

The reference checkout exists only on the development machine, so this build
and the tests that use it are skipped elsewhere; the fixtures it generates
(tests/golden/make_ref_golden.py) travel instead.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "ref_shim")
OUT = os.path.join(HERE, "_ref")
INC = os.path.join(OUT, "inc")
LIB = os.path.join(OUT, "libtwref.so")
REF_ROOT = os.environ.get("TWREF_ROOT", "/root/reference")
ENGINE = os.path.join(REF_ROOT, "TW", "TW_Engine")
CUDA_INC = "/usr/local/cuda/include"

REF_SOURCES = ["TW_paDIC_FFTCC2D.cpp", "TW_paDIC_FFTCC2D_CPU.cpp", "TW_paDIC_ICGN2D.cpp", "TW_paDIC_ICGN2D_CPU.cpp",
               "TW_utils.cpp"]
SHIM_SOURCES = ["ref_shim.cpp", "ref_driver.cpp"]
# the reference's OpenCV includes, by their literal (backslash) names
OPENCV_NAMES = ["opencv2\\opencv.hpp", "opencv2\\core.hpp", "opencv2\\highgui.hpp", "opencv2\\imgproc.hpp",
                "opencv2\\core\\cuda.hpp"]
CXXFLAGS = ["-O2", "-std=c++14", "-fopenmp", "-ffp-contract=off", "-fPIC", "-fpermissive", "-w",
            "-include", os.path.join(SHIM, "prelude.h")]


def available() -> bool:
    return all(os.path.exists(os.path.join(ENGINE, s)) for s in REF_SOURCES) and os.path.isdir(CUDA_INC)


def build(force: bool = False) -> str:
    if not available():
        raise FileNotFoundError(f"reference sources not found under {ENGINE}")
    os.makedirs(INC, exist_ok=True)
    for name in OPENCV_NAMES:
        path = os.path.join(INC, name)
        with open(path, "w") as f:
            f.write(f'#include "{os.path.join(SHIM, "opencv_standin.hpp")}"\n')
    srcs = [os.path.join(ENGINE, s) for s in REF_SOURCES] + [os.path.join(SHIM, s) for s in SHIM_SOURCES]
    newest = max(os.path.getmtime(p) for p in srcs + [os.path.join(SHIM, h) for h in os.listdir(SHIM)])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    objs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        subprocess.check_call(["g++", *CXXFLAGS, "-I", INC, "-I", SHIM, "-I", ENGINE, "-I", CUDA_INC, "-c", s,
                               "-o", o])
        objs.append(o)
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    """Load the reference build and hand it scipy's Fortran LAPACK."""
    global _lib
    if _lib is None:
        from scipy.linalg import cython_lapack
        L = ctypes.CDLL(build())
        get = ctypes.pythonapi.PyCapsule_GetPointer
        get.restype = ctypes.c_void_p
        get.argtypes = [ctypes.py_object, ctypes.c_char_p]
        ptrs = []
        for name in ("spotrf", "spotrs"):
            cap = cython_lapack.__pyx_capi__[name]
            cname = ctypes.pythonapi.PyCapsule_GetName
            cname.restype = ctypes.c_char_p
            cname.argtypes = [ctypes.py_object]
            ptrs.append(get(cap, cname(cap)))
        L.twref_set_lapack(ctypes.c_void_p(ptrs[0]), ctypes.c_void_p(ptrs[1]))
        _lib = L
    return _lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fftcc(ref, tar, g, rx=None, ry=None, multicore=True):
    """The reference's Fftcc2D_CPU on a whole POI grid of geometry g
    (fields img_w, img_h, start_x, start_y, roi_w, roi_h, subset_r, grid,
    margin).  Returns (poi_yx, u, v, zncc)."""
    import numpy as np
    ref = np.ascontiguousarray(ref, np.uint8)
    tar = np.ascontiguousarray(tar, np.uint8)
    rx = g.subset_r if rx is None else rx
    ry = (getattr(g, "subset_ry", 0) or rx) if ry is None else ry
    cap = (g.roi_w // max(g.grid, 1) + 2) * (g.roi_h // max(g.grid, 1) + 2)
    poi = np.zeros((cap, 2), np.int32)
    u, v, z = (np.zeros(cap, np.float32) for _ in range(3))
    L = lib()
    n = L.twref_fftcc(_p(ref), _p(tar), g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, rx, ry, g.grid,
                      g.grid, g.margin, g.margin, int(multicore), cap, _p(poi), _p(u), _p(v), _p(z))
    if n < 0:
        raise ValueError(f"reference FFT-CC rejected the geometry ({n})")
    return poi[:n].copy(), u[:n].copy(), v[:n].copy(), z[:n].copy()


def icgn(ref, tar, g, poi_yx, u0, v0, interp="bicubic", multicore=True):
    """The reference's ICGN2D_CPU over the POIs from guesses (u0, v0).
    Returns (u, v, iters, flags)."""
    import numpy as np
    ref = np.ascontiguousarray(ref, np.uint8)
    tar = np.ascontiguousarray(tar, np.uint8)
    poi_yx = np.ascontiguousarray(poi_yx, np.int32)
    n = len(poi_yx)
    u = np.ascontiguousarray(u0, np.float32).copy()
    v = np.ascontiguousarray(v0, np.float32).copy()
    iters = np.zeros(n, np.int32)
    flags = np.zeros(n, np.uint8)
    ry = getattr(g, "subset_ry", 0) or g.subset_r
    L = lib()
    fn = L.twref_icgn
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 10 + [ctypes.c_float, ctypes.c_int,
                                                                               ctypes.c_int] + [ctypes.c_void_p] * 5
    rc = fn(_p(ref), _p(tar), g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, ry, n,
            g.max_iter, g.delta_p, {"bicubic": 0, "bspline": 1}[interp], int(multicore), _p(poi_yx), _p(u), _p(v),
            _p(iters), _p(flags))
    if rc != 0:
        raise RuntimeError("the reference's IC-GN did not reproduce its own outputs")
    return u, v, iters, flags
