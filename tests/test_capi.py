"""CPU tests of the C ABI: the library loads, exports every symbol that
include/tw_dic.h declares, and the host-side logic (POI grid, parameter
validation with the reference's error conditions) works without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from tw_gb300 import _lib, dic
from tw_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tw_dic.h")


@pytest.fixture(scope="module")
def lib():
    build()
    return _lib.load()


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"TWDIC_API\s+[\w\s\*]+?\b(twdic_\w+)\s*\(", text)))


def test_header_declares_what_the_binding_binds():
    syms = header_symbols()
    assert len(syms) >= 20
    assert set(syms) == set(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for s in header_symbols():
        assert hasattr(lib, s), s
    assert lib.twdic_abi_version() == 2


def test_params_struct_matches_header(lib):
    # 14 int32 fields + 1 float = 60 bytes, no padding
    assert ctypes.sizeof(_lib.Params) == 60
    text = open(HEADER).read()
    body = text[text.index("typedef struct twdic_params"):text.index("} twdic_params;")]
    fields = re.findall(r"\b(\w+)\s*[,;]", re.sub(r"/\*.*?\*/", "", body, flags=re.S))
    names = [f[0] for f in _lib.Params._fields_]
    assert fields == names


@pytest.mark.parametrize("roi,r,g,m", [(510, 16, 10, 20), (2046, 20, 5, 20), (190, 10, 7, 12), (64, 3, 1, 0)])
def test_num_pois_and_grid_match_oracle(lib, roi, r, g, m):
    p = dic.make_params(roi + 2, roi + 2, 1, 1, roi, roi, r, r, g, g, m, m)
    nx, ny = dic.num_pois(p)
    onx, ony, rc = O.num_pois(roi, roi, r, g, m)
    assert (nx, ny) == (onx, ony)
    np.testing.assert_array_equal(dic.poi_positions(p), O.poi_positions(1, 1, nx, ny, m, r, g))


@pytest.mark.parametrize("rw,rh,rx,ry,g,m", [(168, 148, 12, 8, 9, 12), (300, 200, 5, 20, 7, 3), (97, 131, 16, 9, 4, 0)])
def test_non_square_grid_matches_oracle(lib, rw, rh, rx, ry, g, m):
    """Subset half width and height differ (ComputePOIPositions_s takes both,
    TW_utils.cpp:29-94): the library's POI count and grid equal the oracle's."""
    p = dic.make_params(rw + 2, rh + 2, 1, 1, rw, rh, rx, ry, g, g, m, m)
    nx, ny = dic.num_pois(p)
    onx, ony, rc = O.num_pois(rw, rh, rx, g, m, ry=ry)
    assert rc == 0 and (nx, ny) == (onx, ony)
    np.testing.assert_array_equal(dic.poi_positions(p), O.poi_positions(1, 1, nx, ny, m, rx, g, ry=ry))


def test_validation_errors_without_gpu(lib):
    # "Number of POIs is below 0!" (cuFFTCC2D ctor, TW_paDIC_cuFFTCC2D.cu:189-190)
    p = dic.make_params(64, 64, 0, 0, 64, 64, 20, 20, 5, 5, 20, 20)
    with pytest.raises(_lib.TWDICError) as e:
        dic.num_pois(p)
    assert e.value.code == -2
    h = ctypes.c_void_p()
    assert lib.twdic_fftcc_create(ctypes.byref(p), ctypes.byref(h)) == -2
    assert not h.value
    # one-pixel border for the gradients (TW_utils.cpp:254-257)
    p = dic.make_params(128, 128, 0, 0, 128, 128, 10, 10, 5, 5, 3, 3)
    assert lib.twdic_frame_create(ctypes.byref(p), ctypes.byref(h)) == -3
    assert b"boundary" in lib.twdic_last_error()
    # subset radius beyond the library's limit
    p = dic.make_params(256, 256, 1, 1, 254, 254, 32, 32, 5, 5, 3, 3)
    assert lib.twdic_frame_create(ctypes.byref(p), ctypes.byref(h)) == -7
    # ROI outside the image, bad path, NULL arguments
    p = dic.make_params(128, 128, 10, 10, 128, 128, 10, 10, 5, 5, 3, 3)
    assert lib.twdic_fftcc_create(ctypes.byref(p), ctypes.byref(h)) == -1
    p = dic.make_params(128, 128, 1, 1, 126, 126, 10, 10, 5, 5, 3, 3, path=9)
    assert lib.twdic_frame_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert lib.twdic_fftcc_create(None, ctypes.byref(h)) == -1
    assert lib.twdic_frame_process(None, None, 0, 0, None, None, None, None, None, None, 0) == -1
    assert lib.twdic_icgn_create(ctypes.byref(p), 0, 3, ctypes.byref(h)) in (-1, -2)
