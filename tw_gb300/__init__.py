"""GB300 (sm_103a) implementation of TW_Engine's 2D DIC hot path.

Integer-pixel FFT cross-correlation followed by first-order IC-GN with bicubic
interpolation, behind the C ABI of include/tw_dic.h (libtwdic.so) and a
Python mirror of the reference's cuFFTCC2D / cuICGN2D class interfaces.
"""
from ._lib import (INTERP_BICUBIC, INTERP_BSPLINE, MEM_DEVICE, MEM_HOST, PATH_FAST, PATH_PLAIN, SAMPLER_LUT, SAMPLER_NBHD,  # noqa: F401
                   SAMPLER_WINDOW, TWDICError, load)
from .dic import DICBatch, DICFrame, ICGN_FLAGS, cuFFTCC2D, cuICGN2D, make_params, num_pois, poi_positions  # noqa: F401

__all__ = ["cuFFTCC2D", "cuICGN2D", "DICFrame", "make_params", "num_pois", "poi_positions", "TWDICError",
           "PATH_FAST", "PATH_PLAIN", "MEM_HOST", "MEM_DEVICE", "ICGN_FLAGS", "load"]
