"""Host-side mirror of TW_Engine's FFT-CC and IC-GN class interfaces.

Class and method names, argument order and meaning follow the reference
(paths relative to the TWANG006/TW project root):

* ``cuFFTCC2D``  -- TW/TW_Engine/TW_paDIC_cuFFTCC2D.h:18-170 (whole-image
  constructor order imgW, imgH, roiW, roiH, startX, startY, ...), with the
  host-side ``InitializeFFTCC / ComputeFFTCC / DestroyFFTCC`` and device-side
  ``cuInitializeFFTCC / cuComputeFFTCC / cuDestroyFFTCC`` pairs.
* ``cuICGN2D``   -- TW/TW_Engine/TW_paDIC_cuICGN2D.h:9-57 (``cuInitialize``,
  ``cuCompute``, ``cuFinalize``) and, for callers of the MKL path,
  ``ICGN2D_Algorithm`` of TW/TW_Engine/TW_paDIC_ICGN2D_CPU.h:56-85.
* ``DICFrame``   -- one frame of FFT-CC then IC-GN on the same target with the
  reference cached (TW/TW_Core/fftcctworkerthread.cpp:399-481).

Every call goes through libtwdic.so's C ABI; host arrays are numpy, device
arrays are torch CUDA tensors (plumbing only).  Constructor errors raise
TWDICError, as the reference constructors throw std::logic_error.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import _lib
from ._lib import (INTERP_BICUBIC, INTERP_BSPLINE, MEM_DEVICE, MEM_HOST, PATH_FAST, PATH_PLAIN,  # noqa: F401
                   Params, TWDICError, check)

ICGN_FLAGS = ("Success", "DarkSubset", "SingularHessian", "SingularWarp", "OutofROI")


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr())
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return ctypes.c_void_p(x.ctypes.data)
    raise TypeError(f"unsupported buffer type {type(x)}")


def _mem(x) -> int:
    if _is_torch(x):
        return MEM_DEVICE if x.is_cuda else MEM_HOST
    return MEM_HOST


def _image(img, width: int, height: int):
    """uint8 image (numpy or torch) -> (pointer, stride, mem, owner).  Keep
    `owner` alive until the call that uses the pointer returns."""
    if _is_torch(img):
        if str(img.dtype) != "torch.uint8":
            raise TypeError("image must be uint8")
        if tuple(img.shape) != (height, width) or img.stride(1) != 1:
            raise ValueError(f"image must be ({height}, {width}) with unit column stride")
        return ctypes.c_void_p(img.data_ptr()), int(img.stride(0)), _mem(img), img
    a = np.asarray(img)
    if a.dtype != np.uint8 or a.shape != (height, width):
        raise ValueError(f"image must be uint8 of shape ({height}, {width})")
    a = np.ascontiguousarray(a)
    return ctypes.c_void_p(a.ctypes.data), width, MEM_HOST, a


def make_params(img_w, img_h, start_x, start_y, roi_w, roi_h, subset_x, subset_y, grid_x=1, grid_y=1,
                margin_x=0, margin_y=0, max_iterations=20, delta_p=0.001, path=PATH_FAST) -> Params:
    return Params(img_w, img_h, start_x, start_y, roi_w, roi_h, subset_x, subset_y, grid_x, grid_y, margin_x,
                  margin_y, max_iterations, delta_p, path)


def num_pois(params: Params) -> Tuple[int, int]:
    nx, ny = ctypes.c_int32(), ctypes.c_int32()
    check(_lib.load().twdic_num_pois(ctypes.byref(params), ctypes.byref(nx), ctypes.byref(ny)))
    return nx.value, ny.value


def poi_positions(params: Params) -> np.ndarray:
    nx, ny = num_pois(params)
    out = np.zeros((ny * nx, 2), np.int32)
    check(_lib.load().twdic_poi_positions(ctypes.byref(params), _ptr(out)))
    return out


class cuFFTCC2D:
    """Integer-pixel FFT-CC over a POI grid (cuFFTCC2D / Fftcc2D_CPU drop-in)."""

    def __init__(self, iImgWidth, iImgHeight, iROIWidth, iROIHeight, iStartX, iStartY, iSubsetX, iSubsetY,
                 iGridSpaceX, iGridSpaceY, iMarginX, iMarginY, path=PATH_FAST):
        self._lib = _lib.load()
        self.params = make_params(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX,
                                  iSubsetY, iGridSpaceX, iGridSpaceY, iMarginX, iMarginY, path=path)
        h = ctypes.c_void_p()
        check(self._lib.twdic_fftcc_create(ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        nx, ny = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.twdic_fftcc_num_pois(self._h, ctypes.byref(nx), ctypes.byref(ny)))
        self.m_iNumPOIX, self.m_iNumPOIY = nx.value, ny.value

    # inlined getters (TW_paDIC_FFTCC2D.h:99-103)
    def GetNumPOIsX(self):
        return self.m_iNumPOIX

    def GetNumPOIsY(self):
        return self.m_iNumPOIY

    def GetNumPOIs(self):
        return self.m_iNumPOIX * self.m_iNumPOIY

    def GetROISize(self):
        return self.params.roi_width * self.params.roi_height

    def GetImgSize(self):
        return self.params.img_width * self.params.img_height

    def POIPositions(self, device=None):
        """The POI grid as (y, x) pairs (g_cuHandle.m_d_iPOIXY)."""
        n = self.GetNumPOIs()
        if device is not None:
            import torch
            out = torch.empty((n, 2), dtype=torch.int32, device=device)
            check(self._lib.twdic_fftcc_poi_positions(self._h, _ptr(out), MEM_DEVICE))
            return out
        out = np.zeros((n, 2), np.int32)
        check(self._lib.twdic_fftcc_poi_positions(self._h, _ptr(out), MEM_HOST))
        return out

    def ResetRefImg(self, refImg):
        p, stride, mem, _keep = _image(refImg, self.params.img_width, self.params.img_height)
        check(self._lib.twdic_fftcc_reset_ref(self._h, p, stride, mem))

    def SetTarImg(self, tarImg):
        p, stride, mem, _keep = _image(tarImg, self.params.img_width, self.params.img_height)
        check(self._lib.twdic_fftcc_set_tar(self._h, p, stride, mem))

    # high-level (host) methods: outputs are [numPOIY][numPOIX] float32 arrays
    def InitializeFFTCC(self, refImg):
        self.ResetRefImg(refImg)
        shape = (self.m_iNumPOIY, self.m_iNumPOIX)
        return np.zeros(shape, np.float32), np.zeros(shape, np.float32), np.zeros(shape, np.float32)

    def ComputeFFTCC(self, fU, fV, fZNCC, tarImg, status=None):
        self.SetTarImg(tarImg)
        check(self._lib.twdic_fftcc_compute(self._h, _ptr(fU), _ptr(fV), _ptr(fZNCC), _ptr(status), MEM_HOST))

    def DestroyFFTCC(self, *unused):
        self.close()

    # low-level (device) methods: torch CUDA tensors of numPOIs floats
    def cuInitializeFFTCC(self, refImg, device="cuda"):
        import torch
        self.ResetRefImg(refImg)
        n = self.GetNumPOIs()
        return tuple(torch.zeros(n, dtype=torch.float32, device=device) for _ in range(3))

    def cuComputeFFTCC(self, f_d_U, f_d_V, f_d_ZNCC, tarImg, status=None):
        self.SetTarImg(tarImg)
        check(self._lib.twdic_fftcc_compute(self._h, _ptr(f_d_U), _ptr(f_d_V), _ptr(f_d_ZNCC), _ptr(status),
                                            MEM_DEVICE))

    def cuDestroyFFTCC(self, *unused):
        self.close()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_fftcc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class cuICGN2D:
    """First-order IC-GN over a POI list (cuICGN2D / ICGN2D_CPU drop-in)."""

    def __init__(self, iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY,
                 iNumberX, iNumberY, iNumIterations=20, fDeltaP=0.001, path=PATH_FAST, Iflag=INTERP_BICUBIC):
        self._lib = _lib.load()
        self.params = make_params(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX,
                                  iSubsetY, 1, 1, 0, 0, iNumIterations, fDeltaP, path)
        h = ctypes.c_void_p()
        check(self._lib.twdic_icgn_create(ctypes.byref(self.params), iNumberX, iNumberY, ctypes.byref(h)))
        if Iflag != INTERP_BICUBIC:
            check(self._lib.twdic_icgn_set_interpolation(h, Iflag))
        self._h = h
        self.m_iPOINumber = iNumberX * iNumberY
        self.last_p6 = None
        self.last_flags = None

    def ResetRefImg(self, refImg):
        p, stride, mem, _keep = _image(refImg, self.params.img_width, self.params.img_height)
        check(self._lib.twdic_icgn_reset_ref(self._h, p, stride, mem))

    cuInitialize = ResetRefImg
    Initialize = ResetRefImg

    def cuCompute(self, d_fTarImg, d_iPOIXY, d_fU, d_fV, d_dP=None, d_iIterationNums=None, d_flags=None):
        """Device arrays (torch CUDA tensors); d_fU, d_fV are updated in place."""
        p, stride, mem, _keep = _image(d_fTarImg, self.params.img_width, self.params.img_height)
        check(self._lib.twdic_icgn_compute(self._h, p, stride, _ptr(d_iPOIXY), MEM_DEVICE, _ptr(d_fU), _ptr(d_fV),
                                           _ptr(d_dP), _ptr(d_iIterationNums), _ptr(d_flags), MEM_DEVICE))

    def ICGN2D_Algorithm(self, fU, fV, iNumIterations, iPOIpos, tarImg):
        """ICGN2D_CPU::ICGN2D_Algorithm: host arrays, fU/fV/iNumIterations in/out.
        Returns (p6 [n,6], flags [n]) which the reference computes but drops."""
        n = self.m_iPOINumber
        p6 = np.zeros((n, 6), np.float32)
        flags = np.zeros(n, np.uint8)
        poi = np.ascontiguousarray(iPOIpos, np.int32)
        p, stride, mem, _keep = _image(tarImg, self.params.img_width, self.params.img_height)
        if mem != MEM_HOST:
            raise ValueError("ICGN2D_Algorithm takes host images")
        check(self._lib.twdic_icgn_compute(self._h, p, stride, _ptr(poi), MEM_HOST, _ptr(fU), _ptr(fV), _ptr(p6),
                                           _ptr(iNumIterations), _ptr(flags), MEM_HOST))
        self.last_p6, self.last_flags = p6, flags
        return p6, flags

    def cuFinalize(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_icgn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DICFrame:
    """FFT-CC then IC-GN per target frame, reference precompute cached."""

    def __init__(self, params: Params):
        self._lib = _lib.load()
        self.params = params
        h = ctypes.c_void_p()
        check(self._lib.twdic_frame_create(ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        nx, ny = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.twdic_frame_num_pois(self._h, ctypes.byref(nx), ctypes.byref(ny)))
        self.num_x, self.num_y = nx.value, ny.value
        self.n = nx.value * ny.value

    def poi_positions(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.int32)
        check(self._lib.twdic_frame_poi_positions(self._h, _ptr(out), MEM_HOST))
        return out

    def set_reference(self, ref):
        p, stride, mem, _keep = _image(ref, self.params.img_width, self.params.img_height)
        check(self._lib.twdic_frame_set_reference(self._h, p, stride, mem))

    def set_stream(self, stream):
        """Bind to a torch.cuda.Stream (or None for the handle's own stream)."""
        ptr = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
        check(self._lib.twdic_frame_set_stream(self._h, ptr))

    def set_interpolation(self, mode):
        """INTERP_BICUBIC (Hermite bicubic LUT, default) or INTERP_BSPLINE."""
        check(self._lib.twdic_frame_set_interpolation(self._h, mode))

    def set_tuning(self, icgn_threads=128, icgn_ctas_per_sm=0, icgn_sampler=0, fftcc_use_tc=1, icgn_chunk=0):
        """icgn_sampler: SAMPLER_WINDOW, SAMPLER_LUT or SAMPLER_NBHD;
        icgn_chunk: the IC-GN work layout (set_icgn_layout; None keeps it)."""
        check(self._lib.twdic_frame_set_tuning(self._h, icgn_threads, icgn_ctas_per_sm, icgn_sampler,
                                               fftcc_use_tc))
        if icgn_chunk is not None:
            self.set_icgn_layout(icgn_chunk)

    def set_icgn_layout(self, chunk):
        """0: one POI per CTA; > 0: one POI per warp over runs of `chunk`
        consecutive POIs (threads 128 to 1024, a table sampler)."""
        check(self._lib.twdic_frame_set_icgn_layout(self._h, chunk))

    def set_guess_mode(self, mode):
        """Batched calls: 1 skips FFT-CC and starts IC-GN from the u, v passed
        in (e.g. the last frame's); 0 (default) runs FFT-CC."""
        check(self._lib.twdic_frame_set_guess_mode(self._h, mode))

    def set_icgn_unroll(self, unroll):
        """Unrolling of the IC-GN sample loop: 2, 4 or 8 (default)."""
        check(self._lib.twdic_frame_set_icgn_unroll(self._h, unroll))

    def set_fftcc_twiddles(self, hi_lo):
        """1: FP16 hi + lo twiddles in the tensor-core FFT-CC, 0: hi only."""
        check(self._lib.twdic_frame_set_fftcc_twiddles(self._h, hi_lo))

    def set_fftcc_tuning(self, use_tc=1, groups=0, pois_per_group=0):
        check(self._lib.twdic_frame_set_fftcc_tuning(self._h, use_tc, groups, pois_per_group))

    def tuning(self) -> dict:
        t = _lib.Tuning()
        check(self._lib.twdic_frame_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in _lib.Tuning._fields_}

    def autotune(self, tar, cache_path=None) -> dict:
        """Time the launch shapes on this target, keep the fastest (see
        twdic_frame_autotune); `cache_path` reuses and records choices."""
        p, stride, mem_in, _keep = _image(tar, self.params.img_width, self.params.img_height)
        t = _lib.Tuning()
        check(self._lib.twdic_frame_autotune(self._h, p, stride, mem_in,
                                             None if cache_path is None else str(cache_path).encode(),
                                             ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in _lib.Tuning._fields_}

    def process(self, tar, u, v, zncc=None, p6=None, iters=None, flags=None):
        """Outputs are all numpy (host) or all torch CUDA tensors (device)."""
        p, stride, mem_in, _keep = _image(tar, self.params.img_width, self.params.img_height)
        mem_out = _mem(u)
        check(self._lib.twdic_frame_process(self._h, p, stride, mem_in, _ptr(u), _ptr(v), _ptr(zncc), _ptr(p6),
                                            _ptr(iters), _ptr(flags), mem_out))

    def alloc_outputs(self, device=None):
        n = self.n
        if device is None:
            return dict(u=np.zeros(n, np.float32), v=np.zeros(n, np.float32), zncc=np.zeros(n, np.float32),
                        p6=np.zeros((n, 6), np.float32), iters=np.zeros(n, np.int32), flags=np.zeros(n, np.uint8))
        import torch
        return dict(u=torch.zeros(n, dtype=torch.float32, device=device),
                    v=torch.zeros(n, dtype=torch.float32, device=device),
                    zncc=torch.zeros(n, dtype=torch.float32, device=device),
                    p6=torch.zeros((n, 6), dtype=torch.float32, device=device),
                    iters=torch.zeros(n, dtype=torch.int32, device=device),
                    flags=torch.zeros(n, dtype=torch.uint8, device=device))

    def table(self, which):
        """Host copy of one of the frame's tables (twdic_frame_table):
        "bicubic_lut" / "bspline_lut" [roi_h, roi_w, 4, 4], "ref_gradient"
        [roi_h, roi_w, 2], "subset_gradient" [num_pois, S, 2]."""
        p = self.params
        rw, rh = p.roi_width, p.roi_height
        S = (2 * p.subset_x + 1) * (2 * p.subset_y + 1)
        code, shape = {"bicubic_lut": (0, (rh, rw, 4, 4)), "bspline_lut": (1, (rh, rw, 4, 4)),
                       "ref_gradient": (2, (rh, rw, 2)), "subset_gradient": (3, (self.n, S, 2))}[which]
        out = np.zeros(shape, np.float32)
        check(self._lib.twdic_frame_table(self._h, code, _ptr(out)))
        return out

    def phase_times(self):
        t = np.zeros(6, np.float32)
        check(self._lib.twdic_frame_phase_times(self._h, _ptr(t)))
        return dict(upload=float(t[0]), fftcc=float(t[1]), prepare=float(t[2]), icgn=float(t[3]),
                    download=float(t[4]), ref_precompute=float(t[5]))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_frame_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DICBatch:
    """Several DICFrame targets in one set of launches (twdic_batch_*): fast-path
    frames of one subset radius share one tensor-core FFT-CC launch and all
    fast-path frames one persistent IC-GN launch.  `graph=True` replays a CUDA
    graph when a device-resident call repeats with the same frames and arrays."""

    def __init__(self, graph: bool = False):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.twdic_batch_create(ctypes.byref(h)))
        self._h = h
        check(self._lib.twdic_batch_set_graph(self._h, 1 if graph else 0))
        self.replayed = False

    def set_stream(self, stream):
        ptr = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
        check(self._lib.twdic_batch_set_stream(self._h, ptr))

    def set_tuning(self, icgn_threads=1024, icgn_ctas_per_sm=0, icgn_sampler=2, icgn_chunk=32):
        check(self._lib.twdic_batch_set_tuning(self._h, icgn_threads, icgn_ctas_per_sm, icgn_sampler))
        if icgn_chunk is not None:
            self.set_icgn_layout(icgn_chunk)

    def set_icgn_layout(self, chunk):
        check(self._lib.twdic_batch_set_icgn_layout(self._h, chunk))

    def set_icgn_unroll(self, unroll):
        check(self._lib.twdic_batch_set_icgn_unroll(self._h, unroll))

    def process(self, frames, tars, outs):
        """frames: list of DICFrame; tars: their target images; outs: list of
        output dicts (DICFrame.alloc_outputs), all host or all device."""
        k = len(frames)
        if not (len(tars) == k == len(outs)) or k == 0:
            raise ValueError("frames, tars and outs must have the same non-zero length")
        keep = []
        fr = (ctypes.c_void_p * k)(*[f._h.value for f in frames])
        tp = (ctypes.c_void_p * k)()
        st = (ctypes.c_int32 * k)()
        mem_in = None
        for i, (f, t) in enumerate(zip(frames, tars)):
            p, stride, m, owner = _image(t, f.params.img_width, f.params.img_height)
            keep.append(owner)
            tp[i] = p.value
            st[i] = stride
            if mem_in is not None and m != mem_in:
                raise ValueError("targets must be all host or all device")
            mem_in = m

        def arr(key):
            a = (ctypes.c_void_p * k)()
            for i, o in enumerate(outs):
                a[i] = _ptr(o[key]).value
            return a

        mem_out = _mem(outs[0]["u"])
        rep = ctypes.c_int32(0)
        check(self._lib.twdic_batch_process(self._h, k, fr, tp, st, mem_in, arr("u"), arr("v"), arr("zncc"),
                                            arr("p6"), arr("iters"), arr("flags"), mem_out, ctypes.byref(rep)))
        self.replayed = bool(rep.value)

    def phase_times(self):
        """Device time (ms) of the phases of the last call run without a
        graph: preparation (target copies, tables, zeroed outputs), FFT-CC,
        float LUTs, IC-GN."""
        t = np.zeros(4, np.float32)
        check(self._lib.twdic_batch_phase_times(self._h, _ptr(t)))
        return dict(prepare=float(t[0]), fftcc=float(t[1]), lut=float(t[2]), icgn=float(t[3]))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
