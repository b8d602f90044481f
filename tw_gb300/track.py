"""The reference's per-camera tracking loop (twdic_tracker_*): reference
refresh every `interval` frames, accumulated displacements, POIs moved by the
truncated displacement, and the displacement colour map written into
headless ROI-sized RGBA images (dumped as PPM by `write_ppm`)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MEM_HOST, Params, check
from .dic import _image


class DICTracker:
    def __init__(self, params: Params, refresh_interval: int = 50, with_icgn: bool = True):
        self._lib = _lib.load()
        self.params = params
        h = ctypes.c_void_p()
        check(self._lib.twdic_tracker_create(ctypes.byref(params), refresh_interval, 1 if with_icgn else 0,
                                             ctypes.byref(h)))
        self._h = h
        n = ctypes.c_int32()
        check(self._lib.twdic_tracker_num_pois(self._h, ctypes.byref(n)))
        self.n = n.value

    def process(self, img) -> dict:
        """One frame; host outputs u, v, acc_u, acc_v, poi (n x 2, (y, x)), flags."""
        p, stride, mem_in, _keep = _image(img, self.params.img_width, self.params.img_height)
        n = self.n
        out = dict(u=np.zeros(n, np.float32), v=np.zeros(n, np.float32), acc_u=np.zeros(n, np.float32),
                   acc_v=np.zeros(n, np.float32), poi=np.zeros((n, 2), np.int32), flags=np.zeros(n, np.uint8))
        ptr = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
        check(self._lib.twdic_tracker_process(self._h, p, stride, mem_in, ptr(out["u"]), ptr(out["v"]),
                                              ptr(out["acc_u"]), ptr(out["acc_v"]), ptr(out["poi"]),
                                              ptr(out["flags"]), MEM_HOST))
        return out

    def colormap(self, tex_u: np.ndarray, tex_v: np.ndarray, min_u=-20.0, max_u=20.0, min_v=-20.0, max_v=20.0):
        """Draw the last frame into the two ROI-sized uint32 RGBA images (in place)."""
        for t in (tex_u, tex_v):
            if t.dtype != np.uint32 or t.shape != (self.params.roi_height, self.params.roi_width) or \
                    not t.flags.c_contiguous:
                raise ValueError("colour images must be contiguous uint32 of the ROI's shape")
        check(self._lib.twdic_tracker_colormap(self._h, ctypes.c_void_p(tex_u.ctypes.data),
                                               ctypes.c_void_p(tex_v.ctypes.data), min_u, max_u, min_v, max_v,
                                               MEM_HOST))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_tracker_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_ppm(path, tex: np.ndarray):
    """Binary PPM (P6) of an RGBA uint32 image (red in the lowest byte)."""
    h, w = tex.shape
    rgb = np.stack([(tex >> s) & 0xFF for s in (0, 8, 16)], axis=-1).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(rgb.tobytes())
