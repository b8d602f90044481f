"""Serving several camera streams through the native scheduler
(twdic_server_*): per-stream reference cache and tables on the device,
admission by HBM budget, drop-if-full queues, continuous batching of the
pending frames of all streams into batched launches on up to four lanes."""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import PENDING, ServerConfig, ServerCounters, TWDICError, check
from .dic import Params, _image, make_params  # noqa: F401


def frame_device_bytes(params: Params) -> int:
    """Device memory a frame handle with these parameters holds (host-only)."""
    lib = _lib.load()
    b = ctypes.c_uint64(0)
    check(lib.twdic_frame_device_bytes(ctypes.byref(params), ctypes.byref(b)))
    return int(b.value)


class DICServer:
    def __init__(self, hbm_budget_bytes: int = 0, max_batch: int = 32, queue_depth: int = 4, lanes: int = 2,
                 use_graph: bool = True, start_paused: bool = False, icgn_threads: int = 0, icgn_sampler: int = 2,
                 mix_sizes: bool = False):
        self._lib = _lib.load()
        self.cfg = ServerConfig(hbm_budget_bytes, max_batch, queue_depth, lanes, 1 if use_graph else 0,
                                1 if start_paused else 0, icgn_threads, icgn_sampler, 1 if mix_sizes else 0)
        h = ctypes.c_void_p()
        check(self._lib.twdic_server_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self._h = h
        self._streams = {}

    def add_stream(self, params: Params) -> int:
        sid = ctypes.c_int32(-1)
        check(self._lib.twdic_server_add_stream(self._h, ctypes.byref(params), ctypes.byref(sid)))
        nx, ny = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.twdic_num_pois(ctypes.byref(params), ctypes.byref(nx), ctypes.byref(ny)))
        self._streams[sid.value] = (params, nx.value * ny.value)
        return sid.value

    def remove_stream(self, sid: int):
        check(self._lib.twdic_server_remove_stream(self._h, sid))
        self._streams.pop(sid, None)

    def set_reference(self, sid: int, ref: np.ndarray):
        params, _ = self._streams[sid]
        p, stride, _mem, _keep = _image(ref, params.img_width, params.img_height)
        check(self._lib.twdic_server_set_reference(self._h, sid, p, stride))

    def submit(self, sid: int, tar: np.ndarray) -> Optional[int]:
        """Ticket of the queued frame, or None if the stream's queue was full
        (the frame is dropped)."""
        params, _ = self._streams[sid]
        p, stride, _mem, _keep = _image(tar, params.img_width, params.img_height)
        t = ctypes.c_uint64(0)
        rc = self._lib.twdic_submit(self._h, sid, p, stride, ctypes.byref(t))
        if rc == -9:
            return None
        check(rc)
        return int(t.value)

    def poll(self, sid: int, ticket: int, wait: bool = True):
        """Results dict (u, v, zncc, p6, iters, flags, latency_ms), or None if
        the frame is not done and wait is False."""
        _, n = self._streams[sid]
        out = dict(u=np.zeros(n, np.float32), v=np.zeros(n, np.float32), zncc=np.zeros(n, np.float32),
                   p6=np.zeros((n, 6), np.float32), iters=np.zeros(n, np.int32), flags=np.zeros(n, np.uint8))
        lat = ctypes.c_double(0.0)
        rc = self._lib.twdic_poll(self._h, ticket, 1 if wait else 0,
                                  *[ctypes.c_void_p(out[k].ctypes.data) for k in ("u", "v", "zncc", "p6", "iters",
                                                                                  "flags")],
                                  ctypes.byref(lat))
        if rc == PENDING:
            return None
        check(rc)
        out["latency_ms"] = lat.value
        return out

    def resume(self):
        check(self._lib.twdic_server_resume(self._h))

    def stats(self) -> dict:
        c = ServerCounters()
        check(self._lib.twdic_server_stats(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in ServerCounters._fields_}

    def set_stream_guess(self, stream_id: int, mode: int):
        """1: each frame's IC-GN starts from the stream's last displacements
        (FFT-CC skipped after the first frame of a reference); 0: FFT-CC every
        frame (default)."""
        check(self._lib.twdic_server_set_stream_guess(self._h, stream_id, mode))

    def stream_stats(self, stream_id: int) -> dict:
        """One stream's completed and dropped frames, latency percentiles and
        the reference's average processing FPS (see twdic_server_stream_stats)."""
        c = _lib.StreamStats()
        check(self._lib.twdic_server_stream_stats(self._h, stream_id, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in _lib.StreamStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.twdic_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["DICServer", "frame_device_bytes", "TWDICError"]
