"""ctypes binding of libtwdic.so (the C ABI declared in include/tw_dic.h).

Loading fails loudly when the library has not been built: there is no
CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtwdic.so")

OK = 0
ERR = {
    -1: "TWDIC_ERR_INVALID_ARG",
    -2: "TWDIC_ERR_NO_POI",
    -3: "TWDIC_ERR_BORDER",
    -4: "TWDIC_ERR_STATE",
    -5: "TWDIC_ERR_CUDA",
    -6: "TWDIC_ERR_NO_MEMORY",
    -7: "TWDIC_ERR_UNSUPPORTED",
    -8: "TWDIC_ERR_TIMEOUT",
    -9: "TWDIC_ERR_BUSY",
}
PENDING = 1  # twdic_poll: not done yet
INTERP_BICUBIC, INTERP_BSPLINE = 0, 1  # IC-GN target interpolation
MEM_HOST = 0
MEM_DEVICE = 1
PATH_PLAIN = 0
PATH_FAST = 1
# fast IC-GN target samplers (twdic_frame_set_tuning)
SAMPLER_WINDOW, SAMPLER_LUT, SAMPLER_NBHD = 0, 1, 2

# every symbol include/tw_dic.h declares
EXPORTED = (
    "twdic_last_error", "twdic_abi_version", "twdic_num_pois", "twdic_poi_positions",
    "twdic_fftcc_create", "twdic_fftcc_num_pois", "twdic_fftcc_poi_positions", "twdic_fftcc_reset_ref",
    "twdic_fftcc_set_tar", "twdic_fftcc_compute", "twdic_fftcc_destroy",
    "twdic_icgn_create", "twdic_icgn_reset_ref", "twdic_icgn_compute", "twdic_icgn_destroy",
    "twdic_frame_create", "twdic_frame_num_pois", "twdic_frame_poi_positions", "twdic_frame_set_reference",
    "twdic_frame_process", "twdic_frame_set_stream", "twdic_frame_phase_times", "twdic_frame_destroy",
    "twdic_frame_table",
    "twdic_frame_set_tuning", "twdic_frame_set_icgn_layout", "twdic_frame_set_icgn_unroll", "twdic_frame_set_guess_mode", "twdic_frame_set_fftcc_twiddles", "twdic_icgn_compute_noalloc",
    "twdic_batch_create", "twdic_batch_set_stream", "twdic_batch_set_tuning", "twdic_batch_set_icgn_layout", "twdic_batch_set_icgn_unroll", "twdic_batch_set_graph",
    "twdic_batch_process", "twdic_batch_phase_times", "twdic_batch_destroy", "twdic_frame_device_bytes",
    "twdic_server_create", "twdic_server_add_stream", "twdic_server_remove_stream", "twdic_server_set_reference",
    "twdic_submit", "twdic_poll", "twdic_server_resume", "twdic_server_stats", "twdic_server_stream_stats", "twdic_server_set_stream_guess", "twdic_server_destroy",
    "twdic_frame_set_fftcc_tuning", "twdic_frame_get_tuning", "twdic_frame_autotune",
    "twdic_tracker_create", "twdic_tracker_num_pois", "twdic_tracker_process", "twdic_tracker_colormap",
    "twdic_tracker_destroy", "twdic_icgn_set_interpolation", "twdic_frame_set_interpolation",
)


class TWDICError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{ERR.get(code, code)}: {message}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [
        ("img_width", ctypes.c_int32), ("img_height", ctypes.c_int32),
        ("start_x", ctypes.c_int32), ("start_y", ctypes.c_int32),
        ("roi_width", ctypes.c_int32), ("roi_height", ctypes.c_int32),
        ("subset_x", ctypes.c_int32), ("subset_y", ctypes.c_int32),
        ("grid_space_x", ctypes.c_int32), ("grid_space_y", ctypes.c_int32),
        ("margin_x", ctypes.c_int32), ("margin_y", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("delta_p", ctypes.c_float),
        ("path", ctypes.c_int32),
    ]


class ServerConfig(ctypes.Structure):
    """twdic_server_config"""
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_int32), ("queue_depth", ctypes.c_int32),
        ("lanes", ctypes.c_int32), ("use_graph", ctypes.c_int32), ("start_paused", ctypes.c_int32),
        ("icgn_threads", ctypes.c_int32), ("icgn_sampler", ctypes.c_int32), ("mix_sizes", ctypes.c_int32),
    ]


class Tuning(ctypes.Structure):
    """twdic_tuning"""
    _fields_ = [
        ("icgn_threads", ctypes.c_int32), ("icgn_ctas_per_sm", ctypes.c_int32), ("icgn_sampler", ctypes.c_int32),
        ("fftcc_use_tc", ctypes.c_int32), ("fftcc_groups", ctypes.c_int32), ("fftcc_pois_per_group", ctypes.c_int32),
        ("fftcc_ms", ctypes.c_float), ("icgn_ms", ctypes.c_float), ("from_cache", ctypes.c_int32),
        ("icgn_chunk", ctypes.c_int32), ("icgn_unroll", ctypes.c_int32),
    ]


class StreamStats(ctypes.Structure):
    """twdic_stream_stats"""
    _fields_ = [
        ("completed", ctypes.c_uint64), ("dropped", ctypes.c_uint64), ("average_fps", ctypes.c_int32),
        ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
    ]


class ServerCounters(ctypes.Structure):
    """twdic_server_counters"""
    _fields_ = [
        ("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("dropped", ctypes.c_uint64),
        ("batches", ctypes.c_uint64), ("batched_frames", ctypes.c_uint64), ("graph_replays", ctypes.c_uint64),
        ("committed_bytes", ctypes.c_uint64), ("budget_bytes", ctypes.c_uint64), ("streams", ctypes.c_int32),
        ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
        ("max_batch_formed", ctypes.c_uint64), ("peak_lanes_in_flight", ctypes.c_int32),
        ("peak_device_batches", ctypes.c_int32), ("device_busy_ms", ctypes.c_double),
        ("device_overlap_ms", ctypes.c_double),
    ]


_lib = None
_VP = ctypes.c_void_p
_I = ctypes.c_int
_I32P = ctypes.POINTER(ctypes.c_int32)


def load():
    """Load libtwdic.so; raises if it is missing (build it with tw_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(Params)
    sig = {
        "twdic_last_error": ([], ctypes.c_char_p),
        "twdic_abi_version": ([], _I),
        "twdic_num_pois": ([P, _I32P, _I32P], _I),
        "twdic_poi_positions": ([P, _VP], _I),
        "twdic_fftcc_create": ([P, ctypes.POINTER(_VP)], _I),
        "twdic_fftcc_num_pois": ([_VP, _I32P, _I32P], _I),
        "twdic_fftcc_poi_positions": ([_VP, _VP, _I], _I),
        "twdic_fftcc_reset_ref": ([_VP, _VP, ctypes.c_int32, _I], _I),
        "twdic_fftcc_set_tar": ([_VP, _VP, ctypes.c_int32, _I], _I),
        "twdic_fftcc_compute": ([_VP, _VP, _VP, _VP, _VP, _I], _I),
        "twdic_fftcc_destroy": ([_VP], _I),
        "twdic_icgn_create": ([P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_VP)], _I),
        "twdic_icgn_reset_ref": ([_VP, _VP, ctypes.c_int32, _I], _I),
        "twdic_icgn_compute": ([_VP, _VP, ctypes.c_int32, _VP, _I, _VP, _VP, _VP, _VP, _VP, _I], _I),
        "twdic_icgn_destroy": ([_VP], _I),
        "twdic_frame_create": ([P, ctypes.POINTER(_VP)], _I),
        "twdic_frame_num_pois": ([_VP, _I32P, _I32P], _I),
        "twdic_frame_poi_positions": ([_VP, _VP, _I], _I),
        "twdic_frame_set_reference": ([_VP, _VP, ctypes.c_int32, _I], _I),
        "twdic_frame_process": ([_VP, _VP, ctypes.c_int32, _I, _VP, _VP, _VP, _VP, _VP, _VP, _I], _I),
        "twdic_frame_set_stream": ([_VP, _VP], _I),
        "twdic_frame_phase_times": ([_VP, _VP], _I),
        "twdic_frame_table": ([_VP, _I, _VP], _I),
        "twdic_frame_destroy": ([_VP], _I),
        "twdic_frame_set_tuning": ([_VP, _I, _I, _I, _I], _I),
        "twdic_frame_set_icgn_layout": ([_VP, _I], _I),
        "twdic_frame_set_icgn_unroll": ([_VP, _I], _I),
        "twdic_frame_set_guess_mode": ([_VP, _I], _I),
        "twdic_frame_set_fftcc_twiddles": ([_VP, _I], _I),
        "twdic_icgn_compute_noalloc": ([P, _VP, _VP, _VP, ctypes.c_int32, _VP, _VP, _VP, _VP, _VP, _VP], _I),
        "twdic_batch_create": ([ctypes.POINTER(_VP)], _I),
        "twdic_batch_set_stream": ([_VP, _VP], _I),
        "twdic_batch_set_tuning": ([_VP, _I, _I, _I], _I),
        "twdic_batch_set_icgn_layout": ([_VP, _I], _I),
        "twdic_batch_set_icgn_unroll": ([_VP, _I], _I),
        "twdic_batch_set_graph": ([_VP, _I], _I),
        "twdic_batch_process": ([_VP, ctypes.c_int32, _VP, _VP, _VP, _I, _VP, _VP, _VP, _VP, _VP, _VP, _I,
                                 _I32P], _I),
        "twdic_batch_phase_times": ([_VP, _VP], _I),
        "twdic_batch_destroy": ([_VP], _I),
        "twdic_frame_device_bytes": ([P, ctypes.POINTER(ctypes.c_uint64)], _I),
        "twdic_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(_VP)], _I),
        "twdic_server_add_stream": ([_VP, P, _I32P], _I),
        "twdic_server_remove_stream": ([_VP, ctypes.c_int32], _I),
        "twdic_server_set_reference": ([_VP, ctypes.c_int32, _VP, ctypes.c_int32], _I),
        "twdic_submit": ([_VP, ctypes.c_int32, _VP, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)], _I),
        "twdic_poll": ([_VP, ctypes.c_uint64, ctypes.c_int32, _VP, _VP, _VP, _VP, _VP, _VP,
                        ctypes.POINTER(ctypes.c_double)], _I),
        "twdic_server_resume": ([_VP], _I),
        "twdic_server_stats": ([_VP, ctypes.POINTER(ServerCounters)], _I),
        "twdic_server_stream_stats": ([_VP, _I, ctypes.POINTER(StreamStats)], _I),
        "twdic_server_set_stream_guess": ([_VP, _I, _I], _I),
        "twdic_server_destroy": ([_VP], _I),
        "twdic_frame_set_fftcc_tuning": ([_VP, _I, _I, _I], _I),
        "twdic_frame_get_tuning": ([_VP, ctypes.POINTER(Tuning)], _I),
        "twdic_frame_autotune": ([_VP, _VP, ctypes.c_int32, _I, ctypes.c_char_p, ctypes.POINTER(Tuning)], _I),
        "twdic_tracker_create": ([P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_VP)], _I),
        "twdic_tracker_num_pois": ([_VP, _I32P], _I),
        "twdic_tracker_process": ([_VP, _VP, ctypes.c_int32, _I, _VP, _VP, _VP, _VP, _VP, _VP, _I], _I),
        "twdic_tracker_colormap": ([_VP, _VP, _VP, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    _I], _I),
        "twdic_tracker_destroy": ([_VP], _I),
        "twdic_icgn_set_interpolation": ([_VP, _I], _I),
        "twdic_frame_set_interpolation": ([_VP, _I], _I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int):
    if rc != OK:
        msg = load().twdic_last_error()
        raise TWDICError(rc, msg.decode() if msg else "")
    return rc
