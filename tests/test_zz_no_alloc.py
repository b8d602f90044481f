"""twdic_icgn_compute_noalloc: the IC-GN entry point for callers that cannot
allocate device memory (a real-time frame loop that cannot absorb cudaMalloc's
device-wide synchronisation, or memory budgeted up front by another
allocator).  It must give the same results as the handle-based entry point
(twdic_icgn_compute), call after call, although its scratch lives in one
static device array that every call reuses.

This file is named to be collected last, so that a run stopping at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import PATH_FAST, PATH_PLAIN, _lib, dic, synth

pytestmark = pytest.mark.gpu

MAX_POIS = 196608  # TWDIC_NOALLOC_MAX_POIS in include/tw_dic.h


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_handle_entry_point_on_consecutive_calls():
    import torch

    lib = _lib.load()
    pair, g = synth.small_case()
    prm = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                          g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, PATH_FAST)
    poi = dic.poi_positions(prm)
    n = len(poi)
    # integer-pixel guesses from the FFT-CC entry point
    f = dic.cuFFTCC2D(g.img_w, g.img_h, g.roi_w, g.roi_h, g.start_x, g.start_y, g.subset_r, g.subset_r, g.grid,
                      g.grid, g.margin, g.margin, path=PATH_FAST)
    U, V, Z = f.InitializeFFTCC(pair.ref)
    f.ComputeFFTCC(U, V, Z, pair.tar)
    u0 = U.ravel().copy()
    v0 = V.ravel().copy()

    dev = "cuda"
    d_ref = torch.from_numpy(pair.ref).to(dev)
    d_tar = torch.from_numpy(pair.tar).to(dev)
    d_poi = torch.from_numpy(poi).to(dev)

    # existing entry point (handle-owned buffers)
    ic = dic.cuICGN2D(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, n, 1,
                      g.max_iter, g.delta_p, path=PATH_FAST)
    ic.cuInitialize(d_ref)
    ref_u = torch.from_numpy(u0).to(dev)
    ref_v = torch.from_numpy(v0).to(dev)
    ref_p6 = torch.zeros((n, 6), dtype=torch.float32, device=dev)
    ref_it = torch.zeros(n, dtype=torch.int32, device=dev)
    ref_fl = torch.zeros(n, dtype=torch.uint8, device=dev)
    ic.cuCompute(d_tar, d_poi, ref_u, ref_v, ref_p6, ref_it, ref_fl)
    torch.cuda.synchronize()
    want = (ref_p6.cpu().numpy(), ref_it.cpu().numpy(), ref_fl.cpu().numpy())
    assert (want[2] == 0).mean() > 0.95

    # the oracle (the CPU restatement of the reference's IC-GN) from the same guesses
    want_or = O.icgn(pair.ref, pair.tar, g, poi, u0, v0)

    stream = torch.cuda.Stream()
    free_before = None
    for call in range(2):
        u = torch.from_numpy(u0).to(dev)
        v = torch.from_numpy(v0).to(dev)
        p6 = torch.full((n, 6), float("nan"), dtype=torch.float32, device=dev)
        it = torch.zeros(n, dtype=torch.int32, device=dev)
        fl = torch.full((n,), 255, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        if call == 1:
            # after the first call has set up the device, a call allocates nothing
            free_before = torch.cuda.mem_get_info()[0]
            torch_before = torch.cuda.memory_allocated()
        rc = lib.twdic_icgn_compute_noalloc(ctypes.byref(prm), _vp(d_ref), _vp(d_tar), _vp(d_poi), n, _vp(u),
                                            _vp(v), _vp(p6), _vp(it), _vp(fl), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.twdic_last_error()
        stream.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
            assert torch.cuda.memory_allocated() == torch_before
        got = (p6.cpu().numpy(), it.cpu().numpy(), fl.cpu().numpy())
        rep = C.icgn_parity(got[0], got[1], got[2], *want, r=g.subset_r)
        assert rep.ok(), (call, rep)
        rep_or = C.icgn_parity(got[0], got[1], got[2], *want_or, r=g.subset_r)
        assert rep_or.ok(), (call, rep_or)
        np.testing.assert_array_equal(u.cpu().numpy(), got[0][:, 0])
        np.testing.assert_array_equal(v.cpu().numpy(), got[0][:, 3])

    # sizes beyond the static scratch are rejected before any work is queued
    rc = lib.twdic_icgn_compute_noalloc(ctypes.byref(prm), _vp(d_ref), _vp(d_tar), _vp(d_poi), MAX_POIS + 1,
                                        _vp(u), _vp(v), _vp(p6), _vp(it), _vp(fl), None)
    assert rc == -7
    assert b"TWDIC_NOALLOC_MAX_POIS" in lib.twdic_last_error()
    # an ROI without the one-pixel border the gradients need, and the plain
    # path (which needs handle-owned buffers), are rejected the same way
    bad = dic.make_params(g.img_w, g.img_h, 0, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, g.grid, g.grid,
                          g.margin, g.margin, g.max_iter, g.delta_p, PATH_FAST)
    rc = lib.twdic_icgn_compute_noalloc(ctypes.byref(bad), _vp(d_ref), _vp(d_tar), _vp(d_poi), n, _vp(u), _vp(v),
                                        _vp(p6), _vp(it), _vp(fl), None)
    assert rc == -3, lib.twdic_last_error()
    plain = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                            g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, PATH_PLAIN)
    rc = lib.twdic_icgn_compute_noalloc(ctypes.byref(plain), _vp(d_ref), _vp(d_tar), _vp(d_poi), n, _vp(u),
                                        _vp(v), _vp(p6), _vp(it), _vp(fl), None)
    assert rc == -7, lib.twdic_last_error()
