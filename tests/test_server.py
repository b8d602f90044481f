"""Serving (twdic_server_*): admission by HBM budget, drop-if-full queues,
continuous batching across streams of different sizes; each frame's result is
the same alone and in the mix."""
import numpy as np
import pytest

from tw_gb300 import PATH_FAST, dic, synth
from tw_gb300.serve import DICServer, frame_device_bytes


def _params(g, path=PATH_FAST):
    return dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                           g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, path)


def test_frame_device_bytes_formula():
    """Host-only estimate used for admission: images padded to 16-byte rows,
    per-POI buffers, the small buffers (error flag, work counter, twiddles,
    TMA descriptors) and the fast path's cache, gradient image, sample table,
    neighbourhood table and the FFT-CC's reference spectra, each rounded up
    to 2 MiB."""
    _, g = synth.small_case(h=160, w=197, r=10, grid=7)
    p = _params(g)
    n = dic.num_pois(p)[0] * dic.num_pois(p)[1]
    r = lambda b: -(-b // (2 << 20)) * (2 << 20)  # noqa: E731
    pitch = (197 + 15) // 16 * 16
    want = (2 * r(pitch * 160 + 16) + r(8 * n) + 3 * r(4 * n) + r(n) + r(24 * n) + r(4 * n) + r(n) + 4 * r(1024)
            + r(64 * n) + r(168 * n) + r(n) + r(8 * g.roi_w * g.roi_h) + r(16 * 21 * 21) + r(16 * g.roi_w * g.roi_h)
            + r(n * 11 * 20 * 4) + r(8 * n))  # reference spectra (N = 20: 11 rows of 20 FP16 pairs), window sums
    assert frame_device_bytes(p) == want
    big = _params(synth.Geometry(2048, 2048, 1, 1, 2046, 2046, 20, 5, 20))
    assert frame_device_bytes(big) > 128 << 20  # 155k POIs: 67 MB neighbourhood table, 36 MB cache


def test_frame_device_bytes_rejects_bad_params():
    p = dic.make_params(100, 100, 0, 0, 100, 100, 10, 10, 5, 5, 0, 0)  # no image border
    with pytest.raises(dic.TWDICError):
        frame_device_bytes(p)


CASES = [(160, 192, 10, 7, 21), (130, 257, 10, 5, 22), (200, 150, 16, 9, 23)]


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix():
    pairs = [synth.small_case(h=h, w=w, r=r, grid=gr, seed=s) for h, w, r, gr, s in CASES]
    pairs2 = [synth.small_case(h=h, w=w, r=r, grid=gr, seed=s, u0=-0.7, v0=1.3) for h, w, r, gr, s in CASES]
    # frames of any size share a batch here; the server starts paused so that
    # the first frames of all streams are pending together
    srv = DICServer(max_batch=8, queue_depth=4, lanes=2, start_paused=True, mix_sizes=True)
    sids = []
    for pair, g in pairs:
        sid = srv.add_stream(_params(g))
        srv.set_reference(sid, pair.ref)
        sids.append(sid)
    # frames of all streams interleaved, several in flight at once
    tickets = []
    for rnd in range(3):
        for sid, (pair, _), (pair2, _) in zip(sids, pairs, pairs2):
            tar = pair.tar if rnd % 2 == 0 else pair2.tar
            t = srv.submit(sid, tar)
            assert t is not None
            tickets.append((sid, t, rnd))
    srv.resume()
    got = {(sid, rnd): srv.poll(sid, t) for sid, t, rnd in tickets}
    st = srv.stats()
    assert st["completed"] == len(tickets) and st["dropped"] == 0
    assert st["batches"] >= 1 and st["batched_frames"] == len(tickets)
    # the first batch took the pending frame of every stream
    assert st["max_batch_formed"] == len(pairs), st
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for sid, (pair, g), (pair2, _) in zip(sids, pairs, pairs2):
        f = dic.DICFrame(_params(g))
        f.set_reference(pair.ref)
        for rnd in range(3):
            w = f.alloc_outputs()
            f.process(pair.tar if rnd % 2 == 0 else pair2.tar, **w)
            o = got[(sid, rnd)]
            assert (w["flags"] == 0).mean() > 0.9
            for k in w:
                np.testing.assert_array_equal(o[k], w[k], err_msg=f"stream {sid} frame {rnd} {k}")
    srv.close()


@pytest.mark.gpu
def test_batches_form_and_run_on_two_lanes():
    """Four streams of one size, two frames each, queued while the server is
    paused: on resume the scheduler fills both lanes with a batch of two
    frames each (continuous batching over lanes); the device intervals of
    the batches, timed by events on their lanes, are reported; every result
    equals the frame processed alone."""
    pair, g = synth.small_case()
    pair2, _ = synth.small_case(u0=-0.7, v0=1.3)
    srv = DICServer(max_batch=2, queue_depth=4, lanes=2, start_paused=True)
    sids = []
    for _ in range(4):
        sid = srv.add_stream(_params(g))
        srv.set_reference(sid, pair.ref)
        sids.append(sid)
    tickets = [(sid, srv.submit(sid, tar), k) for k, tar in enumerate((pair.tar, pair2.tar)) for sid in sids]
    srv.resume()
    got = {(sid, k): srv.poll(sid, t) for sid, t, k in tickets}
    st = srv.stats()
    print(st)
    assert st["completed"] == 8 and st["batches"] == 4
    assert st["max_batch_formed"] == 2 and st["peak_lanes_in_flight"] == 2, st
    assert st["device_busy_ms"] > 0 and st["peak_device_batches"] >= 1
    f = dic.DICFrame(_params(g))
    f.set_reference(pair.ref)
    for k, tar in enumerate((pair.tar, pair2.tar)):
        w = f.alloc_outputs()
        f.process(tar, **w)
        for sid in sids:
            for key in w:
                np.testing.assert_array_equal(got[(sid, k)][key], w[key], err_msg=f"stream {sid} frame {k} {key}")
    srv.close()


@pytest.mark.gpu
def test_admission_by_hbm_budget():
    (_, g1), (_, g2) = synth.small_case(h=160, w=192, r=10), synth.small_case(h=200, w=150, r=16)
    b1 = frame_device_bytes(_params(g1))
    srv = DICServer(hbm_budget_bytes=b1 + (8 << 20), queue_depth=1)
    srv.add_stream(_params(g1))
    with pytest.raises(dic.TWDICError) as e:
        srv.add_stream(_params(g2))
    assert "NO_MEMORY" in str(e.value)
    st = srv.stats()
    assert st["streams"] == 1 and st["committed_bytes"] <= st["budget_bytes"]
    srv.close()


@pytest.mark.gpu
def test_full_queue_drops_frames():
    pair, g = synth.small_case()
    srv = DICServer(queue_depth=2, start_paused=True)
    sid = srv.add_stream(_params(g))
    srv.set_reference(sid, pair.ref)
    t1, t2 = srv.submit(sid, pair.tar), srv.submit(sid, pair.tar)
    assert t1 is not None and t2 is not None
    assert srv.submit(sid, pair.tar) is None  # both slots taken: dropped
    assert srv.poll(sid, t1, wait=False) is None  # held while paused
    srv.resume()
    a, b = srv.poll(sid, t1), srv.poll(sid, t2)
    for k in ("u", "v", "p6", "iters", "flags"):
        np.testing.assert_array_equal(a[k], b[k])
    st = srv.stats()
    assert st["dropped"] == 1 and st["completed"] == 2
    ss = srv.stream_stats(sid)
    assert ss["dropped"] == 1 and ss["completed"] == 2 and ss["p50_ms"] <= ss["p99_ms"]
    assert ss["average_fps"] == 0  # fewer than 32 completed frames
    srv.close()


@pytest.mark.gpu
def test_stream_fps_statistics():
    """The reference's processing-rate statistic per stream: after 32 paced
    frames its average FPS is set, and it lies within the rates the frame
    spacing allows."""
    import time
    pair, g = synth.small_case()
    srv = DICServer(queue_depth=4)
    sid = srv.add_stream(_params(g))
    srv.set_reference(sid, pair.ref)
    for _ in range(34):
        t = srv.submit(sid, pair.tar)
        assert t is not None
        srv.poll(sid, t)
        time.sleep(0.01)  # at most 100 frames per second
    ss = srv.stream_stats(sid)
    assert ss["completed"] == 34 and ss["dropped"] == 0
    assert 10 <= ss["average_fps"] <= 100, ss
    srv.close()


@pytest.mark.gpu
def test_last_frame_guesses():
    """Guess mode 1: after the first frame of a reference, IC-GN starts from
    the stream's last displacements on the device and FFT-CC is skipped. On a
    drifting camera sequence every frame still meets the parity bar against
    FFT-CC-seeded IC-GN (the oracle), and a new reference restarts from FFT-CC."""
    from oracle import oracle as O
    ref, tars, g = synth.camera_sequence(200, 176, frames=4, seed=41, r=10, grid=9, margin=12)
    p = _params(g)
    poi = dic.poi_positions(p)
    srv = DICServer(queue_depth=2)
    sid = srv.add_stream(p)
    srv.set_stream_guess(sid, 1)
    for rnd in range(2):  # the second round after a fresh reference
        srv.set_reference(sid, ref)
        first = None
        for tar in tars:
            t = srv.submit(sid, tar)
            assert t is not None
            out = srv.poll(sid, t)
            if first is None:
                first = out
            else:  # no FFT-CC ran: the ZNCC array still holds the first frame's
                np.testing.assert_array_equal(out["zncc"], first["zncc"])
                assert (out["u"] != first["u"]).any()
            u_or, v_or, _, _ = O.fftcc(ref, tar, poi, g.subset_r)
            p6_or, it_or, fl_or = O.icgn(ref, tar, g, poi, u_or, v_or)
            both = (out["flags"] == 0) & (fl_or == 0)
            assert both.mean() > 0.9
            bad = (np.abs(out["u"] - p6_or[:, 0]) > 1e-3) | (np.abs(out["v"] - p6_or[:, 3]) > 1e-3)
            assert bad[both].sum() <= 0.01 * both.sum() + 1, (rnd, bad[both].sum())
    assert srv.stream_stats(sid)["completed"] == 2 * len(tars)
    srv.close()


@pytest.mark.gpu
def test_remove_stream_while_polling():
    """A call waiting on a ticket whose stream is removed returns an error
    status instead of reading the freed slots, and a ticket that was read
    once is unknown afterwards."""
    import threading
    import time
    pair, g = synth.small_case()
    srv = DICServer(queue_depth=2, start_paused=True)
    sid = srv.add_stream(_params(g))
    srv.set_reference(sid, pair.ref)
    t = srv.submit(sid, pair.tar)
    rc = []
    th = threading.Thread(
        target=lambda: rc.append(srv._lib.twdic_poll(srv._h, t, 1, None, None, None, None, None, None, None)))
    th.start()
    time.sleep(0.2)  # the poll is waiting: the server is paused
    srv.remove_stream(sid)
    th.join(timeout=10)
    assert not th.is_alive() and rc and rc[0] in (-4, -1), rc  # stream removed / ticket unknown
    sid2 = srv.add_stream(_params(g))
    srv.set_reference(sid2, pair.ref)
    srv.resume()
    t2 = srv.submit(sid2, pair.tar)
    assert srv.poll(sid2, t2)["flags"].size > 0
    assert srv._lib.twdic_poll(srv._h, t2, 0, None, None, None, None, None, None, None) == -1
    srv.close()
