"""Batched processing (twdic_batch_*): image pairs and POI sets of uneven
sizes in one set of launches give the same results as each frame alone, and
graph replay of a repeated device-resident call recomputes from the refreshed
inputs."""
import numpy as np
import pytest

from tw_gb300 import PATH_FAST, PATH_PLAIN, dic, synth

pytestmark = pytest.mark.gpu


def _frame(g, path=PATH_FAST):
    return dic.DICFrame(dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r,
                                        g.subset_r, g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p,
                                        path))


CASES = [  # (h, w, r, grid, seed, path): two window sizes, uneven images and POI counts, one plain frame
    (160, 192, 10, 7, 11, PATH_FAST),
    (130, 257, 10, 5, 12, PATH_FAST),
    (200, 150, 16, 9, 13, PATH_FAST),
    (120, 120, 10, 6, 14, PATH_FAST),
    (160, 192, 10, 7, 15, PATH_PLAIN),
]


def _alone(cases):
    frames, tars, want = [], [], []
    for h, w, r, grid, seed, path in cases:
        pair, g = synth.small_case(h=h, w=w, r=r, grid=grid, seed=seed)
        f = _frame(g, path)
        f.set_reference(pair.ref)
        o = f.alloc_outputs()
        f.process(pair.tar, **o)
        frames.append(f)
        tars.append(pair.tar)
        want.append(o)
    return frames, tars, want


def test_batch_equals_frames_alone():
    frames, tars, want = _alone(CASES)
    b = dic.DICBatch()
    outs = [f.alloc_outputs() for f in frames]
    b.process(frames, tars, outs)
    for i, (o, w) in enumerate(zip(outs, want)):
        assert (w["flags"] == 0).mean() > 0.9, i
        for k in w:
            np.testing.assert_array_equal(o[k], w[k], err_msg=f"frame {i} {k}")
    # the phases of the call (no graph): preparation, FFT-CC and IC-GN took time
    ph = b.phase_times()
    assert ph["prepare"] > 0 and ph["fftcc"] > 0 and ph["icgn"] > 0, ph
    # a second call on the same handles (caches warm) gives the same results
    outs2 = [f.alloc_outputs() for f in frames]
    b.process(frames, tars, outs2)
    for o, w in zip(outs2, want):
        for k in w:
            np.testing.assert_array_equal(o[k], w[k])


def test_batch_more_frames_than_one_launch_holds():
    """130 frames: more than the 128 one IC-GN (and one FFT-CC) launch takes,
    with two window sizes, so the batch runs two launches of each."""
    cases = [(64, 72 + 4 * (i % 5), 5 + (i % 2), 6, 100 + i, PATH_FAST) for i in range(130)]
    frames, tars, want = _alone(cases)
    b = dic.DICBatch()
    outs = [f.alloc_outputs() for f in frames]
    b.process(frames, tars, outs)
    for o, w in zip(outs, want):
        for k in w:
            np.testing.assert_array_equal(o[k], w[k])


def test_batch_graph_replay_reads_refreshed_inputs():
    import torch
    cases = CASES[:4]
    pairs = [synth.small_case(h=h, w=w, r=r, grid=gr, seed=s) for h, w, r, gr, s, _ in cases]
    pairs2 = [synth.small_case(h=h, w=w, r=r, grid=gr, seed=s, u0=-0.7, v0=1.3) for h, w, r, gr, s, _ in cases]
    frames = []
    for (pair, g) in pairs:
        f = _frame(g)
        f.set_reference(pair.ref)
        frames.append(f)
    dev_tars = [torch.from_numpy(p.tar).cuda() for p, _ in pairs]
    outs = [f.alloc_outputs(device="cuda") for f in frames]
    b = dic.DICBatch(graph=True)
    b.process(frames, dev_tars, outs)  # runs, then records the graph
    assert not b.replayed
    # new target contents in the same device arrays; the replay must see them
    for t, (p2, _) in zip(dev_tars, pairs2):
        t.copy_(torch.from_numpy(p2.tar))
    b.process(frames, dev_tars, outs)
    assert b.replayed
    torch.cuda.synchronize()
    for f, o, (p2, _) in zip(frames, outs, pairs2):
        w = f.alloc_outputs()
        # each frame alone, on the same reference (its cache is unchanged)
        f.process(p2.tar, **w)
        for k in w:
            np.testing.assert_array_equal(o[k].cpu().numpy(), w[k])


def test_batch_with_bspline_frames_equals_alone():
    """B-spline frames share the batch's IC-GN launches (grouped by sampler:
    neighbourhood table with the B-spline weights) with bicubic ones, and a
    plain-path B-spline frame runs on its own; each equals the frame alone."""
    from tw_gb300 import INTERP_BSPLINE
    frames, tars, want = [], [], []
    for k, (h, w, r, grid, seed, path) in enumerate(CASES):
        pair, g = synth.small_case(h=h, w=w, r=r, grid=grid, seed=seed)
        f = _frame(g, path)
        if k in (1, 3, 4):
            f.set_interpolation(INTERP_BSPLINE)
        f.set_reference(pair.ref)
        o = f.alloc_outputs()
        f.process(pair.tar, **o)
        frames.append(f)
        tars.append(pair.tar)
        want.append(o)
    b = dic.DICBatch()
    outs = [f.alloc_outputs() for f in frames]
    b.process(frames, tars, outs)
    for o, w in zip(outs, want):
        for k in w:
            np.testing.assert_array_equal(o[k], w[k])


def test_batch_graph_recaptured_after_interpolation_change():
    """A captured graph holds each frame's sampler and target table: after a
    frame switches to the B-spline interpolation the next call is captured
    anew, and that frame's results equal the frame alone."""
    import torch
    from tw_gb300 import INTERP_BSPLINE
    pairs = [synth.small_case(h=h, w=w, r=r, grid=gr, seed=s) for h, w, r, gr, s, _ in CASES[:2]]
    frames = []
    for pair, g in pairs:
        f = _frame(g)
        f.set_reference(pair.ref)
        frames.append(f)
    dev_tars = [torch.from_numpy(p.tar).cuda() for p, _ in pairs]
    outs = [f.alloc_outputs(device="cuda") for f in frames]
    b = dic.DICBatch(graph=True)
    b.process(frames, dev_tars, outs)
    b.process(frames, dev_tars, outs)
    assert b.replayed
    frames[1].set_interpolation(INTERP_BSPLINE)
    b.process(frames, dev_tars, outs)
    assert not b.replayed
    torch.cuda.synchronize()
    pair, g = pairs[1]
    f = _frame(g)
    f.set_interpolation(INTERP_BSPLINE)
    f.set_reference(pair.ref)
    w = f.alloc_outputs()
    f.process(pair.tar, **w)
    for k in w:
        np.testing.assert_array_equal(outs[1][k].cpu().numpy(), w[k], err_msg=k)
