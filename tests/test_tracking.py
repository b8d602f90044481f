"""Tracking loop and colour map (twdic_tracker_*): reference refresh every
`interval` frames, accumulated displacements, POIs moved by the truncated
displacement, every frame's IC-GN result at the current POIs within the
parity bar of the oracle, and the colour map equal to the numpy
restatement."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import track as T
from tw_gb300 import dic, synth

# entries of the reference's colour table (TW/TW_Core/cuda_utils.cu:15-47),
# as (index, 0xAABBGGRR)
REFERENCE_JET = [(0, 0xFF830000), (31, 0xFFFF0000), (32, 0xFFFF0400), (63, 0xFFFF8000), (64, 0xFFFF8300),
                 (95, 0xFFFFFF00), (96, 0xFFFBFF04), (127, 0xFF80FF80), (128, 0xFF7CFF83), (159, 0xFF00FFFF),
                 (160, 0xFF00FBFF), (223, 0xFF0000FF), (224, 0xFF0000FB), (255, 0xFF000080)]


def test_jet_table_matches_reference_entries():
    jet = T.jet256()
    for i, want in REFERENCE_JET:
        assert int(jet[i]) == want, (i, hex(int(jet[i])), hex(want))
    # monotone ramps: every channel changes by at most 4 per entry
    ch = np.stack([(jet >> s) & 0xFF for s in (0, 8, 16)], axis=1).astype(int)
    assert np.abs(np.diff(ch, axis=0)).max() <= 4


def test_track_update_truncates_and_holds_in_roi():
    poi = np.array([[50, 50], [50, 50], [20, 90]], np.int32)
    u = np.array([1.9, -1.9, 30.0], np.float32)
    v = np.array([-0.5, 2.5, -30.0], np.float32)
    p, au, av = T.track_update(poi, u, v, np.zeros(3, np.float32), np.zeros(3, np.float32), 15, 85, 15, 95)
    np.testing.assert_array_equal(p, [[50, 51], [52, 49], [15, 95]])
    np.testing.assert_array_equal(au, u)


def test_write_ppm(tmp_path):
    from tw_gb300.track import write_ppm
    tex = np.array([[0xFF0000FF, 0xFF00FF00], [0xFFFF0000, 0xFF123456]], np.uint32)
    path = tmp_path / "c.ppm"
    write_ppm(path, tex)
    raw = path.read_bytes()
    assert raw.startswith(b"P6\n2 2\n255\n")
    assert list(raw[-12:]) == [255, 0, 0, 0, 255, 0, 0, 0, 255, 0x56, 0x34, 0x12]


@pytest.mark.gpu
def test_tracking_loop_and_colormap():
    ref, tars, g = synth.camera_sequence(200, 176, frames=6, seed=41, r=10, grid=9, margin=12)
    frames = [ref] + tars
    interval = 3
    p = dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r, g.grid,
                        g.grid, g.margin, g.margin, g.max_iter, g.delta_p)
    tr = __import__("tw_gb300.track", fromlist=["DICTracker"]).DICTracker(p, refresh_interval=interval)
    poi = dic.poi_positions(p)
    acc_u = np.zeros(len(poi), np.float32)
    acc_v = np.zeros(len(poi), np.float32)
    bounds = (g.start_y + g.subset_r, g.start_y + g.roi_h - 1 - g.subset_r, g.start_x + g.subset_r,
              g.start_x + g.roi_w - 1 - g.subset_r)
    last = None
    cur_ref = None
    moved = False
    for k, img in enumerate(frames, 1):
        out = tr.process(img)
        if (k - 1) % interval == 0:
            if k > interval:
                poi, acc_u, acc_v = T.track_update(poi, last["u"], last["v"], acc_u, acc_v, *bounds)
                moved = moved or bool((poi != dic.poi_positions(p)).any())
            cur_ref = img
        np.testing.assert_array_equal(out["poi"], poi, err_msg=f"frame {k}")
        np.testing.assert_array_equal(out["acc_u"], acc_u)
        np.testing.assert_array_equal(out["acc_v"], acc_v)
        # this frame against the current reference at the current POIs, by the oracle
        u_or, v_or, z_or, st_or = O.fftcc(cur_ref, img, out["poi"], g.subset_r)
        p6_or, it_or, fl_or = O.icgn(cur_ref, img, g, out["poi"], u_or, v_or)
        both = (out["flags"] == 0) & (fl_or == 0)
        assert both.mean() > 0.9, k
        bad = (np.abs(out["u"] - p6_or[:, 0]) > 1e-3) | (np.abs(out["v"] - p6_or[:, 3]) > 1e-3)
        assert bad[both].sum() <= 0.01 * both.sum() + 1, (k, bad[both].sum())
        last = out
    assert moved  # the POIs did move at a refresh
    rh, rw = g.roi_h, g.roi_w
    tu = np.zeros((rh, rw), np.uint32)
    tv = np.zeros((rh, rw), np.uint32)
    tr.colormap(tu, tv, -3.0, 3.0, -3.0, 3.0)
    wu, wv = T.colormap(np.zeros_like(tu), np.zeros_like(tv), last["poi"], last["u"], last["v"], last["acc_u"],
                        last["acc_v"], g.start_x, g.start_y, rw, rh, -3.0, 3.0, -3.0, 3.0)
    # overlapping 3x3 blocks: the GPU's write order is unspecified, so compare
    # pixels drawn by exactly one POI, and that every drawn pixel has a colour
    ys = last["poi"][:, 0] + np.trunc(last["v"]).astype(int) - g.start_y
    xs = last["poi"][:, 1] + np.trunc(last["u"]).astype(int) - g.start_x
    cover = np.zeros((rh, rw), int)
    for y, x in zip(ys, xs):
        cover[max(0, y - 1):y + 2, max(0, x - 1):x + 2] += 1
    one = cover == 1
    np.testing.assert_array_equal(tu[one], wu[one])
    np.testing.assert_array_equal(tv[one], wv[one])
    assert ((tu != 0) == (cover > 0)).all()
