"""Autotuner (twdic_frame_autotune): it picks among launch shapes that all
meet the parity bar, records its choice in a cache file keyed by GPU and
geometry, and reuses it without timing."""
import numpy as np
import pytest

from oracle import compare as C
from oracle import oracle as O
from tw_gb300 import PATH_FAST, dic, synth

pytestmark = pytest.mark.gpu


def _params(g):
    return dic.make_params(g.img_w, g.img_h, g.start_x, g.start_y, g.roi_w, g.roi_h, g.subset_r, g.subset_r,
                           g.grid, g.grid, g.margin, g.margin, g.max_iter, g.delta_p, PATH_FAST)


def test_fftcc_tiles_give_identical_results():
    """Groups per CTA and POIs per group batch change only the schedule: each
    POI's GEMM rows and exact re-evaluation are the same."""
    pair, g = synth.plain_512()
    ref = None
    for groups in (0, 1):
        for ppg in (0, 2, 1):
            f = dic.DICFrame(_params(g))
            f.set_fftcc_tuning(1, groups, ppg)
            f.set_reference(pair.ref)
            o = f.alloc_outputs()
            f.process(pair.tar, **o)
            if ref is None:
                ref = o
            for k in o:
                np.testing.assert_array_equal(o[k], ref[k], err_msg=f"groups {groups} ppg {ppg} {k}")


def test_autotune_choice_meets_parity_and_is_cached(tmp_path):
    pair, g = synth.plain_512()
    nx, ny, _ = O.num_pois(g.roi_w, g.roi_h, g.subset_r, g.grid, g.margin)
    poi = O.poi_positions(g.start_x, g.start_y, nx, ny, g.margin, g.subset_r, g.grid)
    u_or, v_or, z_or, st_or = O.fftcc(pair.ref, pair.tar, poi, g.subset_r)
    p6_or, it_or, fl_or = O.icgn(pair.ref, pair.tar, g, poi, u_or, v_or)
    cache = tmp_path / "tuning.txt"
    f = dic.DICFrame(_params(g))
    f.set_reference(pair.ref)
    t = f.autotune(pair.tar, cache_path=cache)
    assert t["from_cache"] == 0 and t["icgn_threads"] in (32, 64, 128, 256, 512, 1024)
    assert t["icgn_sampler"] in (0, 1, 2) and t["icgn_chunk"] in (0, 32, 64) and t["icgn_unroll"] in (2, 4, 8)
    assert t["icgn_ms"] > 0 and t["fftcc_ms"] > 0
    assert f.tuning()["icgn_threads"] == t["icgn_threads"]
    o = f.alloc_outputs()
    f.process(pair.tar, **o)
    rep = C.icgn_parity(o["p6"], o["iters"], o["flags"], p6_or, it_or, fl_or, r=g.subset_r)
    assert rep.ok(), (t, rep)
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and "|r16x16|" in lines[0]
    # a second handle with the same geometry takes the cached choice
    f2 = dic.DICFrame(_params(g))
    f2.set_reference(pair.ref)
    t2 = f2.autotune(pair.tar, cache_path=cache)
    assert t2["from_cache"] == 1
    for k in ("icgn_threads", "icgn_sampler", "icgn_chunk", "icgn_unroll", "fftcc_groups", "fftcc_pois_per_group"):
        assert t2[k] == t[k]
    assert len(cache.read_text().strip().splitlines()) == 1


def test_damaged_cache_entry_is_measured_again(tmp_path):
    """A cached line with values no setter accepts (an internal sampler
    number, an unroll of 3) is skipped: the shapes are measured again, the
    new choice is appended, and that one is reused."""
    pair, g = synth.small_case()
    cache = tmp_path / "tuning.txt"
    f = dic.DICFrame(_params(g))
    f.set_reference(pair.ref)
    f.autotune(pair.tar, cache_path=cache)
    key, vals = cache.read_text().strip().splitlines()[0].split(" ", 1)
    v = vals.split()
    v[2], v[4] = "4", "3"  # icgn_sampler, icgn_unroll
    cache.write_text(key + " " + " ".join(v) + "\n")
    f2 = dic.DICFrame(_params(g))
    f2.set_reference(pair.ref)
    t2 = f2.autotune(pair.tar, cache_path=cache)
    assert t2["from_cache"] == 0 and t2["icgn_sampler"] in (0, 1, 2) and t2["icgn_unroll"] in (2, 4, 8)
    assert len(cache.read_text().strip().splitlines()) == 2
    f3 = dic.DICFrame(_params(g))
    f3.set_reference(pair.ref)
    t3 = f3.autotune(pair.tar, cache_path=cache)
    assert t3["from_cache"] == 1 and t3["icgn_sampler"] == t2["icgn_sampler"]
    assert t3["icgn_unroll"] == t2["icgn_unroll"]
