"""GPU checks of batch runs (many rooms as one wavefront, pach_batch_begin) and of the graph-mode
device loop: every room of a batch traces exactly as a single run with the same primary numbering."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from pachydermacoustic_universal_gb300 import rooms, tracer  # noqa: E402

pytestmark = pytest.mark.gpu


def _rooms():
    hall = rooms.irregular_hall_c2(target_tris=2000)
    return [rooms.shoebox_c1(), rooms.proposal_room_c4(3), hall]


def test_batch_rooms_match_single_runs():
    ws = _rooms()
    ds = [tracer.DeviceScene(w.scene) for w in ws]
    rays = [3000, 2000, 700]
    seed = 11
    hb, sb = tracer.trace_batch(ws, dscenes=ds, rays=rays, seed=seed)
    off = 0
    seg = 0
    for i, w in enumerate(ws):
        hs, ss = tracer.trace(w, dscene=ds[i], rays=rays[i], seed=seed, ray_begin=off)
        T = hs["energy"].shape[-1]
        for name in ("energy", "pressure", "dir_pos", "dir_neg", "analysis"):
            a, b = hb[i][name][..., :T], hs[name]
            assert np.allclose(a, b, rtol=1e-9, atol=1e-30), (i, name)
        seg += ss["segments"]
        off += rays[i]
    assert sb["segments"] == seg
    assert sb["primaries"] == sum(rays)


def test_batch_scaling_is_per_room():
    ws = _rooms()[:2]
    ds = [tracer.DeviceScene(w.scene) for w in ws]
    rays = [1500, 500]
    raw, _ = tracer.trace_batch(ws, dscenes=ds, rays=rays, seed=3)
    sc, _ = tracer.trace_batch(ws, dscenes=ds, rays=rays, seed=3, scaled=True)
    for i in range(2):
        ns = len(ws[i].sources)
        assert np.allclose(sc[i]["energy"], raw[i]["energy"] * ns / rays[i], rtol=1e-9)


def test_graph_loop_matches_host_loop():
    w = rooms.shoebox_c1()
    ds = tracer.DeviceScene(w.scene)
    hg, sg = tracer.trace(w, dscene=ds, rays=4000, seed=9)
    hh, sh = tracer.trace(w, dscene=ds, rays=4000, seed=9, kernel_timing=True)
    assert sg["segments"] == sh["segments"]
    assert np.allclose(hg["energy"], hh["energy"], rtol=1e-9, atol=1e-30)
    assert sh["trace_ms"] > 0 and sg["trace_ms"] == 0


def test_batch_of_c3_rooms_runs():
    ws = rooms.batched_rooms_c3(n_rooms=16, max_rays=20_000)
    h, s = tracer.trace_batch(ws, rays=[min(w.rays, 600) for w in ws], seed=5)
    assert len(h) == 16
    for i, w in enumerate(ws):
        assert h[i]["energy"].shape[0] == len(w.receivers)
        assert np.all(np.isfinite(h[i]["energy"]))
        assert h[i]["energy"].sum() > 0
    assert s["queue_overflows"] == 0


def test_autotune_picks_and_caches(tmp_path):
    ws = _rooms()[:2]
    ds = [tracer.DeviceScene(w.scene) for w in ws]
    cache = str(tmp_path / "tune.txt")
    t1 = tracer.autotune(ws, dscenes=ds, rays=[2000, 2000], sample_rays=600, cache_path=cache)
    assert t1["from_cache"] == 0 and t1["trials"] >= 5 and t1["segments_per_s"] > 0
    assert t1["wave_kilo_items"] in (2048, 4096, 8192, 16384) and t1["block_threads"] in (128, 256)
    assert t1["blocks_per_sm"] in (4, 6) and t1["traversal"] in (1, 2, 3)
    t2 = tracer.autotune(ws, dscenes=ds, rays=[2000, 2000], sample_rays=600, cache_path=cache)
    assert t2["from_cache"] == 1
    assert all(t2[k] == t1[k] for k in tracer.TUNE_KNOBS)
    # the tuned knobs change scheduling only: same histograms as the defaults
    ha, _ = tracer.trace_batch(ws, dscenes=ds, rays=[800, 400], seed=2, tune=t1)
    hb, _ = tracer.trace_batch(ws, dscenes=ds, rays=[800, 400], seed=2)
    for i in range(2):
        assert np.allclose(ha[i]["energy"], hb[i]["energy"], rtol=1e-9, atol=1e-30)


def test_quantised_nodes_trace_the_same_rays():
    """64-byte nodes hold conservative boxes of the 128-byte ones: the same nearest hits, except that
    the walk order decides exact FP32 ties (a ray through an edge shared by two walls), which sends a
    few rays in a million down the other wall's path."""
    for w in (rooms.shoebox_c1(), rooms.irregular_hall_c2(target_tris=4000)):
        ds = tracer.DeviceScene(w.scene)
        ha, sa = tracer.trace(w, dscene=ds, rays=1500, seed=21, bvh_format=1)
        hb, sb = tracer.trace(w, dscene=ds, rays=1500, seed=21, bvh_format=2)
        assert abs(sa["segments"] - sb["segments"]) <= 1e-4 * sa["segments"]
        assert hb["energy"].sum() == pytest.approx(ha["energy"].sum(), rel=1e-3)


def test_fused_walk_traces_the_same_rays():
    """traversal 3 walks the rays inside the shading kernel with the same walk as the trace kernel's
    one-leaf-at-a-time variant: identical hits, identical histograms."""
    for w in (rooms.shoebox_c1(), rooms.irregular_hall_c2(target_tris=3000)):
        ds = tracer.DeviceScene(w.scene)
        ha, sa = tracer.trace(w, dscene=ds, rays=1500, seed=8, traversal=1)
        hb, sb = tracer.trace(w, dscene=ds, rays=1500, seed=8, traversal=3)
        assert sa["segments"] == sb["segments"]
        assert np.allclose(ha["energy"], hb["energy"], rtol=1e-9, atol=1e-30)


def test_scenes_built_together_equal_scenes_built_one_by_one():
    """pach_scenes_create (parallel host builds) gives the scenes pach_scene_create gives."""
    ws = rooms.batched_rooms_c3(max_rays=20_000)[:6]
    many = tracer.DeviceScene.many([w.scene for w in ws], threads=4)
    one = [tracer.DeviceScene(w.scene) for w in ws]
    for a, b in zip(many, one):
        ia, ib = a.info(), b.info()
        assert ia["n_triangles"] == ib["n_triangles"]
        np.testing.assert_array_equal(ia["poly_area"], ib["poly_area"])
    ha, sa = tracer.trace_batch(ws, dscenes=many, rays=[200] * len(ws), seed=9)
    hb, sb = tracer.trace_batch(ws, dscenes=one, rays=[200] * len(ws), seed=9)
    assert sa["segments"] == sb["segments"] and sa["accel"] == sb["accel"]
    for x, y in zip(ha, hb):
        np.testing.assert_allclose(x["energy"], y["energy"], rtol=1e-12, atol=1e-300)
