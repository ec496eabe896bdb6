"""GPU parity: the sm_103a engine (through the C ABI) against the FP64 oracle and analytic answers.

Tolerances, stated per test:
* emission directions: |d_gpu - d_oracle| < 2e-6 (FP32 vs FP64 of the same uniforms);
* pure-specular shoebox paths: same wall sequence, legs within 1e-4 relative (FP32 geometry);
* pure-specular ETC (oracle (a), the shoebox configuration's 100k primaries): band totals within 1e-4
  relative, 99 % of occupied bins within 1e-3 relative -- the rest are 1 ms bin-edge straddles and
  grazing sphere hits; direction components within 2e-4 of their band's energy total;
* stochastic mode (oracle (b)): both sides draw the same Philox streams, so in the shoebox the
  totals agree within 5e-3 and T30/EDT/C80/D50 within a tenth of a JND (JND: 5 % T30/EDT,
  1 dB C80, 0.05 D50); in the chaotic jittered hall within one JND.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from pachydermacoustic_universal_gb300 import rooms, tracer, _capi
from pachydermacoustic_universal_gb300.simulation import (AcousticalMath, GeodesicSource, Polygon_Scene, Receiver_Bank,
                                                          SplitRayTracer, ThreadState, room_parameters)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
FACE_AXIS_SIDE = {0: (2, 0), 1: (2, 1), 2: (1, 0), 3: (1, 1), 4: (0, 1), 5: (0, 0)}
JND = {"T30": 0.05, "EDT": 0.05, "C80": 1.0, "D50": 5.0}   # T30/EDT relative; C80 dB; D50 percent points


def _shoebox(L, alpha=0.1):
    b = rooms._Builder()
    rooms._box_faces(b, (0, 0, 0), L)
    v, offs, idx = b.arrays()
    P = offs.size - 1
    return rooms.SceneArrays(v, offs, idx, np.full((P, 8), alpha), np.zeros((P, 8)), np.zeros((P, 8)))


def direct_times(w):
    """Direct-sound arrival (s) at each receiver from the nearest source: the start time of the
    C80 / D50 windows (Clarity / Definition startTime)."""
    c = 331.0 + 0.6 * w.scene.temp_c
    return [min(np.linalg.norm(np.subtract(r.origin, s.origin)) for s in w.sources) / c for r in w.receivers]


def params_of(h, w, fs=1000):
    """T30/EDT/C80/D50 per receiver and band from raw energy histograms."""
    E = h["energy"]
    direct = direct_times(w)
    out = {k: np.zeros(E.shape[:2]) for k in JND}
    for r in range(E.shape[0]):
        for o in range(E.shape[1]):
            p = room_parameters(E[r, o], fs, direct[r])
            for k in JND:
                out[k][r, o] = p[k]
    return out


def assert_params_close(pg, po, frac):
    for k, j in JND.items():
        a, b = pg[k], po[k]
        ok = np.isfinite(a) & np.isfinite(b)
        assert ok.mean() > 0.8, (k, ok.mean())
        assert np.array_equal(np.isfinite(a), np.isfinite(b)), k
        if k in ("T30", "EDT"):
            err = np.abs(a[ok] - b[ok]) / np.abs(b[ok])
        else:
            err = np.abs(a[ok] - b[ok])
        assert err.max() <= frac * j, (k, err.max(), frac * j)


# ---------------------------------------------------------------- emission
@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("nsrc", [1, 3])
def test_emission_directions_match_oracle(kind, nsrc):
    n = 2048
    d = tracer.emit_directions(7, 1000, n, nsrc, kind)
    ref = np.array([O.emit_direction(7, 1000 + i, nsrc, kind) for i in range(n)])
    assert np.abs(d - ref).max() < 2e-6
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)


# ---------------------------------------------------------------- traversal
def test_specular_paths_follow_the_image_lattice():
    with open(os.path.join(GOLD, "shoebox_paths.json")) as f:
        g = json.load(f)
    ds = tracer.DeviceScene(_shoebox(tuple(g["size"])))
    o = np.array([r["origin"] for r in g["rays"]])
    d = np.array([r["dir"] for r in g["rays"]])
    nb = 20
    poly, t, pts = tracer.specular_paths(ds, o, d, nb)
    for i, r in enumerate(g["rays"]):
        for b in range(nb):
            assert FACE_AXIS_SIDE[poly[i, b] // 2] == tuple(r["walls"][b]), (i, b)
        np.testing.assert_allclose(t[i], r["legs"][:nb], rtol=1e-4, atol=1e-4)
        np.testing.assert_allclose(pts[i], r["points"][:nb], atol=2e-3)


def _edge_distance(scene, poly, x):
    """Distance of point x to the boundary of polygon `poly`."""
    V = scene.vertices[scene.poly_indices[scene.poly_offsets[poly]:scene.poly_offsets[poly + 1]]]
    best = np.inf
    for k in range(len(V)):
        a, b = V[k], V[(k + 1) % len(V)]
        ab = b - a
        t = np.clip(np.dot(x - a, ab) / np.dot(ab, ab), 0.0, 1.0)
        best = min(best, float(np.linalg.norm(x - (a + t * ab))))
    return best


def test_specular_paths_in_jittered_hall_match_oracle():
    """Per-ray hit sequences of the FP32 walk (with its FP64 re-test) against the FP64 oracle over 8
    bounces: each sequence must match, except certified ties -- a ray whose first differing hit lies
    within TIE_M of an edge of the polygon either side hit (where the two engines' accumulated position
    difference can put the rays on different sides), or whose two candidate hits are equidistant."""
    TIE_M = 5e-3
    w = rooms.irregular_hall_c2(target_tris=20_000)
    ds = tracer.DeviceScene(w.scene)
    rng = np.random.default_rng(9)
    n = 4096
    o = np.repeat(np.array(w.sources[0].origin)[None], n, axis=0)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nb = 8
    pg, tg, xg = tracer.specular_paths(ds, o, d, nb)
    po, to, xo = O.specular_paths(w.scene, o, d, nb, grid_domain=31)
    # first leg from the source: always identical
    assert np.all(pg[:, 0] == po[:, 0])
    same = np.all(pg == po, axis=1)
    assert same.mean() >= 0.995, same.mean()
    for i in np.where(~same)[0]:
        b = int(np.argmax(pg[i] != po[i]))
        tie = abs(tg[i, b] - to[i, b]) <= 1e-4 * max(to[i, b], 1.0)
        for poly, x in ((pg[i, b], xg[i, b]), (po[i, b], xo[i, b])):
            tie = tie or (poly >= 0 and _edge_distance(w.scene, poly, x) <= TIE_M)
        assert tie, ("divergent hit sequence that is not an edge tie", i, b, pg[i, b], po[i, b])
    # hit points of the matching sequences: FP32 drift stays below 2 mm over 8 bounces
    assert np.linalg.norm(xg[same] - xo[same], axis=2).max() < 2e-3
    np.testing.assert_allclose(tg[same], to[same], rtol=2e-3, atol=5e-4)


# ---------------------------------------------------------------- oracle (a): pure specular
def test_pure_specular_etc_matches_oracle():
    """Oracle (a) at the shoebox configuration's full 100k primaries."""
    w = rooms.shoebox_c1()
    n = 100_000
    hg, sg = tracer.trace(w, rays=n, seed=5, pure_specular=True)
    ho, so = O.trace(w, rays=n, seed=5, pure_specular=True, threads=0)
    assert sg["primaries"] == n and sg["queue_overflows"] == 0 and sg["capped"] == 0
    tot_g, tot_o = hg["energy"].sum(axis=2), ho["energy"].sum(axis=2)
    np.testing.assert_allclose(tot_g, tot_o, rtol=1e-4)
    assert abs(sg["segments"] - so["segments"]) <= 1e-4 * so["segments"]
    Eg, Eo = hg["energy"], ho["energy"]
    occ = Eo > 1e-12 * Eo.max()
    rel = np.abs(Eg[occ] - Eo[occ]) / Eo[occ]
    assert np.mean(rel < 1e-3) >= 0.99, np.mean(rel < 1e-3)
    for k in ("pressure", "analysis"):
        np.testing.assert_allclose(hg[k].sum(axis=-1), ho[k].sum(axis=-1), rtol=2e-4, atol=1e-30)
    # a direction component holds one sign of d.x E (a fraction of the band's energy), so its error is
    # bounded by the band's energy total: within 2e-4 of it
    for k in ("dir_pos", "dir_neg"):
        d = np.abs(hg[k].sum(axis=-1) - ho[k].sum(axis=-1)) / tot_o[:, None, :]
        assert d.max() <= 2e-4, (k, d.max())


# ---------------------------------------------------------------- oracle (b): stochastic
def test_stochastic_shoebox_matches_oracle_with_shared_streams():
    w = rooms.shoebox_c1()
    n = 400
    hg, sg = tracer.trace(w, rays=n, seed=21)
    ho, so = O.trace(w, rays=n, seed=21, threads=0)
    assert sg["queue_overflows"] == 0
    np.testing.assert_allclose(hg["energy"].sum(axis=2), ho["energy"].sum(axis=2), rtol=5e-3)
    assert abs(sg["segments"] - so["segments"]) <= 5e-3 * so["segments"]
    assert abs(sg["octave_rays"] - so["octave_rays"]) <= 5e-3 * so["octave_rays"]
    assert_params_close(params_of(hg, w), params_of(ho, w), 0.1)


def test_stochastic_hall_matches_oracle_within_jnd():
    w = rooms.irregular_hall_c2()
    n = 600
    hg, sg = tracer.trace(w, rays=n, seed=3)
    ho, so = O.trace(w, rays=n, seed=3, threads=0, grid_domain=31)
    assert sg["fp64_retests"] > 0 and sg["queue_overflows"] == 0
    np.testing.assert_allclose(hg["energy"].sum(), ho["energy"].sum(), rtol=0.03)
    assert abs(sg["segments"] - so["segments"]) <= 0.03 * so["segments"]
    assert_params_close(params_of(hg, w), params_of(ho, w), 1.0)


# ---------------------------------------------------------------- properties at size
def test_sharding_reproducibility_and_linearity():
    w = rooms.shoebox_c1()
    n = 20_000
    ds = tracer.DeviceScene(w.scene)
    h_all, s_all = tracer.trace(w, dscene=ds, rays=n, seed=8)
    h_a, s_a = tracer.trace(w, dscene=ds, rays=n // 2, seed=8)
    h_b, s_b = tracer.trace(w, dscene=ds, rays=n - n // 2, seed=8, ray_begin=n // 2)
    assert s_a["segments"] + s_b["segments"] == s_all["segments"]
    for k in h_all:
        np.testing.assert_allclose(h_a[k] + h_b[k], h_all[k], rtol=1e-9, atol=1e-300)
    h_rep, s_rep = tracer.trace(w, dscene=ds, rays=n, seed=8)
    assert s_rep["segments"] == s_all["segments"]
    np.testing.assert_allclose(h_rep["energy"], h_all["energy"], rtol=1e-9, atol=1e-300)
    loud = rooms.Workload(w.name, w.scene, [rooms.SourceSpec(w.sources[0].origin, (130.0,) * 8)], w.receivers,
                          w.rays, w.cutoff_s)
    h_loud, s_loud = tracer.trace(loud, dscene=ds, rays=n, seed=8)
    assert s_loud["segments"] == s_all["segments"]
    np.testing.assert_allclose(h_loud["energy"], 10.0 * h_all["energy"], rtol=2e-6, atol=1e-300)


# ---------------------------------------------------------------- the reference's API
def test_split_ray_tracer_api_flow():
    w = rooms.shoebox_c1()
    room = Polygon_Scene.from_arrays(w.scene)
    room.partition()
    src = GeodesicSource([120.0] * 8, w.sources[0].origin, 0)
    bank = Receiver_Bank([r.origin for r in w.receivers], src, room, 1000, 2000.0)
    for r in bank.Rec_List:
        r.Radius = 0.5
    rt = SplitRayTracer(src, bank, room, 2.0 * room.Sound_speed(0), [0, 7], -1, 3000, seed=4)
    assert rt.Sim_Type() == "Stochastic Ray Tracing"
    rt.Begin()
    seen = rt.ProgressMsg()
    assert isinstance(seen, str)
    rt.Combine_ThreadLocal_Results()
    assert rt.ThreadState() == ThreadState.Stopped
    raw, st = tracer.trace(w, rays=3000, seed=4)
    for i, rec in enumerate(rt.GetReceiver.Rec_List):
        np.testing.assert_allclose(rec.GetEnergyHistogram(3), raw["energy"][i, 3] / 3000, rtol=1e-9, atol=1e-300)
        np.testing.assert_allclose(rec.GetEnergyHistogram(8), raw["energy"][i].sum(axis=0) / 3000, rtol=1e-9, atol=1e-300)
    assert 0.0 <= rt.PercentLost < 1.0
    rt.close()


# ---------------------------------------------------------------- errors
def test_invalid_runs_are_rejected():
    w = rooms.shoebox_c1()
    ds = tracer.DeviceScene(w.scene)
    with pytest.raises(_capi.PachError) as ei:
        tracer.trace(w, dscene=ds, rays=10, ray_begin=-1)
    assert ei.value.status == 1
    with pytest.raises(_capi.PachError) as ei:  # convergence mode takes no emission overrides
        tracer.trace(w, dscene=ds, rays=0, prim_dirs=np.zeros((1, 3)))
    assert ei.value.status == 1 and "convergence mode" in str(ei.value)
    with pytest.raises(_capi.PachError):
        tracer.trace(w, dscene=ds, rays=10, oct_range=(3, 9))
    bad = rooms.Workload(w.name, w.scene, w.sources, [rooms.ReceiverSpec((1, 1, 1), -0.5)], 10, 2.0)
    with pytest.raises(_capi.PachError):
        tracer.trace(bad, dscene=ds)
    lossless = rooms.SceneArrays(w.scene.vertices, w.scene.poly_offsets, w.scene.poly_indices,
                                 np.zeros_like(w.scene.absorption), np.zeros_like(w.scene.scattering),
                                 w.scene.transmission)
    with pytest.raises(_capi.PachError) as ei:
        tracer.trace(rooms.Workload(w.name, lossless, w.sources, w.receivers, 10, 2.0))
    assert "would not terminate" in str(ei.value)


def test_cancel_stops_between_chunks():
    w = rooms.irregular_hall_c2()
    ds = tracer.DeviceScene(w.scene)
    params = tracer.make_params(rays=2_000_000, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=3000.0, seed=1,
                                feed_batch=1 << 14)
    run = tracer.Run(ds, w.sources, w.receivers, params)
    run.cancel()
    with pytest.raises(_capi.PachError) as ei:
        run.wait()
    assert ei.value.status == 5
    p = run.poll()
    assert p["state"] == 3 and p["rays_done"] < 2_000_000
    run.close()
