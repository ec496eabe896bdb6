"""GPU parity of the mapping receivers (PachMapReceiver) against the FP64 oracle.

Tolerances, stated per test:
* one ray between parallel walls through one receiver: every bin within 2e-5 relative (FP32 path
  lengths and air factors against FP64), both walks;
* pure specular, 48-receiver audience plane: map totals per receiver and band within 1e-3 relative,
  98 % of occupied bins within 1e-3 -- the rest are 1 ms bin-edge straddles, sphere grazes and
  cell-boundary ties of the FP32 walk;
* stochastic mode with shared streams: map totals within 1 %, parameter maps within a tenth of a
  JND (5 % T30/EDT, 1 dB C80, 5 points D50) where both sides are finite;
* the device parameter kernel against the host AcousticalMath on the same histograms: 1e-9 relative.
"""
import types

import numpy as np
import pytest

from oracle import oracle as O
from pachydermacoustic_universal_gb300 import rooms, tracer
from pachydermacoustic_universal_gb300.simulation import AcousticalMath

pytestmark = pytest.mark.gpu
ALPHA = 0.1
JND = {"t_x": 0.05, "edt": 0.05, "clarity": 1.0, "definition": 5.0}


def _box(L=(10.0, 8.0, 4.0), alpha=ALPHA):
    b = rooms._Builder()
    rooms._box_faces(b, (0, 0, 0), L)
    v, offs, idx = b.arrays()
    P = offs.size - 1
    return rooms.SceneArrays(v, offs, idx, np.full((P, 8), alpha), np.zeros((P, 8)), np.zeros((P, 8)))


def _shifted(w, org, off=(3.0, 2.0, 1.0)):
    """The workload and map moved off the coordinate planes.  The reference's broadband grid walk
    steers by the sign of the ray's position, so a hit on a wall at x = 0 (say) leaves a position
    whose sign is that of a rounding residual (+-1e-7 in FP32, +-1e-16 in FP64): the two engines
    then walk differently by construction.  Away from 0 every position is safely positive."""
    off = np.asarray(off)
    sc = w.scene
    scene = rooms.SceneArrays(sc.vertices + off, sc.poly_offsets, sc.poly_indices, sc.absorption, sc.scattering,
                              sc.transmission)
    srcs = [rooms.SourceSpec(tuple(np.add(s.origin, off)), s.power_db, s.kind) for s in w.sources]
    recs = [rooms.ReceiverSpec(tuple(np.add(r.origin, off)), r.radius) for r in w.receivers]
    return rooms.Workload(w.name + "_shifted", scene, srcs, recs, w.rays, w.cutoff_s), org + off


def _both(w, m, rays, seed, oracle_kw=None, **kw):
    hg, sg = tracer.trace(w, rays=rays, seed=seed, map_receivers=m, **kw)
    om = types.SimpleNamespace(origins=m.origins, increment=m.increment, cutoff_ms=m.cutoff_ms, time_1pt=m.time_1pt,
                               walk=m.walk)
    ho, so = O.trace(w, rays=rays, seed=seed, map_receivers=om, threads=4, **kw, **(oracle_kw or {}))
    return hg, sg, ho, so


def test_single_receiver_matches_oracle_both_walks():
    w = rooms.Workload("box", _box(), [rooms.SourceSpec((2.0, 2.0, 1.5))], [], 1, 2.0)
    for walk in (0, 1):
        m = tracer.MapReceivers(np.array([[5.0, 2.0, 1.5]]), 1.0, 3000.0, walk=walk)
        hg, sg, ho, so = _both(w, m, 1, 1, pure_specular=True, prim_dirs=np.array([[1.0, 0.0, 0.0]]))
        Eg, Eo = hg["map"]["energy"], ho["map_energy"]
        assert np.array_equal(Eg > 0, Eo > 0), walk
        occ = Eo > 0
        np.testing.assert_allclose(Eg[occ], Eo[occ], rtol=2e-5)
        np.testing.assert_allclose(hg["map"]["direct_time"], ho["map_direct"], rtol=1e-15)


@pytest.mark.parametrize("walk", [0, 1])
def test_pure_specular_audience_plane_matches_oracle(walk):
    w, org = _shifted(rooms.shoebox_c1(), rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 1.0))
    m = tracer.MapReceivers(org, 1.0, 2000.0, walk=walk)
    hg, sg, ho, so = _both(w, m, 2000, 5, pure_specular=True)
    assert sg["queue_overflows"] == 0 and sg["capped"] == 0
    Eg, Eo = hg["map"]["energy"], ho["map_energy"]
    np.testing.assert_allclose(Eg.sum(axis=2), Eo.sum(axis=2), rtol=1e-3)
    occ = Eo > 1e-12 * Eo.max()
    rel = np.abs(Eg[occ] - Eo[occ]) / Eo[occ]
    assert np.mean(rel < 1e-3) >= 0.98, np.mean(rel < 1e-3)
    np.testing.assert_allclose(hg["map"]["pressure"].sum(axis=2), ho["map_pressure"].sum(axis=2), rtol=1e-3)


def test_walks_differ_as_the_reference_code_does():
    """Walk 0 loses the broadband legs the reference's walk skips; walk 1 keeps every detection."""
    w = rooms.shoebox_c1()
    org = rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 1.0)
    e = {}
    for walk in (0, 1):
        h, _ = tracer.trace(w, rays=3000, seed=7, pure_specular=True,
                            map_receivers=tracer.MapReceivers(org, 1.0, 2000.0, walk=walk))
        e[walk] = h["map"]["energy"].sum()
    assert e[0] < 0.9 * e[1]


def test_stochastic_map_and_parameter_maps_match_oracle():
    w, org = _shifted(rooms.shoebox_c1(), rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 1.0))
    m = tracer.MapReceivers(org, 1.0, 2000.0)
    n = 400
    ds = tracer.DeviceScene(w.scene)
    params = tracer.make_params(rays=n, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=w.cutoff_s * 1000.0,
                                seed=21, map_receivers=m)
    run = tracer.Run(ds, w.sources, w.receivers, params)
    run.wait()
    hm = run.map_histograms(scaled=True)
    pg = run.map_parameters(30, 80)
    run.close()
    om = types.SimpleNamespace(origins=org, increment=1.0, cutoff_ms=2000.0, time_1pt=False, walk=0)
    ho, _ = O.trace(w, rays=n, seed=21, map_receivers=om, threads=4)
    Eo = ho["map_energy"] / n
    np.testing.assert_allclose(hm["energy"].sum(axis=2), Eo.sum(axis=2), rtol=1e-2)
    po = {k: np.zeros(Eo.shape[:2]) for k in JND}
    for i in range(Eo.shape[0]):
        for o in range(8):
            sch = O.schroeder(Eo[i, o])
            po["t_x"][i, o] = O.t_x(sch, 30, 1000)
            po["edt"][i, o] = O.edt(sch, 1000)
            po["clarity"][i, o] = O.clarity(Eo[i, o], 1000.0, 0.08, 0.0)
            po["definition"][i, o] = O.definition(Eo[i, o], 1000.0, 0.05, 0.0)
    for k, j in JND.items():
        a, b = pg[k], po[k]
        ok = np.isfinite(a) & np.isfinite(b)
        assert ok.mean() > 0.9, (k, ok.mean())
        err = np.abs(a[ok] - b[ok]) / (np.abs(b[ok]) if k in ("t_x", "edt") else 1.0)
        assert err.max() <= 0.1 * j, (k, err.max())


def test_parameter_kernel_matches_host_math():
    w = rooms.shoebox_c1()
    org = rooms.audience_plane((2.0, 2.0), (8.0, 6.0), 1.0, 1.0)
    m = tracer.MapReceivers(org, 1.0, 2000.0, walk=1)
    ds = tracer.DeviceScene(w.scene)
    params = tracer.make_params(rays=2000, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=2000.0, seed=3,
                                map_receivers=m)
    run = tracer.Run(ds, w.sources, w.receivers, params)
    run.wait()
    E = run.map_histograms(scaled=True)["energy"]
    for depth, cms in ((30, 80), (20, 50)):
        pg = run.map_parameters(depth, cms)
        for i in range(E.shape[0]):
            for o in range(8):
                sch = AcousticalMath.Schroeder_Integral(E[i, o])
                ref = (AcousticalMath.T_X(sch, depth, 1000), AcousticalMath.EarlyDecayTime(sch, 1000),
                       AcousticalMath.Clarity(E[i, o], 1000, cms / 1000.0, 0.0, False),
                       AcousticalMath.Definition(E[i, o], 1000, 0.05, 0.0, False), E[i, o].sum())
                got = (pg["t_x"][i, o], pg["edt"][i, o], pg["clarity"][i, o], pg["definition"][i, o],
                       pg["energy"][i, o])
                np.testing.assert_allclose(got, ref, rtol=1e-9, equal_nan=True)
    run.close()


def test_one_point_map_matches_oracle():
    w = rooms.shoebox_c1()
    org = rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 2.0)
    m = tracer.MapReceivers(org, 2.0, 2000.0, time_1pt=True, walk=1)
    hg, sg, ho, so = _both(w, m, 1000, 9, pure_specular=True)
    assert hg["map"]["energy"].shape == (org.shape[0], 8, 1)
    np.testing.assert_allclose(hg["map"]["energy"], ho["map_energy"], rtol=2e-3)
    assert not hg["map"]["pressure"].any()


def test_hall_map_matches_oracle_within_jnd():
    w, org = _shifted(rooms.irregular_hall_c2(), rooms.audience_plane((6.0, 4.0), (34.0, 21.0), 1.0, 2.0))
    m = tracer.MapReceivers(org, 2.0, 2000.0)
    n = 300
    hg, sg, ho, so = _both(w, m, n, 11, oracle_kw={"grid_domain": 31})
    assert sg["queue_overflows"] == 0
    np.testing.assert_allclose(hg["map"]["energy"].sum(), ho["map_energy"].sum(), rtol=0.03)


def test_split_ray_tracer_fills_a_pach_map_receiver_and_parameter_maps():
    from pachydermacoustic_universal_gb300.mapping import (Get_Clarity_Map, Get_Definition_Map, Get_EDT_Map,
                                                           Get_RT_Map, MapMesh, PachMapReceiver)
    from pachydermacoustic_universal_gb300.simulation import GeodesicSource, Polygon_Scene, SplitRayTracer
    w, _ = _shifted(rooms.shoebox_c1(), np.zeros((1, 3)))
    room = Polygon_Scene.from_arrays(w.scene)
    src = GeodesicSource([120.0] * 8, w.sources[0].origin)
    mesh = MapMesh.grid((4.0, 3.0), (12.0, 9.0), 2.0, 1.0)
    pm = PachMapReceiver(mesh, src, 1000, 1.0, room, 2000.0, False, True, False, False, False)
    rt = SplitRayTracer(src, pm, room, w.cutoff_length_m, (0, 7), -1, 2000, seed=3)
    rt.Begin()
    rt.Combine_ThreadLocal_Results()
    rt.close()
    h, _ = tracer.trace(w, rays=2000, seed=3, scaled=True, map_receivers=pm.map_receivers())
    np.testing.assert_allclose(pm._E, h["map"]["energy"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose([r.Direct_Time for r in pm.Rec_List], h["map"]["direct_time"], rtol=1e-15)
    for oct in (1, 5):
        maps = {"t_x": Get_RT_Map([pm], 30, oct, [0]), "edt": Get_EDT_Map([pm], oct, [0]),
                "clarity": Get_Clarity_Map([pm], 80, oct, [0]), "definition": Get_Definition_Map([pm], oct, [0])}
        for i in range(pm.Count):
            etc = np.zeros(2000 + 16384)
            etc[:2000] = pm._E[i, oct]
            sch = AcousticalMath.Schroeder_Integral(etc)
            ref = {"t_x": AcousticalMath.T_X(sch, 30, 1000), "edt": AcousticalMath.EarlyDecayTime(sch, 1000),
                   "clarity": AcousticalMath.Clarity(etc, 1000, 0.08, 0.0, False),
                   "definition": AcousticalMath.Definition(etc, 1000, 0.05, 0.0, False)}
            for k in maps:
                np.testing.assert_allclose(maps[k][i], ref[k], rtol=1e-9, equal_nan=True, err_msg=k)
    # each map receiver's filter (Receiver_Bank.Create_Filter / GetFilter) against the FP64 oracle
    from oracle import filters as OF
    assert not pm.HasFilter() and not pm.GetFilter(0).any()
    pm.Create_Filter()
    for i in (0, pm.Count // 2, pm.Count - 1):
        ref = OF.receiver_filters(pm._E[i], pm._P[i], None, None, [120.0] * 8, 1000, directional=False)[0]
        got = pm.GetFilter(i)
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_directional_map_matches_oracle():
    """Directional_Histogram in a map: pressure sqrt(E rho c) and the +/- arrival sums."""
    w, org = _shifted(rooms.shoebox_c1(), rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 1.0))
    m = tracer.MapReceivers(org, 1.0, 2000.0, walk=1, directional=True)
    hg, sg = tracer.trace(w, rays=1500, seed=13, pure_specular=True, map_receivers=m)
    om = types.SimpleNamespace(origins=org, increment=1.0, cutoff_ms=2000.0, time_1pt=False, walk=1, directional=True)
    ho, so = O.trace(w, rays=1500, seed=13, pure_specular=True, map_receivers=om, threads=4)
    g = hg["map"]
    np.testing.assert_allclose(g["energy"].sum(axis=2), ho["map_energy"].sum(axis=2), rtol=1e-3)
    np.testing.assert_allclose(g["pressure"].sum(axis=2), ho["map_pressure"].sum(axis=2), rtol=1e-3)
    for k, ko in (("dir_pos", "map_dir_pos"), ("dir_neg", "map_dir_neg")):
        a, b = g[k].sum(axis=-1), ho[ko].sum(axis=-1)
        np.testing.assert_allclose(a, b, rtol=2e-3, atol=1e-6 * np.abs(b).max())
    assert (g["dir_pos"] >= 0).all() and (g["dir_neg"] <= 0).all()
