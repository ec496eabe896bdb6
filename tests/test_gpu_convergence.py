"""Convergence mode on the GPU (SplitRayTracer with rayCount < 1; TaskAll:111-176, 300-330, 783-1107)
against the FP64 oracle's restatement (oracle/convergence.py), whose stopping points are committed in
tests/golden/convergence.json (made by tests/golden/make_convergence.py: the oracle needs about a
minute per mode).

Both engines trace revolutions of 80 primaries per source on the same Philox streams and replay the
reference's checks after each revolution, so the run must stop after the same revolution, watch the
same receivers, and end with the same band energies (within 1 %: FP32 geometry against FP64)."""
import json
import os

import numpy as np
import pytest

from pachydermacoustic_universal_gb300 import rooms, tracer
from pachydermacoustic_universal_gb300.simulation import GeodesicSource, Polygon_Scene, Receiver_Bank, SplitRayTracer

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "convergence.json")


def _fixture():
    with open(GOLD) as f:
        return json.load(f)


def _workload():
    w = rooms.shoebox_c1()
    w.cutoff_s = 1.0
    return w


@pytest.mark.parametrize("ray_count", [0, -1])
def test_convergence_mode_stops_where_the_oracle_stops(ray_count):
    g = _fixture()
    case = next(c for c in g["cases"] if c["ray_count"] == ray_count)
    w = _workload()
    h, st = tracer.trace(w, rays=ray_count, seed=g["seed"], max_rays=40000)
    assert st["converged"] == 1 and case["converged"]
    assert list(st["check_receivers"]) == list(case["check_receivers"])
    assert st["revolutions"] == case["revolutions"], (st["revolutions"], case["revolutions"])
    assert st["primaries"] == case["primaries"] == 80 * case["revolutions"]
    np.testing.assert_allclose(h["energy"].sum(axis=2), np.array(case["band_energy"]), rtol=1e-2)
    assert abs(st["segments"] - case["segments"]) <= 1e-2 * case["segments"]


def test_convergence_mode_caps_at_max_rays_and_scales_by_the_primaries_traced():
    w = _workload()
    ds = tracer.DeviceScene(w.scene)
    h, st = tracer.trace(w, dscene=ds, rays=0, seed=5, max_rays=400)
    assert st["converged"] == 0 and st["revolutions"] == 5 and st["primaries"] == 400
    raw, _ = tracer.trace(w, dscene=ds, rays=400, seed=5)
    np.testing.assert_allclose(h["energy"], raw["energy"], rtol=1e-9, atol=1e-300)
    hs, _ = tracer.trace(w, dscene=ds, rays=0, seed=5, max_rays=400, scaled=True)
    np.testing.assert_allclose(hs["energy"], raw["energy"] / 400, rtol=1e-9, atol=1e-300)


def test_split_ray_tracer_runs_convergence_mode():
    g = _fixture()
    case = next(c for c in g["cases"] if c["ray_count"] == -1)
    w = _workload()
    room = Polygon_Scene.from_arrays(w.scene)
    room.partition()
    src = GeodesicSource([120.0] * 8, w.sources[0].origin, 0)
    bank = Receiver_Bank([r.origin for r in w.receivers], src, room, 1000, 1000.0)
    for r in bank.Rec_List:
        r.Radius = 0.5
    rt = SplitRayTracer(src, bank, room, 1.0 * room.Sound_speed(0), [0, 7], -1, -1, seed=g["seed"], max_rays=40000)
    rt.Begin()
    assert "until convergence" in rt.ProgressMsg() or "Preparing" in rt.ProgressMsg()
    rt.Combine_ThreadLocal_Results()
    n = case["primaries"]
    assert rt._currentRay[0] == n
    tot = np.array(case["band_energy"])
    for i, rec in enumerate(rt.GetReceiver.Rec_List):
        e = np.array([rec.GetEnergyHistogram(o).sum() for o in range(8)])
        np.testing.assert_allclose(e, tot[i] / n, rtol=1e-2)
    rt.close()
