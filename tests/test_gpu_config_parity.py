"""GPU parity on every benchmark configuration: the sm_103a tracer (through the C ABI) against the FP64
oracle's runs of the same seeds, committed in tests/golden/config_parity.json (made by
tests/golden/make_config_parity.py; the oracle needs minutes per case).

Both sides draw the same Philox streams (seed, primary, split-tree stream), so each GPU run is paired
with the oracle run of its seed: where the FP32 walk and the FP64 walk make the same decisions the two
histograms are the same up to FP32 rounding, and the paired difference of a parameter is the error
the FP32 geometry and decay math add.  Cases:

* c1  the 10 x 8 x 4 m shoebox, 5 seeds x 2000 primaries
* c2  the 40 x 25 x 15 m jittered hall (~20k triangles), 5 seeds x 20000 primaries
* c3  rooms 14, 07, 40, 62 of the 64-room batch (612-36k triangles), one batch run, 2000 primaries each
* c5  the 120 x 90 x 35 m arena (~500k triangles), 3 seeds x 20000 primaries

Tolerances (JND, ISO 3382-1 Annex A: 5 % T30/EDT, 1 dB C80, 5 points D50):
* c1, c2: the mean over seeds of each receiver-band parameter within 0.25 JND of the oracle's mean and
  every single paired run within 0.5 JND; c3: each room's run within 0.5 JND;
* c5: the arena's 64 small receivers in a 378,000 m^3 volume collect too few detections at 20k
  primaries for a JND statement per receiver (the oracle's own seed spread is about 4 JND on T30,
  10 on EDT); there the seed means must lie within two combined standard errors for every receiver
  and band, and the curve summed over all receivers must match within 0.25 JND per paired run;
* band energy totals within 1 % per receiver and band (c5: 5 %), segment counts within 1 %.
The measured FP32-vs-FP64 error table (mean and largest |difference| per configuration, band and
parameter) is written as JSON when PACH_ERROR_TABLE names a file.
"""
import json
import os

import numpy as np
import pytest

from pachydermacoustic_universal_gb300 import rooms, tracer
from pachydermacoustic_universal_gb300.simulation import room_parameters

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "config_parity.json")
JND = {"T30": 0.05, "EDT": 0.05, "C80": 1.0, "D50": 5.0}
RELATIVE = {"T30": True, "EDT": True, "C80": False, "D50": False}
MEAN_TOL_JND = 0.25
RUN_TOL_JND = 0.5
ENERGY_RTOL = 1e-2


def _fixture():
    with open(GOLD) as f:
        return json.load(f)


def _arr(rows):
    return np.array([[np.nan if x is None else x for x in row] for row in rows], dtype=float)


def _workload(name):
    if name.startswith("batched_rooms_c3["):
        return rooms.batched_rooms_c3()[int(name[len("batched_rooms_c3["):-1])]
    return getattr(rooms, name)()


def _direct_times(w):
    c = 331.0 + 0.6 * w.scene.temp_c
    return [min(np.linalg.norm(np.subtract(r.origin, s.origin)) for s in w.sources) / c for r in w.receivers]


def _parameters(E, w, fs=1000):
    direct = _direct_times(w)
    out = {k: np.zeros(E.shape[:2]) for k in JND}
    for r in range(E.shape[0]):
        for o in range(E.shape[1]):
            p = room_parameters(E[r, o], fs, direct[r])
            for k in JND:
                out[k][r, o] = p[k]
    return out


def _aggregate(E, w, fs=1000):
    """The four parameters [8] of the receivers' summed curve per band, windows from the earliest
    direct arrival (the fixture's agg_* statistic)."""
    etc = E.sum(axis=0)
    start = min(_direct_times(w))
    out = {k: np.zeros(E.shape[1]) for k in JND}
    for o in range(E.shape[1]):
        p = room_parameters(etc[o], fs, start)
        for k in JND:
            out[k][o] = p[k]
    return out


def gpu_runs(case):
    """GPU side of a fixture case: per record, parameters [R][8], band energy [R][8] and segments."""
    recs = _fixture()[case]
    out = []
    if case == "c3":
        ws = [_workload(r["workload"]) for r in recs]
        ds = tracer.DeviceScene.many([w.scene for w in ws])
        hs, st = tracer.trace_batch(ws, dscenes=ds, seed=recs[0]["seed"], rays=[r["rays"] for r in recs],
                                    ray_begin=recs[0]["ray_begin"])
        seg = st["segments"]
        for w, h in zip(ws, hs):
            out.append({"params": _parameters(h["energy"], w), "band_energy": h["energy"].sum(axis=2),
                        "segments": None, "batch_segments": seg})
        return recs, out
    w = _workload(recs[0]["workload"])
    ds = tracer.DeviceScene(w.scene)
    for r in recs:
        h, st = tracer.trace(w, dscene=ds, rays=r["rays"], ray_begin=r.get("ray_begin", 0), seed=r["seed"])
        assert st["queue_overflows"] == 0 and st["capped"] == 0
        out.append({"params": _parameters(h["energy"], w), "agg": _aggregate(h["energy"], w),
                    "band_energy": h["energy"].sum(axis=2), "segments": st["segments"]})
    return recs, out


def _diff(k, g, o):
    """Paired difference in the parameter's own unit (relative for T30/EDT)."""
    return (g - o) / np.abs(o) if RELATIVE[k] else g - o


def error_table(case, recs, runs):
    """Per parameter and band: mean and largest |GPU - oracle| over receivers and seeds, in the
    parameter's unit (percent for T30/EDT, dB for C80, points for D50) and in JND."""
    tab = {}
    for k in JND:
        ds = [_diff(k, g["params"][k], _arr(r[k])) for g, r in zip(runs, recs)]  # per run [R][8]
        scale = 100.0 if RELATIVE[k] else 1.0
        band = []
        for o in range(8):
            v = np.abs(np.concatenate([d[:, o] for d in ds]))
            v = v[np.isfinite(v)]
            band.append({"mean": float(v.mean() * scale) if v.size else None,
                         "max": float(v.max() * scale) if v.size else None,
                         "max_jnd": float(v.max() / JND[k]) if v.size else None, "n": int(v.size)})
        tab[k] = band
    return tab


def _write_table(case, tab):
    path = os.environ.get("PACH_ERROR_TABLE")
    if not path:
        return
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[case] = tab
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def _check(case, recs, runs, mean_tol, spread_mode=False, energy_rtol=ENERGY_RTOL):
    """Per parameter: both engines find the same parameters finite; then either JND bounds on every
    paired run and on the seed means (parameters the runs determine: c1, c2, c3), or -- where the
    receivers' own curves are too sparse for a JND statement at oracle-affordable ray counts (the
    arena) -- seed means within two combined standard errors for every receiver and band, and JND
    bounds on the receivers' summed curve per band."""
    for k, j in JND.items():
        g = np.stack([x["params"][k] for x in runs])
        o = np.stack([_arr(r[k]) for r in recs])
        fin_g, fin_o = np.isfinite(g), np.isfinite(o)
        assert np.mean(fin_g == fin_o) >= 0.99, (case, k, np.mean(fin_g == fin_o))
        both = fin_g & fin_o
        assert both.mean() > 0.5, (case, k, both.mean())
        if not spread_mode:
            d = np.abs(_diff(k, g, o))
            worst = np.nanmax(np.where(both, d, np.nan))
            assert worst <= RUN_TOL_JND * j, (case, k, "paired run", worst / j)
            if mean_tol is not None:
                ok = np.all(both, axis=0)
                dm = np.abs(_diff(k, g.mean(axis=0), o.mean(axis=0)))[ok]
                assert dm.max() <= mean_tol * j, (case, k, "seed mean", dm.max() / j)
            continue
        ok = np.all(both, axis=0)
        se = np.sqrt(g.var(axis=0, ddof=1) / g.shape[0] + o.var(axis=0, ddof=1) / o.shape[0])
        z = np.abs(g.mean(axis=0) - o.mean(axis=0))[ok] / np.maximum(se[ok], 1e-300)
        assert z.max() <= 2.0, (case, k, "seed mean in combined standard errors", z.max())
        if "agg_" + k in recs[0]:
            ga = np.stack([x["agg"][k] for x in runs])
            oa = np.stack([np.array([np.nan if v is None else v for v in r["agg_" + k]]) for r in recs])
            da = np.abs(_diff(k, ga, oa))
            assert np.nanmax(da) <= MEAN_TOL_JND * j, (case, k, "summed curve, paired run", np.nanmax(da) / j)
    for x, r in zip(runs, recs):
        eg, eo = x["band_energy"], _arr(r["band_energy"])
        m = eo > 0
        np.testing.assert_allclose(eg[m], eo[m], rtol=energy_rtol)
        if x["segments"] is not None:
            assert abs(x["segments"] - r["segments"]) <= 0.01 * r["segments"], (case, x["segments"], r["segments"])


@pytest.mark.parametrize("case", ["c1", "c2"])
def test_stochastic_configuration_matches_oracle_over_seeds(case):
    recs, runs = gpu_runs(case)
    assert len(recs) >= 5
    _write_table(case, error_table(case, recs, runs))
    _check(case, recs, runs, MEAN_TOL_JND)


def test_arena_matches_oracle_within_its_seed_spread():
    recs, runs = gpu_runs("c5")
    assert len(recs) >= 3
    _write_table("c5", error_table("c5", recs, runs))
    _check("c5", recs, runs, None, spread_mode=True, energy_rtol=5e-2)


def test_batch_rooms_each_match_oracle():
    recs, runs = gpu_runs("c3")
    assert len(recs) >= 4
    _write_table("c3", error_table("c3", recs, runs))
    for x, r in zip(runs, recs):  # rooms differ in receiver count: one room at a time
        _check("c3 " + r["workload"], [r], [x], None)
    tot = sum(r["segments"] for r in recs)
    assert abs(runs[0]["batch_segments"] - tot) <= 0.01 * tot
