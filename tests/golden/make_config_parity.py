"""Generates tests/golden/config_parity.json: FP64-oracle room-acoustic parameters of every benchmark
configuration, the reference side of the GPU parity tests (tests/test_gpu_config_parity.py).

Each case traces a seeded workload with the CPU FP64 restatement of the reference's split ray tracer
(oracle/, TaskAll:335-536) and keeps, per receiver and octave band, the band's total raw energy and
T30 / EDT / C80 / D50 as AcousticalMath derives them (Classes_Math.cs:282-586, 934-962; the oracle's
own FP64 restatement of those functions), the same four of the receivers' summed curve per band
(agg_*), plus the run's segment and octave-ray counts.  The GPU
tracer draws the same Philox streams, so each GPU run is compared with the oracle run of the same
seed; the per-seed differences are the FP32-vs-FP64 error of each parameter.

Cases (the oracle needs minutes for them, so they are computed once here and committed):
  c1    the 10 x 8 x 4 m shoebox (12 triangles), 5 seeds x 2000 primaries, voxel grid 7
  c2    the 40 x 25 x 15 m jittered hall (~20k triangles), 5 seeds x 20000 primaries, grid 31
  c3    rooms 14, 07, 40 and 62 of the 64-room batch (612 to 36k triangles), 2000 primaries each,
        numbered as one batch run of the four rooms numbers them (room k from k x 2000)
  c5    the 120 x 90 x 35 m arena (~500k triangles), 3 seeds x 20000 primaries, grid 128

Run:  python tests/golden/make_config_parity.py [case ...]   (all cases by default; 8 cores: ~20 min)
Test infrastructure: imports the oracle as the checker.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import oracle as O  # noqa: E402
from pachydermacoustic_universal_gb300 import rooms  # noqa: E402

OUT = os.path.join(HERE, "config_parity.json")
C3_ROOMS = (14, 7, 40, 62)


def cases():
    """Per case: (workload factory, seed, primaries, first primary, voxel grid domain) for each oracle run."""
    return {
        "c1": [("shoebox_c1", s, 2000, 0, 7) for s in (101, 102, 103, 104, 105)],
        "c2": [("irregular_hall_c2", s, 20000, 0, 31) for s in (201, 202, 203, 204, 205)],
        "c3": [(f"batched_rooms_c3[{i}]", 301, 2000, 2000 * k, 31) for k, i in enumerate(C3_ROOMS)],
        "c5": [("arena_c5", s, 20000, 0, 128) for s in (501, 502, 503)],
    }


def make_workload(name: str):
    if name.startswith("batched_rooms_c3["):
        return rooms.batched_rooms_c3()[int(name[len("batched_rooms_c3["):-1])]
    return getattr(rooms, name)()


def direct_times(w):
    """Direct arrival (s) at each receiver from its nearest source: the C80 / D50 start time."""
    c = 331.0 + 0.6 * w.scene.temp_c
    return [min(np.linalg.norm(np.subtract(r.origin, s.origin)) for s in w.sources) / c for r in w.receivers]


def oracle_parameters(E, w, fs=1000):
    """T30, EDT, C80, D50 [R][8] of raw energy histograms E [R][8][T] by the oracle's AcousticalMath."""
    direct = direct_times(w)
    out = {k: np.zeros(E.shape[:2]) for k in ("T30", "EDT", "C80", "D50")}
    for r in range(E.shape[0]):
        for o in range(E.shape[1]):
            etc = E[r, o]
            sch = O.schroeder(etc)
            out["T30"][r, o] = O.t_x(sch, 30, fs)
            out["EDT"][r, o] = O.edt(sch, fs)
            out["C80"][r, o] = O.clarity(etc, fs, 0.08, direct[r], False)
            out["D50"][r, o] = O.definition(etc, fs, 0.05, direct[r], False)
    return out


def aggregate_parameters(E, w, fs=1000):
    """T30, EDT, C80, D50 [8] of the receivers' summed energy-time curve per band, the C80 / D50 windows
    starting at the earliest direct arrival: a room-average statistic that stays determined when each
    small receiver's own curve is too sparse (the arena at affordable oracle ray counts)."""
    start = min(direct_times(w))
    out = {k: np.zeros(E.shape[1]) for k in ("T30", "EDT", "C80", "D50")}
    for o in range(E.shape[1]):
        etc = E[:, o].sum(axis=0)
        sch = O.schroeder(etc)
        out["T30"][o] = O.t_x(sch, 30, fs)
        out["EDT"][o] = O.edt(sch, fs)
        out["C80"][o] = O.clarity(etc, fs, 0.08, start, False)
        out["D50"][o] = O.definition(etc, fs, 0.05, start, False)
    return out


def _json_num(a):
    """Nested lists with non-finite values as None (JSON has no NaN)."""
    return [[(float(x) if np.isfinite(x) else None) for x in row] for row in np.asarray(a)]


def run_case(name, factory, seed, rays, ray_begin, grid):
    w = make_workload(factory)
    t0 = time.time()
    h, st = O.trace(w, rays=rays, ray_begin=ray_begin, seed=seed, threads=0, grid_domain=grid)
    dt = time.time() - t0
    p = oracle_parameters(h["energy"], w)
    agg = aggregate_parameters(h["energy"], w)
    rec = {"case": name, "workload": factory, "seed": seed, "rays": rays, "ray_begin": ray_begin, "grid_domain": grid,
           "band_energy": _json_num(h["energy"].sum(axis=2)),
           "segments": int(st["segments"]), "octave_rays": int(st["octave_rays"]),
           "detections": int(st["detections"]), "oracle_seconds": round(dt, 2)}
    for k, v in p.items():
        rec[k] = _json_num(v)
        rec["agg_" + k] = _json_num(agg[k][None])[0]
    print(f"{name} {factory} seed {seed}: {rays} primaries, {st['segments']} segments, {dt:.1f} s", flush=True)
    return rec


def main(argv):
    want = argv or list(cases())
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    for name in want:
        data[name] = [run_case(name, *c) for c in cases()[name]]
        with open(OUT, "w") as f:
            json.dump(data, f, separators=(",", ":"))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
