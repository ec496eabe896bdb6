"""Generates tests/golden/convergence.json: where the FP64 oracle's convergence mode stops
(oracle/convergence.py, the restatement of SplitRayTracer with rayCount < 1, TaskAll:111-176, 300-330,
783-1107), the reference side of tests/test_gpu_convergence.py.

Case: the 10 x 8 x 4 m shoebox (12 triangles, 3 receivers) with a 1 s cutoff, seed 17, both checks
(rayCount 0: SpecMin_Convergence_Check, rayCount -1: Minimum_Convergence_Check).  Kept per mode: the
revolutions traced, whether the checks agreed, the checks' receivers, and the band energy totals
[R][8] of the raw histograms the run ends with.

Run:  python tests/golden/make_convergence.py   (8 cores: ~2.5 min)
Test infrastructure: imports the oracle as the checker.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import convergence as OC  # noqa: E402
from pachydermacoustic_universal_gb300 import rooms  # noqa: E402

OUT = os.path.join(HERE, "convergence.json")


def workload():
    w = rooms.shoebox_c1()
    w.cutoff_s = 1.0
    return w


def main():
    out = {"workload": "shoebox_c1, cutoff 1.0 s", "seed": 17, "cases": []}
    for ray_count in (0, -1):
        h, st = OC.converge(workload(), seed=17, mode=0 if ray_count == 0 else 1, max_rays=40000)
        out["cases"].append({"ray_count": ray_count, "revolutions": st["revolutions"], "converged": st["converged"],
                             "check_receivers": st["check_receivers"], "primaries": st["primaries"],
                             "segments": int(st["segments"]),
                             "band_energy": h["energy"].sum(axis=2).tolist()})
        print(ray_count, st["revolutions"], st["converged"], st["check_receivers"], flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
