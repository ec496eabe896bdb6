"""Generates the committed fixtures in tests/golden/ (run: python tests/golden/make_golden.py).

The reference ships no tests, fixtures or golden vectors for this path and cannot run here (C#,
unvendored Hare geometry library), so the fixtures are analytic known answers, each produced by an
implementation that shares no code with the oracle or the engine:

* philox_kat.json      -- Philox4x32-10 known-answer vectors published with the Random123 library
                          (Salmon et al., SC'11), the counter generator both sides draw from.
* iso9613.json         -- Calculate_Attenuation as coded (Classes_Medium_Props.cs:75-88, C# integer
                          divisions in the exponents kept), restated here in plain Python, plus the
                          Uniform_Medium density and sound speed, at several air states.
* shoebox_paths.json   -- pure-specular paths in an axis-aligned shoebox by per-axis unfolding
                          (the image-lattice construction): wall hit, leg length, hit point.
* decay_params.json    -- ideal exponential energy decays with known reverberation time T; the
                          Schroeder/T30/EDT/C80/D50 values follow in closed form.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def philox_kat():
    # (counter, key, expected output) -- Random123 kat_vectors for philox4x32_10
    return [
        {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
        {"ctr": [0xffffffff] * 4, "key": [0xffffffff] * 2, "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
        {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
         "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]},
    ]


def iso9613_as_coded(temp_c, hr, pa_hpa):
    F = [62.5, 125, 250, 500, 1000, 2000, 4000, 8000]
    Tk = temp_c + 273.15
    Pa = pa_hpa / 10.0                       # Uniform_Medium passes Pa/10 (hPa -> kPa)
    h = hr * 10 ** (-6.8346 * (273.16 / Tk) ** 1.261 + 4.6151) / (Pa / 101.325)
    out = []
    for f in F:
        frO = (Pa / 101.325) * (24 + 4.04e4 * h * ((0.02 + h) / (0.391 + h)))
        frN = (Pa / 101.325) * (Tk / 293.15) ** 0 * (9 + 280 * h * math.exp(-4.170 * ((Tk / 293.15) ** 0 - 1)))
        z = 0.1068 * math.exp(-3352 / Tk) / (frN + f * f / frN)
        y = (Tk / 293.15) ** (-2) * (0.01275 * math.exp(-2239.1 / Tk) / (frO + f * f / frO) + z)
        out.append(8.686 * f * f * ((1.84e-11 / (Pa / 101.325) * (Tk / 293.15) ** 0) + y))
    P = pa_hpa * 100
    T = temp_c
    Pv = hr * 6.1078 * 10 ** ((7.5 * T) / (237.3 + T))
    rho = (P / (287.05 * Tk)) * (1 - 0.378 * Pv / P)
    return out, 331 + 0.6 * temp_c, rho


def shoebox_paths(L=(10.0, 8.0, 4.0), n=24, bounces=40, seed=11):
    rng = np.random.default_rng(seed)
    rays = []
    for _ in range(n):
        p = np.array([rng.uniform(0.5, L[0] - 0.5), rng.uniform(0.5, L[1] - 0.5), rng.uniform(0.5, L[2] - 0.5)])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        o0, d0 = p.copy(), d.copy()
        walls, legs, pts = [], [], []
        for _ in range(bounces):
            ts = [((L[a] - p[a]) / d[a]) if d[a] > 0 else (-p[a] / d[a]) if d[a] < 0 else math.inf for a in range(3)]
            a = int(np.argmin(ts))
            t = ts[a]
            p = p + d * t
            side = 1 if d[a] > 0 else 0
            walls.append([a, side])
            legs.append(t)
            pts.append(p.tolist())
            d[a] = -d[a]
        rays.append({"origin": o0.tolist(), "dir": d0.tolist(), "walls": walls, "legs": legs, "points": pts})
    return {"size": list(L), "rays": rays}


def decay_params():
    """E(t) = exp(-k t) on 1 ms bins with k = 6 ln(10) / T: the Schroeder curve falls 60 dB in T
    seconds, so T30 = EDT = T up to the truncation of the geometric tail (< 1e-4 relative here).
    C80 and D50 with the direct sound at t = 0: geometric sums over the 80 / 50 ms early bins."""
    out = []
    for T in (0.5, 1.0, 1.7, 2.4):
        fs, n = 1000, 3000
        k = 6.0 * math.log(10) / T
        r = math.exp(-k / fs)
        total = (1 - r ** n) / (1 - r)
        early80 = (1 - r ** 80) / (1 - r)
        early50 = (1 - r ** 50) / (1 - r)
        out.append({"T": T, "fs": fs, "rate": k, "n": n, "T30": T, "EDT": T,
                    "C80": 10 * math.log10(early80 / (total - early80)), "D50": 100 * early50 / total})
    return out


def main():
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(philox_kat(), f, indent=1)
    states = [(20.0, 50.0, 1013.25), (20.0, 30.0, 1013.25), (20.0, 80.0, 1013.25), (10.0, 50.0, 1013.25),
              (30.0, 60.0, 1000.0), (0.0, 70.0, 1013.25)]
    iso = []
    for (t, hr, pa) in states:
        att, c, rho = iso9613_as_coded(t, hr, pa)
        iso.append({"temp_c": t, "hr": hr, "pa_hpa": pa, "atten_db_per_m": att, "c": c, "rho": rho})
    with open(os.path.join(HERE, "iso9613.json"), "w") as f:
        json.dump(iso, f, indent=1)
    with open(os.path.join(HERE, "shoebox_paths.json"), "w") as f:
        json.dump(shoebox_paths(), f)
    with open(os.path.join(HERE, "decay_params.json"), "w") as f:
        json.dump(decay_params(), f, indent=1)


if __name__ == "__main__":
    main()
