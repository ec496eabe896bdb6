"""FP64 restatement of the split ray tracer's convergence mode (SplitRayTracer with rayCount < 1).

TEST INFRASTRUCTURE ONLY: the checker of the GPU engine's convergence mode; the product never
imports it.  Paths are relative to Pachyderm_Acoustic_Universal/; "TaskAll" is
"Classes_Complete_Trace - TaskAll.cs".

* Receivers (TaskAll:111-176, Check_Validity 178-200): from the source's Origin (a SourceCluster's is
  the mean of its members', Classes_Sources.cs:684-689) one ray towards each receiver; visible when
  nothing is hit before the receiver.  Check 0 watches the farthest visible receiver, check 1 the
  farthest hidden one.
* Revolutions (Calculate_Conv, TaskAll:286-326): Revolution_Period() primaries (80 per point source,
  the members' sum for a cluster, Classes_Sources.cs:197-200, 687) are traced, then every non-null
  check's Check() runs (all of them, C# `&=`); the run stops after the first revolution where all agree.
* SpecMin_Convergence_Check (rayCount == 0, TaskAll:806-921) and Minimum_Convergence_Check
  (rayCount < 0, TaskAll:1015-1107) on the raw energy histogram of band h_oct and its
  Reflection_Analysis_Data, with AcousticalMath.Envelope / SlidingMax (Classes_Math.cs:327-388) and
  SPL_Intensity (97-102) as written, including SlidingMax's ring-buffer overwrite and SpecMin's
  integer-division n = 343 spec_cross / T.
Parity with the reference itself is unpinned (see pach_oracle.h).
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O


def spl_intensity(x):
    with np.errstate(divide="ignore"):
        spl = 10.0 * np.log10(np.asarray(x, dtype=np.float64) / 1e-12)
    return np.where(spl < 0, 0.0, spl)


def sliding_max(x, window):
    """SlidingMax as written: deque indices in a ring of `window` slots, push before the stale head
    is dropped."""
    n = len(x)
    out = np.zeros(n)
    dq = [0] * window
    head, tail = 0, -1
    for i in range(n):
        while tail >= head and x[i] >= x[dq[tail % window]]:
            tail -= 1
        tail += 1
        dq[tail % window] = i
        if dq[head % window] < i - window + 1:
            head += 1
        out[i] = x[dq[head % window]]
    return out


def envelope(x, fs, attack, release, window_s=0.02):
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return x
    w = max(1, int(round(window_s * fs)))
    lm = sliding_max(x, w)
    a = 1.0 - math.exp(-1.0 / (attack * fs))
    r = 1.0 - math.exp(-1.0 / (release * fs))
    y = np.zeros_like(x)
    prev = x[0]
    y[0] = min(prev, lm[0])
    for i in range(1, x.size):
        c = a if x[i] > prev else r
        yn = min(prev + c * (x[i] - prev), lm[i])
        y[i] = yn
        prev = yn
    return y


class MinimumCheck:
    """Minimum_Convergence_Check: energy before 50 ms, before 80 ms and after 80 ms of the direct
    arrival stable to 2 %, 2 %, 10 % for six revolutions in a row."""

    def __init__(self, distance, c, fs, T):
        self.start = int(math.floor(distance / c * fs))
        self.s50 = int(math.floor(50.0 * fs / 1000)) + self.start
        self.s80 = int(math.floor(80.0 * fs / 1000)) + self.start
        self.inf = T
        self.snap = (0.0, 0.0, 0.0)
        self.count = 0
        self.nmin = 0

    def check(self, E, A):
        sn50 = float(np.sum(E[self.start:self.s50]))
        sn80 = sn50 + float(np.sum(E[self.s50:self.s80]))
        sninf = float(np.sum(E[self.s80:self.inf]))
        with np.errstate(divide="ignore", invalid="ignore"):
            c1 = abs(sn50 - self.snap[0]) / np.float64(self.snap[0])
            c2 = abs(sn80 - self.snap[1]) / np.float64(self.snap[1])
            ci = abs(sninf - self.snap[2]) / np.float64(self.snap[2])
        if sn50 == 0 or c1 > 0.02 or sn80 == 0 or c2 > 0.02 or sninf == 0 or ci > 0.1:
            self.count = 0
        else:
            self.count += 1
        self.snap = (sn50, sn80, sninf)
        return self.count > 5


class SpecMinCheck:
    """SpecMin_Convergence_Check: 50 ms block energies stable to 10 % (up to the last block with
    specular energy) for more than ten revolutions, and at least Nmin rays counted as 80 per revolution."""

    def __init__(self, fs, T):
        self.fs = fs
        self.step = fs // 20
        self.binct = T // self.step
        self.T = T
        self.snapshot = np.zeros(self.binct)
        self.rayct = 0
        self.count = 0
        self.nmin = 0

    def check(self, E, A):
        self.rayct += 80
        n_used = self.binct * self.step
        sn = E[:n_used].reshape(self.binct, self.step).sum(axis=1)
        sn_spec = A[0][:n_used].reshape(self.binct, self.step).sum(axis=1)
        sn_diff = A[1][:n_used].reshape(self.binct, self.step).sum(axis=1)
        si_spec = spl_intensity(envelope(A[0], self.fs, 0.001, 0.01)) - 110
        si_comb = spl_intensity(envelope(A[1], self.fs, 0.001, 0.01) + envelope(A[2], self.fs, 0.001, 0.01)) - 110
        conv = 0.0
        if self.binct > 0:
            lim = sn_diff[0] * 1e-6
            stop = self.binct - 1
            while stop >= 0 and sn_spec[stop] < lim and stop != 1:
                stop -= 1
            for i in range(self.binct):
                if sn[i] == 0 or self.snapshot[i] == 0:
                    continue
                if i < stop:
                    conv = max(conv, abs(sn[i] - self.snapshot[i]) / self.snapshot[i])
        spec_cross = 0
        for i in range(self.T - 1, 0, -1):
            spec_cross = i
            if si_spec[i] > si_comb[i] + 4:
                break
        n = float((343 * spec_cross) // self.T)
        self.nmin = max(5000, int(math.ceil(4 * n * n)))
        self.snapshot = sn
        if conv == 0:
            return False
        if conv > 0.1:
            self.count = 0
        self.count += 1
        return self.count > 10 and self.rayct > self.nmin


def make_check(mode, distance, c, fs, T):
    return SpecMinCheck(fs, T) if mode == 0 else MinimumCheck(distance, c, fs, T)


def pick_receivers(workload, grid_domain=7):
    """(rows, distances) of the two checks: the farthest receiver the source's Origin sees, the farthest
    it does not (row -1: none)."""
    ctr = np.mean([np.asarray(s.origin, float) for s in workload.sources], axis=0)
    best = [(-1, 0.0), (-1, 0.0)]
    for i, r in enumerate(workload.receivers):
        d = np.asarray(r.origin, float) - ctr
        dist = float(np.linalg.norm(d))
        if not dist > 0:
            continue
        poly, t, _ = O.shoot(workload.scene, ctr, d / dist, grid_domain=grid_domain)
        valid = poly < 0 or t >= dist
        k = 0 if valid else 1
        if best[k][1] < dist:
            best[k] = (i, dist)
    return [b[0] for b in best], [b[1] for b in best]


def replay(per_rev, mode, distance, c, fs):
    """First revolution (1-based) after which one check agrees, over per-revolution contributions
    per_rev [revs][4][T] (energy, analysis 0..2); 0 if none.  Returns (stop, check)."""
    T = per_rev.shape[2]
    chk = make_check(mode, distance, c, fs, T)
    E, A = np.zeros(T), np.zeros((3, T))
    for r in range(per_rev.shape[0]):
        E += per_rev[r, 0]
        A += per_rev[r, 1:]
        if chk.check(E, A):
            return r + 1, chk
    return 0, chk


def converge(workload, *, seed, mode, max_rays=1 << 24, grid_domain=7, threads=0, ray_begin=0):
    """Convergence mode on the FP64 oracle: returns (raw histograms, stats with revolutions, converged,
    check_receivers)."""
    _, st0 = O.trace(workload, rays=1, seed=seed, threads=1, grid_domain=grid_domain)
    h_oct, c, fs = st0["h_oct"], st0["sound_speed"], workload.sample_rate
    T = int(workload.sample_rate * workload.cutoff_s)
    rows, dist = pick_receivers(workload, grid_domain)
    checks = [make_check(mode, dist[k], c, fs, T) if rows[k] >= 0 else None for k in range(2)]
    period = 80 * len(workload.sources)
    tot = None
    stats = {}
    done, revs, converged = 0, 0, False
    while done < max_rays:
        h, st = O.trace(workload, rays=period, ray_begin=ray_begin + done, seed=seed, threads=threads,
                        grid_domain=grid_domain)
        if tot is None:
            tot = {k: v.copy() for k, v in h.items()}
        else:
            for k in tot:
                tot[k] += h[k]
        for k, v in st.items():
            if isinstance(v, (int, float)) and k not in ("h_oct", "bins", "cotime_s", "sound_speed", "rho_c"):
                stats[k] = stats.get(k, 0) + v
        done += period
        revs += 1
        agree = True
        for k in range(2):
            if checks[k] is None:
                continue
            r = rows[k]
            agree = checks[k].check(tot["energy"][r, h_oct], tot["analysis"][r, :, h_oct]) and agree
        if agree:
            converged = True
            break
    stats.update(revolutions=revs, converged=converged, check_receivers=rows, h_oct=h_oct, primaries=done)
    return tot, stats
