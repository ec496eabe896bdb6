"""Learned vs uniform emission: wall time until T30 / EDT / C80 / D50 reach one just-noticeable
difference, on seeded rooms drawn like the 10 x 8 x 4 m shoebox (rooms.proposal_room_c4).

Protocol (``python -m pachydermacoustic_universal_gb300.proposal_study``):

1. Training data: ``train_rooms`` rooms, each traced with uniform emission and capture on
   (``train_rays`` primaries, ``train_receivers`` receivers per room); one target per receiver
   (proposal.capture_targets_l2 from per-primary capture, or proposal.capture_targets).  A tenth of the rooms is held back for the validation loss.
2. Training: full-batch Adam on the GPU (pach_mlp_train, a captured CUDA graph per step).
3. Evaluation on ``eval_rooms`` further rooms: ``seeds`` independent runs of ``eval_rays`` primaries
   with uniform emission (source kind 2) and with the learned proposal (each mixture weight of
   uniform emission in ``mixes``).  Both estimators are unbiased, so the expected squared error of a parameter at N rays
   is its variance, sigma_N^2 = sigma^2 / N: the rays to reach one JND are N_JND = N (sigma_N / JND)^2
   (relative sigma for T30 and EDT), and the wall time is N_JND times the measured device time per
   primary of that method.  A room's time for "T30 and C80 within 1 JND" is the largest over both
   parameters, every receiver and every band.
4. Bias check: the learned mean of every parameter against the uniform mean, in units of the
   combined standard error.

JNDs (ISO 3382-1 Annex A): T30 and EDT 5 % relative, C80 1 dB, D50 0.05 (5 points of the %).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import proposal, rooms, tracer
from .simulation import room_parameters

JND = {"T30": 0.05, "EDT": 0.05, "C80": 1.0, "D50": 5.0}
RELATIVE = {"T30": True, "EDT": True, "C80": False, "D50": False}


def uniform_sources(w):
    w.sources = [rooms.SourceSpec(s.origin, s.power_db, 2) for s in w.sources]
    return w


def direct_times(w):
    c = 331.0 + 0.6 * w.scene.temp_c
    return [min(np.linalg.norm(np.subtract(r.origin, s.origin)) for s in w.sources) / c for r in w.receivers]


def parameters(E, w, fs=1000):
    """T30/EDT/C80/D50 [R][8] of raw energy histograms E [R][8][T]."""
    direct = direct_times(w)
    out = {k: np.full(E.shape[:2], np.nan) for k in JND}
    for r in range(E.shape[0]):
        for o in range(E.shape[1]):
            p = room_parameters(E[r, o], fs, direct[r])
            for k in JND:
                out[k][r, o] = p[k]
    return out


def runs(w, ds, n_rays, seeds, seed0, raw=None, mix=0.3):
    """Parameters of independent runs, [seeds][R][8] per name, and device ms per primary."""
    acc = {k: [] for k in JND}
    dev_ms = 0.0
    for s in range(seeds):
        if raw is None:
            h, st = tracer.trace(w, dscene=ds, rays=n_rays, seed=seed0 + s)
        else:
            h, st = proposal.trace_learned(w, raw, mix=mix, dscene=ds, rays=n_rays, seed=seed0 + s)
        dev_ms += st["device_ms"]
        p = parameters(h["energy"], w)
        for k in JND:
            acc[k].append(p[k])
    return {k: np.asarray(v) for k, v in acc.items()}, dev_ms / (seeds * n_rays)


def rays_to_jnd(P, n_rays):
    """Per parameter: rays to one JND for every receiver and band (max over them), from the seed spread."""
    out = {}
    for k, v in P.items():
        ok = np.all(np.isfinite(v), axis=0)
        if not ok.any():
            out[k] = float("nan")
            continue
        sd = v.std(axis=0, ddof=1)
        if RELATIVE[k]:
            sd = sd / np.abs(v.mean(axis=0))
        n = n_rays * (sd / JND[k]) ** 2
        out[k] = float(np.max(n[ok]))
    return out


def bias_z(Pu, Pl):
    """Largest |mean difference| / combined standard error over receivers and bands, per parameter."""
    z = {}
    for k in JND:
        a, b = Pu[k], Pl[k]
        ok = np.all(np.isfinite(a), axis=0) & np.all(np.isfinite(b), axis=0)
        if not ok.any():
            z[k] = float("nan")
            continue
        se = np.sqrt(a.var(axis=0, ddof=1) / a.shape[0] + b.var(axis=0, ddof=1) / b.shape[0])
        d = np.abs(a.mean(axis=0) - b.mean(axis=0)) / np.maximum(se, 1e-30)
        z[k] = float(np.max(d[ok]))
    return z


def study(train_rooms=200, train_rays=100_000, eval_rooms=50, eval_rays=10_000, seeds=8, steps=3000, lr=1e-3,
          mixes=(0.3,), seed=7, train_receivers=12, target="linear", log=print):
    t0 = time.perf_counter()
    rooms_train = [rooms.proposal_room_c4(1000 + i, n_receivers=train_receivers) for i in range(train_rooms)]
    cond, tgt, t_collect = proposal.collect(rooms_train, train_rays, seed=seed, target=target)
    n_val = max(1, train_rooms // 10) * train_receivers
    net = proposal.ProposalNet(seed=seed, max_rows=max(cond.shape[0], 128))
    net.set_data(cond[n_val:], tgt[n_val:])
    t1 = time.perf_counter()
    curve = np.concatenate([net.train(steps // 2, lr=lr), net.train(steps - steps // 2, lr=lr * 0.3)])
    train_loss = float(curve[-1])
    t_train = time.perf_counter() - t1
    net.set_data(cond[:n_val], tgt[:n_val])
    val_loss, _ = net.loss_grad(with_grad=False)
    # entropy of the targets: the loss a perfect fit reaches (bin-centre rule, up to the bin solid angles)
    _, om = proposal.direction_bins()
    tv = tgt[:n_val].astype(np.float64)
    ent = float(-np.mean(np.sum(np.where(tv > 0, tv * np.log(np.maximum(tv, 1e-30) / om), 0.0), axis=1)))
    uni = float(math.log(4 * math.pi))
    log(f"collect {t_collect:.1f} s ({train_rooms} rooms x {train_rays} rays), train {t_train:.1f} s "
        f"({steps} steps): train loss {train_loss:.3f}, validation loss {val_loss:.3f}, "
        f"uniform {uni:.3f}, target entropy {ent:.3f}")

    per_room = []
    for i in range(eval_rooms):
        w = uniform_sources(rooms.proposal_room_c4(5000 + i))
        ds = tracer.DeviceScene(w.scene)
        raw = net.forward(proposal.conditions(w))
        Pu, ms_u = runs(w, ds, eval_rays, seeds, 10_000 * (i + 1))
        nu = rays_to_jnd(Pu, eval_rays)
        rec = {"room": w.name, "ms_per_ray": {"uniform": ms_u}, "rays_to_jnd": {"uniform": nu}, "bias_z": {},
               "ms_to_jnd": {}}
        for mix in mixes:
            Pl, ms_l = runs(w, ds, eval_rays, seeds, 10_000 * (i + 1) + 5000, raw=raw, mix=mix)
            nl = rays_to_jnd(Pl, eval_rays)
            tag = f"learned_{mix:g}"
            rec["ms_per_ray"][tag] = ms_l
            rec["rays_to_jnd"][tag] = nl
            rec["bias_z"][tag] = bias_z(Pu, Pl)
            for name, keys in (("T30_C80", ("T30", "C80")), ("all", tuple(JND))):
                rec["ms_to_jnd"].setdefault(name, {})["uniform"] = max(nu[k] for k in keys) * ms_u
                rec["ms_to_jnd"][name][tag] = max(nl[k] for k in keys) * ms_l
        ds.close()
        per_room.append(rec)
        log(json.dumps({"room": w.name, "rays_to_jnd": rec["rays_to_jnd"], "bias_z": rec["bias_z"],
                        "ms_to_jnd": rec["ms_to_jnd"]}))

    def gmean(x):
        x = np.asarray([v for v in x if np.isfinite(v) and v > 0])
        return float(np.exp(np.mean(np.log(x)))) if x.size else float("nan")

    summary = {"target": target, "train_rooms": train_rooms, "train_receivers": train_receivers,
               "train_rays": train_rays,
               "eval_rooms": eval_rooms, "eval_rays": eval_rays, "seeds": seeds, "steps": steps, "mixes": list(mixes),
               "collect_s": t_collect, "train_s": t_train, "train_loss": train_loss, "val_loss": val_loss,
               "uniform_loss": uni, "target_entropy": ent}
    extra = 1000.0 * (t_collect + t_train) / max(1, eval_rooms)  # one-off cost spread over the evaluated rooms
    for mix in mixes:
        tag = f"learned_{mix:g}"
        res = {}
        for k in JND:
            res[f"speedup_rays_{k}"] = gmean([r["rays_to_jnd"]["uniform"][k] / r["rays_to_jnd"][tag][k]
                                              for r in per_room])
        for name in ("T30_C80", "all"):
            tu = [r["ms_to_jnd"][name]["uniform"] for r in per_room]
            tl = [r["ms_to_jnd"][name][tag] for r in per_room]
            res[f"wall_ms_to_jnd_{name}"] = {"uniform": gmean(tu), "learned": gmean(tl),
                                             "speedup": gmean([a / b for a, b in zip(tu, tl)]),
                                             "learned_incl_training": gmean(tl) + extra}
        res["max_bias_z"] = {k: float(np.nanmax([r["bias_z"][tag][k] for r in per_room])) for k in JND}
        summary[tag] = res
    summary["wall_s"] = time.perf_counter() - t0
    return summary


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train-rooms", type=int, default=200)
    ap.add_argument("--train-rays", type=int, default=100_000)
    ap.add_argument("--eval-rooms", type=int, default=50)
    ap.add_argument("--eval-rays", type=int, default=10_000)
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--mix", type=float, nargs="+", default=[0.3])
    ap.add_argument("--train-receivers", type=int, default=12)
    ap.add_argument("--target", default="linear", choices=["linear", "l2"])
    a = ap.parse_args()
    s = study(a.train_rooms, a.train_rays, a.eval_rooms, a.eval_rays, a.seeds, a.steps, a.lr, tuple(a.mix),
              train_receivers=a.train_receivers, target=a.target)
    print(json.dumps(s))


if __name__ == "__main__":
    main()
