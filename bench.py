"""Benchmark: segment-bounces/s of the split ray tracer.

Default workload (one GPU): the 120 x 90 x 35 m arena (~500k triangles: jittered shell, tiered
seating facets, 2000 diffuser panels), 4 sources, 64 receivers of radius 0.5 m, 3.5 s cutoff, 1 ms
bins, 10M primary rays -- the largest single-GPU configuration.  The timed steps together trace the
10M-ray job: each step traces its own 10M / steps primaries (ray_begin = step * batch); the warm-up
and kernel-timing steps trace primaries after them.
--workload hall: the 40 x 25 x 15 m jittered hall (~20k triangles, 2 sources, 16 receivers, 1M rays);
shoebox: the 12-triangle 10 x 8 x 4 m shoebox (100k rays); hall_map: the hall with a 608-receiver
audience map (1 m squares at 1.5 m, the reference's grid walks); batched: the 64-room batch (each
room's ray count x --ray-scale per step) as one batch run with autotuned knobs.

Metric: segment-bounces/s = shoot calls (broadband + octave rays, hit or miss) per second.
  value  -- device time of the engine's device loop (one CUDA-graph launch per step, the product
            default; CUDA events on the engine's stream), scene resident, summed over the steps.
  e2e    -- the same job through the public C ABI from host buffers: the scene built from host arrays
            and uploaded once per job, then every step's trace and its histograms downloaded into
            pinned host buffers.
  roofline -- per-kernel CUDA-event times from a separate kernel-timing pass over the same workload.
  filters -- the receivers' filters (7 per receiver, FP64 FFT convolution on the GPU) of the last
            end-to-end step's histograms: device time, end to end through the host-array call, and the
            FP64 oracle per filter on one host core (--metric filters prints this as its own line).
  jnd    -- (arena line) the metric's second half at a compact size: wall time to T30/C80 within 1 JND,
            learned emission proposal against uniform emission (--metric jnd runs the larger study).
The reference arm (--impl reference) times the CPU FP64 restatement of the reference algorithm
(voxel grid of 7 cells per axis as Pach_Properties defaults) on all host cores: the reference's own
C# engine cannot run on this machine (no .NET runtime, unvendored geometry library).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "ray-bounces/s (segment-bounces/s, 1 GB300)"
UNIT = "segments/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks + throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            os.unlink(self.path)
        except Exception:
            return out
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) < 9:
                continue
            for i, n in enumerate(names):
                if r[5 + i].strip().lower() == "active":
                    reasons.add(n)
        out["sm_mhz"] = statistics.median(sm) if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
        return dist
    return None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x, device=None):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x, device=None):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def map_of(w, oracle_side=False):
    """The workload's mapping receivers, for the engine (tracer.MapReceivers) or the oracle."""
    m = w.extra.get("map")
    if m is None:
        return None
    if oracle_side:
        import types
        return types.SimpleNamespace(time_1pt=False, directional=False, **m)
    from pachydermacoustic_universal_gb300 import tracer
    return tracer.MapReceivers(**m)


def reference_work(ws, sample_rays, seed):
    """k_cell, k_tri: mean voxel cells stepped and polygon tests per segment of the reference
    traversal (grid domain 7) on a sample of the same rays (shared among the rooms ws)."""
    from oracle import oracle as O
    t0 = time.time()
    tot = {}
    per = max(1, sample_rays // len(ws))
    for w in ws:
        _, st = O.trace(w, rays=per, seed=seed, threads=0, grid_domain=7, map_receivers=map_of(w, True))
        for k, v in st.items():
            if isinstance(v, (int, float)):
                tot[k] = tot.get(k, 0) + v
    dt = time.time() - t0
    return tot, dt


def cpu_baseline(ws, sample_rays, seed):
    st, dt = reference_work(ws, sample_rays, seed)
    cores = os.cpu_count() or 1
    return {"value": st["segments"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sample_rays} primaries of the workload ({len(ws)} room(s), {int(st['segments'])} segments, "
                      f"{dt:.1f} s), FP64 restatement, voxel grid domain 7, {cores} threads"}, st


def workload(name, ray_scale):
    """The rooms of a bench workload: the 500k-triangle arena (default), the irregular hall, the
    12-triangle shoebox, the hall with an audience map, or the 64-room batch (ray counts scaled by
    ray_scale)."""
    from pachydermacoustic_universal_gb300 import rooms
    if name == "hall":
        return [rooms.irregular_hall_c2()]
    if name == "shoebox":
        return [rooms.shoebox_c1()]
    if name == "arena":
        return [rooms.arena_c5()]
    if name == "hall_map":
        w = rooms.irregular_hall_c2()
        w.extra["map"] = dict(origins=rooms.audience_plane((4.0, 3.0), (36.0, 22.0), 1.0, 1.0), increment=1.0,
                              cutoff_ms=3000.0, walk=0)
        return [w]
    ws = rooms.batched_rooms_c3()
    for w in ws:
        w.rays = max(100, int(round(w.rays * ray_scale)))
    return ws


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    rooms_ = workload(args.workload, args.ray_scale)[:4]
    sample = args.ref_sample
    per = max(1, sample // len(rooms_))
    tot_seg, tot_t = 0, 0.0
    for step in range(args.warmup + args.steps):
        t0 = time.time()
        seg = 0
        for w in rooms_:
            _, st = O.trace(w, rays=per, ray_begin=step * per, seed=args.seed, threads=0, grid_domain=7,
                            map_receivers=map_of(w, True))
            seg += st["segments"]
        dt = time.time() - t0
        if step >= args.warmup:
            tot_seg += seg
            tot_t += dt
    val = tot_seg / tot_t
    cores = os.cpu_count() or 1
    w = rooms_[0]
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded room generator)",
            "impl": "reference",
            "config": {"workload": w.name if len(rooms_) == 1 else f"batched (first {len(rooms_)} rooms)",
                       "rays_per_step": per * len(rooms_), "cutoff_s": w.cutoff_s,
                       "sources": len(w.sources), "receivers": len(w.receivers), "triangles": w.scene.n_triangles},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per * len(rooms_)} primaries per step, FP64 restatement of the reference "
                                       f"algorithm (voxel grid domain 7), {cores} threads; the C# reference "
                                       f"cannot run here (no .NET runtime, Hare unvendored)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------
# --metric jnd: wall time until T30 and C80 reach one JND, learned emission proposal vs uniform
# ------------------------------------------------------------------------------------------
JND = {"T30": 0.05, "EDT": 0.05, "C80": 1.0, "D50": 5.0}   # ISO 3382-1 Annex A; T30/EDT relative
JND_RELATIVE = {"T30": True, "EDT": True, "C80": False, "D50": False}


def _uniform_sources(w):
    from pachydermacoustic_universal_gb300 import rooms
    w.sources = [rooms.SourceSpec(s.origin, s.power_db, 2) for s in w.sources]
    return w


def _direct_times(w):
    c = 331.0 + 0.6 * w.scene.temp_c
    return [min(np.linalg.norm(np.subtract(r.origin, s.origin)) for s in w.sources) / c for r in w.receivers]


def jnd_parameters(E, w, fs=1000):
    """T30/EDT/C80/D50 [R][8] of raw energy histograms E [R][8][T] (AcousticalMath)."""
    from pachydermacoustic_universal_gb300.simulation import room_parameters
    direct = _direct_times(w)
    out = {k: np.full(E.shape[:2], np.nan) for k in JND}
    for r in range(E.shape[0]):
        for o in range(E.shape[1]):
            p = room_parameters(E[r, o], fs, direct[r])
            for k in JND:
                out[k][r, o] = p[k]
    return out


def jnd_runs(w, ds, n_rays, seeds, seed0, raw=None, mix=0.3):
    """Parameters of independent runs, [seeds][R][8] per name, and device ms per primary."""
    from pachydermacoustic_universal_gb300 import proposal, tracer
    acc = {k: [] for k in JND}
    dev_ms = 0.0
    for s in range(seeds):
        if raw is None:
            h, st = tracer.trace(w, dscene=ds, rays=n_rays, seed=seed0 + s)
        else:
            h, st = proposal.trace_learned(w, raw, mix=mix, dscene=ds, rays=n_rays, seed=seed0 + s)
        dev_ms += st["device_ms"]
        p = jnd_parameters(h["energy"], w)
        for k in JND:
            acc[k].append(p[k])
    return {k: np.asarray(v) for k, v in acc.items()}, dev_ms / (seeds * n_rays)


def rays_to_jnd(P, n_rays):
    """Per parameter: primaries until its standard error is one JND, for every receiver and band (the
    largest over them).  Both estimators are unbiased, so the expected squared error at N rays is the
    variance sigma^2 / N, estimated from the seed spread of runs of n_rays."""
    out = {}
    for k, v in P.items():
        ok = np.all(np.isfinite(v), axis=0)
        if not ok.any():
            out[k] = float("nan")
            continue
        sd = v.std(axis=0, ddof=1)
        if JND_RELATIVE[k]:
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


def _gmean(x):
    x = np.asarray([v for v in x if np.isfinite(v) and v > 0])
    return float(np.exp(np.mean(np.log(x)))) if x.size else float("nan")


def jnd_study(train_rooms, train_rays, eval_rooms, eval_rays, seeds, steps, lr=1e-3, mix=0.3, seed=7,
              train_receivers=12, target="linear"):
    """Learned vs uniform emission on seeded rooms drawn like the 10 x 8 x 4 m shoebox
    (rooms.proposal_room_c4).

    1. Training data: train_rooms rooms traced with uniform emission and capture on (train_rays
       primaries, train_receivers receivers each), one target distribution per receiver; a tenth of
       the rooms is held back for the validation loss.
    2. Training: full-batch Adam on the GPU (pach_mlp_train, the library's tcgen05 kernels).
    3. Evaluation on eval_rooms further rooms: `seeds` runs of eval_rays primaries each with uniform
       emission and with the learned proposal (defensive mixture, uniform weight `mix`); rays to one
       JND from the seed spread (rays_to_jnd), times the measured device ms per primary of each method.
       A room's time for "T30 and C80 within 1 JND" is the largest over both parameters, every
       receiver and band.
    4. Bias check: learned mean against uniform mean per parameter, in combined standard errors."""
    from pachydermacoustic_universal_gb300 import proposal, rooms, tracer
    t0 = time.perf_counter()
    rooms_train = [rooms.proposal_room_c4(1000 + i, n_receivers=train_receivers) for i in range(train_rooms)]
    cond, tgt, t_collect = proposal.collect(rooms_train, train_rays, seed=seed, target=target)
    n_val = max(1, train_rooms // 10) * train_receivers
    net = proposal.ProposalNet(seed=seed, max_rows=max(cond.shape[0], 128))
    net.set_data(cond[n_val:], tgt[n_val:])
    t1 = time.perf_counter()
    curve = np.concatenate([net.train(steps // 2, lr=lr), net.train(steps - steps // 2, lr=lr * 0.3)])
    t_train = time.perf_counter() - t1
    net.set_data(cond[:n_val], tgt[:n_val])
    val_loss, _ = net.loss_grad(with_grad=False)
    per_room = []
    for i in range(eval_rooms):
        w = _uniform_sources(rooms.proposal_room_c4(5000 + i))
        ds = tracer.DeviceScene(w.scene)
        raw = net.forward(proposal.conditions(w))
        Pu, ms_u = jnd_runs(w, ds, eval_rays, seeds, 10_000 * (i + 1))
        Pl, ms_l = jnd_runs(w, ds, eval_rays, seeds, 10_000 * (i + 1) + 5000, raw=raw, mix=mix)
        nu, nl = rays_to_jnd(Pu, eval_rays), rays_to_jnd(Pl, eval_rays)
        rec = {"rays_to_jnd": {"uniform": nu, "learned": nl}, "bias_z": bias_z(Pu, Pl), "ms_to_jnd": {}}
        for name, keys in (("T30_C80", ("T30", "C80")), ("all", tuple(JND))):
            rec["ms_to_jnd"][name] = {"uniform": max(nu[k] for k in keys) * ms_u,
                                      "learned": max(nl[k] for k in keys) * ms_l}
        ds.close()
        per_room.append(rec)
    net.close()
    extra = 1000.0 * (t_collect + t_train) / max(1, eval_rooms)  # one-off cost spread over the evaluated rooms
    res = {"train_loss": float(curve[-1]), "val_loss": float(val_loss), "collect_s": t_collect, "train_s": t_train}
    for k in JND:
        res[f"speedup_rays_{k}"] = _gmean([r["rays_to_jnd"]["uniform"][k] / r["rays_to_jnd"]["learned"][k]
                                           for r in per_room])
    for name in ("T30_C80", "all"):
        tu = [r["ms_to_jnd"][name]["uniform"] for r in per_room]
        tl = [r["ms_to_jnd"][name]["learned"] for r in per_room]
        res[f"wall_ms_to_jnd_{name}"] = {"uniform": _gmean(tu), "learned": _gmean(tl),
                                         "speedup": _gmean([a / b for a, b in zip(tu, tl)]),
                                         "learned_incl_training": _gmean(tl) + extra,
                                         "speedup_incl_training": _gmean(tu) / (_gmean(tl) + extra)}
    res["max_bias_z"] = {k: float(np.nanmax([r["bias_z"][k] for r in per_room])) for k in JND}
    res["bias_comparisons"] = int(eval_rooms * 3 * 8)
    res["wall_s"] = time.perf_counter() - t0
    return res


def run_jnd_arm(args):
    """One JSON line: wall time to T30 and C80 within 1 JND, learned proposal against uniform emission."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import torch
    torch.cuda.set_device(local)
    from pachydermacoustic_universal_gb300 import _capi
    _capi.lib()
    res = jnd_study(args.train_rooms, args.train_rays, args.eval_rooms, args.eval_rays, args.seeds, args.train_steps,
                    mix=args.mix, seed=args.seed, target=args.target)
    t = res["wall_ms_to_jnd_T30_C80"]
    line = {"metric": "wall time to T30/C80 <= 1 JND, learned vs uniform (1 GB300)", "value": t["speedup"],
            "unit": "x (uniform time / learned time, geometric mean over held-out rooms)", "n_gpus": 1,
            "higher_is_better": True, "vs_baseline": None, "dtype": "f32 geometry, f64 histograms, bf16 network",
            "data": "synthetic (seeded rooms drawn like the 10 x 8 x 4 m shoebox)",
            "config": {"workload": "learned_proposal_rooms", "train_rooms": args.train_rooms,
                       "train_rays_per_room": args.train_rays, "train_receivers": 12, "eval_rooms": args.eval_rooms,
                       "eval_rays_per_run": args.eval_rays, "seeds_per_method": args.seeds,
                       "train_steps": args.train_steps, "uniform_mix": args.mix, "target": args.target,
                       "network": "12 -> 3 x 256 GELU -> 32 vMF lobes (160), BF16 tcgen05, FP32 accumulate"},
            "jnd": res}
    print(json.dumps(line), flush=True)
    return 0


def filters_measure(h0, fs, reps, flush, device):
    """Receiver filters (Directional_Histogram.Create_Filter, 7 per receiver) of one step's histograms:
    device time of the filter kernels (CUDA events on the launching stream, L2 flushed between calls),
    the host-array call end to end, and the FP64 oracle on the host cores for one receiver."""
    import torch
    import ctypes as C
    from pachydermacoustic_universal_gb300 import _capi, tracer
    L = _capi.lib()
    E, P, Dp, Dn = (np.ascontiguousarray(h0[k]) for k in ("energy", "pressure", "dir_pos", "dir_neg"))
    R, _, T = P.shape
    n = R * 7
    d = {k: torch.from_numpy(v).to(device) for k, v in dict(E=E, P=P, Dp=Dp, Dn=Dn).items()}
    wsb = L.pach_filters_workspace_bytes(n, T)
    ws = torch.empty(wsb, dtype=torch.uint8, device=device)
    out = torch.empty((R, 7, T + 12287), dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream(device)
    sp = C.c_void_p(stream.cuda_stream)

    def call():
        _capi.check(L.pach_filters_device(d["E"].data_ptr(), d["P"].data_ptr(), d["Dp"].data_ptr(), d["Dn"].data_ptr(),
                                          None, R, T, 7, fs, None, 4096, out.data_ptr(), ws.data_ptr(), wsb, sp))

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    ms = 0.0
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    ms /= reps
    t0 = time.perf_counter()
    for _ in range(reps):
        tracer.receiver_filters(P, E, Dp, Dn, sample_rate=fs)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    from oracle import filters as OF
    t0 = time.perf_counter()
    OF.receiver_filters(E[0], P[0], Dp[0], Dn[0], [120.0] * 8, fs)
    cpu_ms = (time.perf_counter() - t0) * 1e3 / 7
    geo = 1 << (T + 16383 - 1).bit_length()
    roof = None
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_inputs.json")) as f:
            fp = json.load(f).get("filters", {})
    except (OSError, ValueError):
        fp = {}
    if fp.get("dp_inst_per_filter") and geo == 32768:
        # FP64 issue: DP lane-instructions per second against SMs x 2 FP64 lanes x the SM clock
        props = torch.cuda.get_device_properties(device)
        mhz = (_peaks()[0] or {}).get("sm_max_mhz", 2070.0)
        peak = props.multi_processor_count * fp["fp64_lanes_per_sm_cycle"] * mhz * 1e6
        ach = fp["dp_inst_per_filter"] * n / (ms * 1e-3)
        roof = {"bound": "fp64 issue", "achieved": ach / 1e9, "peak": peak / 1e9, "unit": "G DP lane-instructions/s",
                "frac": ach / peak, "per_unit": f"{fp['dp_inst_per_filter'] / 1e6:.2f} M DP instructions per filter "
                                                "of a 32768-point transform (ncu)",
                "peak_source": f"{props.multi_processor_count} SMs x {fp['fp64_lanes_per_sm_cycle']} FP64 lanes x "
                               f"{mhz:.0f} MHz", "source": fp.get("source")}
    return {"filters": n, "receivers": R, "bins": T, "transform_length": geo, "filter_samples": T + 12287,
            "device_ms": ms, "device_us_per_filter": ms * 1e3 / n, "e2e_ms": e2e_ms,
            "e2e_h2d_bytes": int(E.nbytes + P.nbytes + Dp.nbytes + Dn.nbytes), "e2e_d2h_bytes": int(n * (T + 12287) * 8),
            "launches": 4 + 3 * -(-n // max(1, min(n, (512 << 20) // (5 * geo * 16)))),
            "cpu_baseline": {"value": cpu_ms, "unit": "ms per filter", "cores": 1, "kind": "port",
                             "sample": "the 7 filters of receiver 0 (numpy FP64 FFT convolution)"},
            "roofline": roof,
            "timing": "CUDA events around pach_filters_device on its stream, 256 MiB written between calls"}


def run_filters_arm(args):
    """One JSON line: receiver filters of the arena's 64 receivers (7 each) from one traced step."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import torch
    torch.cuda.set_device(local)
    from pachydermacoustic_universal_gb300 import tracer, _capi
    _capi.lib()
    w = workload("arena", 1.0)[0]
    ds = tracer.DeviceScene(w.scene)
    h, _ = tracer.trace(w, dscene=ds, rays=args.batch or 200_000, seed=args.seed, scaled=True)
    ds.close()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    f = filters_measure(h, w.sample_rate, max(1, args.steps), flush, f"cuda:{local}")
    line = {"metric": "receiver filters per second (Directional_Histogram.Create_Filter, 1 GB300)",
            "value": f["filters"] / (f["device_ms"] * 1e-3), "unit": "filters/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 3, "higher_is_better": True, "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (histograms of one traced step of the arena)",
            "config": {"workload": "arena_filters", "receivers": f["receivers"], "bins": f["bins"],
                       "filters_per_receiver": 7},
            "e2e": {"value": f["filters"] / (f["e2e_ms"] * 1e-3), "unit": "filters/s",
                    "h2d_bytes_per_step": f["e2e_h2d_bytes"], "d2h_bytes_per_step": f["e2e_d2h_bytes"]},
            "detail": f}
    print(json.dumps(line), flush=True)
    return 0


def scene_bytes(scene):
    return int(scene.vertices.nbytes + scene.poly_offsets.nbytes + scene.poly_indices.nbytes +
               scene.absorption.nbytes + scene.scattering.nbytes + scene.transmission.nbytes)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--metric", default="bounces", choices=["bounces", "jnd", "filters"],
                    help="bounces: segment-bounces/s (default); jnd: wall time to 1 JND, learned vs uniform")
    ap.add_argument("--train-rooms", type=int, default=100, help="jnd: training rooms")
    ap.add_argument("--train-rays", type=int, default=20000, help="jnd: uniform primaries per training room")
    ap.add_argument("--eval-rooms", type=int, default=12, help="jnd: held-out rooms")
    ap.add_argument("--eval-rays", type=int, default=4000, help="jnd: primaries per evaluation run")
    ap.add_argument("--seeds", type=int, default=8, help="jnd: runs per method and room")
    ap.add_argument("--train-steps", type=int, default=3000, help="jnd: Adam steps")
    ap.add_argument("--mix", type=float, default=0.3, help="jnd: weight of uniform emission in the proposal")
    ap.add_argument("--target", default="linear", choices=["linear", "l2"], help="jnd: training target")
    ap.add_argument("--no-jnd", action="store_true",
                    help="skip the compact learned-vs-uniform JND study the default arena line carries")
    ap.add_argument("--workload", default="arena", choices=["hall", "shoebox", "batched", "arena", "hall_map"])
    ap.add_argument("--rays-total", type=int, default=None,
                    help="primaries the timed steps trace together (default: the workload's job, arena 10M)")
    ap.add_argument("--batch", type=int, default=None, help="primaries per step (default: rays_total / steps)")
    ap.add_argument("--timing-steps", type=int, default=3, help="steps of the per-kernel timing pass (roofline)")
    ap.add_argument("--e2e-steps", type=int, default=None, help="end-to-end steps (default: all timed steps)")
    ap.add_argument("--ray-sort", type=int, default=0,
                    help="1: order each wave by direction octant and origin cell before the walk (opt-in)")
    ap.add_argument("--ring-log2", type=int, default=0,
                    help="ring queue of 2^n octave rays (0: the engine's default; small cases for profiling)")
    ap.add_argument("--ray-scale", type=float, default=0.004, help="batched: fraction of each room's rays per step")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="primaries of the CPU baseline sample (default: about 10 s of CPU work per workload)")
    ap.add_argument("--ref-sample", type=int, default=None, help="primaries per step of the reference arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    # bounded CPU samples: the FP64 restatement's grid makes a 500k-triangle arena ~100x slower per segment
    if args.cpu_sample is None:
        args.cpu_sample = {"hall": 3000, "shoebox": 3000, "batched": 400, "arena": 400, "hall_map": 3000}[args.workload]
    if args.ref_sample is None:
        args.ref_sample = {"hall": 200, "shoebox": 200, "batched": 200, "arena": 48, "hall_map": 200}[args.workload]

    if args.impl == "reference":
        return run_reference_arm(args)
    if args.metric == "jnd":
        return run_jnd_arm(args)
    if args.metric == "filters":
        return run_filters_arm(args)

    ws, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = init_dist(ws, "nccl")
    from pachydermacoustic_universal_gb300 import tracer, _capi
    _capi.lib()
    rooms_ = workload(args.workload, args.ray_scale)
    batched = len(rooms_) > 1
    scenes = tracer.DeviceScene.many([w.scene for w in rooms_])
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    if batched:
        B = sum(w.rays for w in rooms_)
    else:
        total = args.rays_total or rooms_[0].rays
        B = args.batch or -(-total // args.steps)
    n_steps_all = args.warmup + args.steps + args.timing_steps
    # this rank's primaries: steps are consecutive batches; ranks own disjoint ranges
    base = rank * n_steps_all * B
    tune = None
    if batched:  # packet size and block shape from the autotuner (timed before the warm-up, cached)
        tune = tracer.autotune(rooms_, dscenes=scenes, sample_rays=min(B, 20000), seed=args.seed)

    # result buffers of the end-to-end steps in pinned host memory (the histograms' device-to-host copies
    # go straight into them)
    R_all = sum(len(w.receivers) for w in rooms_)
    T_all = int(rooms_[0].sample_rate * (max(w.cutoff_s for w in rooms_) * 1000.0) / 1000.0)  # as Run.T
    pinned = None
    if not args.no_e2e:
        def _pin(shape):
            return torch.zeros(int(np.prod(shape)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape)
        pinned = {"energy": _pin((R_all, 8, T_all)), "pressure": _pin((R_all, 8, T_all)),
                  "dir_pos": _pin((R_all, 3, 8, T_all)), "dir_neg": _pin((R_all, 3, 8, T_all)),
                  "analysis": _pin((R_all, 3, 8, T_all))}

    def step_trace(idx, ds, timing=False, out=None):
        """One step: primaries [base + idx B, base + (idx + 1) B) through the public API.  timing: the
        host-driven loop with CUDA events around every kernel (per-kernel times), else the product
        default, one CUDA-graph launch of the whole device loop."""
        kw = dict(seed=args.seed, ray_begin=base + idx * B, kernel_timing=timing, ring_log2=args.ring_log2,
                  ray_sort=args.ray_sort)
        t0 = time.perf_counter()
        if batched:
            h, s = tracer.trace_batch(rooms_, dscenes=ds, tune=tune, out=out, **kw)
        else:
            mr = map_of(rooms_[0])
            if mr is not None:
                kw["map_receivers"] = mr
            h, s = tracer.trace(rooms_[0], dscene=ds[0], rays=B, out=out, **kw)
            h.pop("map", None)
            h = [h]
        return h, s, time.perf_counter() - t0

    # step indices: [0, steps) timed, then the warm-up steps, then the kernel-timing steps
    for i in range(args.warmup):
        flush.zero_()
        step_trace(args.steps + i, scenes)
    torch.cuda.synchronize()
    barrier(dist)
    sampler = ClockSampler()
    sampler.start()
    dev_ms, segs, launches = 0.0, 0, 0
    stats = []
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        _, s, _ = step_trace(i, scenes)
        dev_ms += s["device_ms"]
        segs += s["segments"]
        launches += s["kernel_launches"]
        stats.append(s)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    barrier(dist)
    dev_ms_max = max_over_ranks(dist, dev_ms, device=f"cuda:{local}")
    segs_all = sum_over_ranks(dist, segs, device=f"cuda:{local}")
    value = segs_all / (dev_ms_max * 1e-3)

    # per-kernel times (roofline): the host-driven loop with CUDA events around every kernel
    tstats = []
    for i in range(args.timing_steps):
        flush.zero_()
        torch.cuda.synchronize()
        tstats.append(step_trace(args.steps + args.warmup + i, scenes, timing=True)[1])
    if not tstats:
        tstats = stats

    # e2e through the C ABI with host buffers: the scene built from the host arrays and uploaded once
    # per job, then every step's trace with its histograms downloaded into pinned host buffers
    e2e = None
    if not args.no_e2e:
        e_steps = max(1, min(args.steps, args.e2e_steps or args.steps))
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        ds = tracer.DeviceScene.many([w.scene for w in rooms_])
        t_scene = time.perf_counter() - t0
        es = 0
        for i in range(e_steps):
            h, s, _ = step_trace(i, ds, out=pinned)
            es += s["segments"]
        for d in ds:
            d.close()
        torch.cuda.synchronize()
        tt = time.perf_counter() - t0
        tt = max_over_ranks(dist, tt, device=f"cuda:{local}")
        es = sum_over_ranks(dist, es, device=f"cuda:{local}")
        h2d_scene = sum(scene_bytes(w.scene) for w in rooms_)
        h2d = int(h2d_scene / e_steps) + sum(88 * len(w.sources) + 32 * len(w.receivers) for w in rooms_)
        d2h = int(sum(v.nbytes for hh in h for v in hh.values()))
        e2e = {"value": es / tt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": e_steps, "scene_build_upload_s": t_scene, "wall_s": tt,
               "includes": "one scene build (host BVH) and upload per job, then per step: run set-up, trace, "
                           "histogram download into pinned host buffers; scene bytes amortised over the steps"}

    peaks, peak_kind = _peaks()
    agg = {k: sum(s[k] for s in tstats) for k in ("segments", "detections", "fp64_retests", "octave_rays",
                                                    "segments_broadband", "segments_phase_b", "segments_phase_c",
                                                    "trace_ms", "shade_ms", "broadband_ms", "waves",
                                                    "bvh_nodes_visited", "tri_tests", "device_ms")}
    # HBM roofline of the dominant wavefront kernel, algorithmic bytes per octave-ray segment:
    #   k_trace  reads the ray's position, direction and plane (48 B) and writes (triangle, t) (8 B);
    #   k_shade  reads the 64 B ray and its 8 B hit, writes the surviving ray and split children
    #            (64 B each) and 6 FP64 histogram atomics (48 B) per detection.
    # The scene and BVH (a few MB) stay L2-resident and are not counted.
    seg_oct = agg["segments_phase_b"] + agg["segments_phase_c"]
    trace_bytes = 56.0 * seg_oct
    shade_bytes = 72.0 * seg_oct + 64.0 * (seg_oct + agg["octave_rays"]) + 48.0 * agg["detections"]
    kern = "k_trace" if agg["trace_ms"] >= agg["shade_ms"] else "k_shade"
    k_ms = agg["trace_ms"] if kern == "k_trace" else agg["shade_ms"]
    k_bytes = trace_bytes if kern == "k_trace" else shade_bytes
    achieved_gbs = k_bytes / (k_ms * 1e-3) / 1e9 if k_ms > 0 else None
    oct_launch = agg["waves"]
    # the on-chip side of the walk: BVH node (128 B) and triangle (48 B) reads served by L1/L2
    node_bytes = float(stats[0]["walk"] % 1000) or 128.0
    bvh_gbs = ((node_bytes * agg["bvh_nodes_visited"] + 48.0 * agg["tri_tests"]) / (agg["trace_ms"] * 1e-3) / 1e9
               if agg["trace_ms"] > 0 else None)
    tris = sum(w.scene.n_triangles for w in rooms_)
    cfg = {"workload": rooms_[0].name if not batched else f"batched_{len(rooms_)}_rooms",
           "rays_per_step": B, "rays_total": B * args.steps * ws, "triangles": tris,
           "timing": "graph-mode device loop per step (CUDA events); per-kernel times from "
                     f"{len(tstats)} further kernel-timing steps",
           "sources": sum(len(w.sources) for w in rooms_), "receivers": sum(len(w.receivers) for w in rooms_),
           "cutoff_s": max(w.cutoff_s for w in rooms_), "bins_ms": 1, "l2": "256 MiB buffer written between steps",
           "bvh_nodes_leaves_depth": stats[0]["accel"], "walk": stats[0]["walk"]}
    if rooms_[0].extra.get("map") is not None:
        m = rooms_[0].extra["map"]
        cfg["workload"] += "_map"
        cfg["map_receivers"] = int(len(m["origins"]))
        cfg["map_increment_m"] = m["increment"]
        cfg["map_walk"] = m["walk"]
    if batched:
        cfg["rooms"] = len(rooms_)
        cfg["ray_scale"] = args.ray_scale
        cfg["autotune"] = {k: tune[k] for k in tracer.TUNE_KNOBS + ("from_cache",)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 geometry, f64 histograms", "data": "synthetic (seeded room generator)",
        "config": cfg,
        "gpu_launches": launches,
        "clocks": clocks,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": kern,
                     "achieved": achieved_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": (achieved_gbs / peaks["hbm_gbs"]) if achieved_gbs else None,
                     "traffic": None, "peak_source": peak_kind,
                     "per_unit": ("56 B per octave segment" if kern == "k_trace" else
                                  "72 B in + 64 B per output ray per octave segment + 48 B per detection"),
                     "bvh_reads_gbs": bvh_gbs,
                     "bvh_reads_note": f"BVH node ({node_bytes:.0f} B) and triangle (48 B) reads of the walk per "
                                       "second of k_trace, served by L1/L2 (the walk's binding resource is on-chip)"},
        "detail": {"trace_ms": agg["trace_ms"], "shade_ms": agg["shade_ms"], "broadband_ms": agg["broadband_ms"],
                   "waves": agg["waves"], "wall_s": wall, "segments": agg["segments"],
                   "detections": agg["detections"], "fp64_retests": agg["fp64_retests"],
                   "octave_rays": agg["octave_rays"], "peak_live_rays": max(s["peak_live_rays"] for s in stats),
                   "bvh_nodes_per_segment": agg["bvh_nodes_visited"] / max(1, seg_oct),
                   "tri_tests_per_segment": agg["tri_tests"] / max(1, seg_oct),
                   "segments_phase_c_frac": agg["segments_phase_c"] / max(1, agg["segments"]),
                   "kernel_timing_pass_segments_per_s": agg["segments"] / max(agg["device_ms"] * 1e-3, 1e-30)},
    }
    # ncu figures per octave segment of the dominant kernel on this workload (profiles/roofline_inputs.json):
    # DRAM bytes (-> traffic per launch) and executed lane-instructions (-> the issue roofline)
    prof = {}
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_inputs.json")) as f:
            prof = json.load(f).get(args.workload, {}).get(kern, {})
    except (OSError, ValueError):
        prof = {}
    if prof.get("dram_bytes_per_segment") and not batched:
        line["roofline"]["traffic"] = prof["dram_bytes_per_segment"] * seg_oct / max(1, oct_launch)
        line["roofline"]["traffic_source"] = prof.get("source")
    if prof.get("thread_inst_per_segment") and k_ms > 0:
        # The walk is bound by instruction issue, not HBM: useful lane-instructions per second against
        # the SM issue peak, SMs x 4 schedulers x 32 lanes x the sampled SM clock.
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
        lane_peak = sms * 4 * 32 * mhz * 1e6
        lane_rate = prof["thread_inst_per_segment"] * seg_oct / (k_ms * 1e-3)
        warp_rate = prof.get("warp_inst_per_segment", 0.0) * seg_oct / (k_ms * 1e-3)
        line["roofline"]["binding"] = {
            "resource": "issue", "kernel": kern, "achieved": lane_rate / 1e12, "peak": lane_peak / 1e12,
            "unit": "T lane-instructions/s", "frac": lane_rate / lane_peak,
            "warp_issue_frac": warp_rate / (lane_peak / 32),
            "lanes_active_per_warp_instruction": (prof["thread_inst_per_segment"] /
                                                  max(prof.get("warp_inst_per_segment", 0.0), 1e-30)),
            "per_unit": f"{prof['thread_inst_per_segment']:.0f} lane-instructions and "
                        f"{prof.get('warp_inst_per_segment', 0.0):.0f} warp-instructions per octave segment (ncu)",
            "peak_source": f"{sms} SMs x 4 schedulers x 32 lanes x {mhz:.0f} MHz (sampled)",
            "source": prof.get("source")}
    if rank == 0 and ws >= 1 and not args.no_cpu_baseline:
        sample_rooms = rooms_[:4]
        cb, st = cpu_baseline(sample_rooms, args.cpu_sample, args.seed)
        line["cpu_baseline"] = cb
        k_cell = st["cells_visited"] / st["segments"]
        k_tri = st["tri_tests"] / st["segments"]
        det = st["detections"] / st["segments"]
        R = sum(len(w.receivers) for w in sample_rooms) / len(sample_rooms)
        flops_seg = 9 * k_cell + 27 * k_tri + 20 * R + 40
        bytes_seg = 8 * k_cell + 36 * k_tri + 2 * 48 + 12 * det
        line["reference_work"] = {"k_cell": k_cell, "k_tri": k_tri, "detections_per_segment": det,
                                  "flops_per_segment": flops_seg, "bytes_per_segment": bytes_seg,
                                  "reference_work_tflops": flops_seg * value / 1e12,
                                  "reference_work_gbs": bytes_seg * value / 1e9,
                                  "note": "work the reference traversal (grid domain 7) does for the same "
                                          "segments, at this run's segment rate"}
    if rank == 0 and e2e is not None and not batched and rooms_[0].receivers:
        # the receivers' filters (auralisation impulse responses) of the last end-to-end step
        line["filters"] = filters_measure(h[0], rooms_[0].sample_rate, 5, flush, f"cuda:{local}")
    if rank == 0 and not args.no_jnd and args.workload == "arena":
        # the metric's second half, measured in the same run at a compact size (bench.py --metric jnd
        # runs the larger study): wall time to T30 and C80 within 1 JND, learned proposal vs uniform
        res = jnd_study(40, 20000, 8, 4000, 8, 2000, mix=0.3, seed=args.seed)
        t = res["wall_ms_to_jnd_T30_C80"]
        line["jnd"] = {"metric": "wall time to T30/C80 <= 1 JND, learned vs uniform",
                       "speedup": t["speedup"], "uniform_ms": t["uniform"], "learned_ms": t["learned"],
                       "learned_incl_training_ms": t["learned_incl_training"],
                       "speedup_rays": {k: res[f"speedup_rays_{k}"] for k in JND},
                       "max_bias_z": res["max_bias_z"], "collect_s": res["collect_s"], "train_s": res["train_s"],
                       "config": "40 training rooms x 12 receivers x 20k uniform primaries, 2000 Adam steps; "
                                 "8 held-out rooms x 8 seeds x 4000 primaries per method; uniform weight 0.3",
                       "wall_s": res["wall_s"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
