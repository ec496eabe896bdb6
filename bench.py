"""Benchmark: segment-bounces/s of the split ray tracer.

Default workload (one GPU): the 40 x 25 x 15 m jittered hall with 200 diffusers (~20k triangles),
2 sources, 16 receivers of radius 0.5 m, 3 s cutoff, 1 ms bins, 1M primary rays.  A step traces
one batch of primaries (default 131072); the timed steps together cover the 1M-ray job, each step
tracing its own primaries (ray_begin = step * batch), the warm-up steps trace primaries after them.
--workload shoebox: the 12-triangle 10 x 8 x 4 m shoebox; --workload arena: the 500k-triangle
120 x 90 x 35 m arena; --workload hall_map: the hall with a 608-receiver audience map (1 m squares at
1.5 m, the reference's grid walks); --workload batched: the 64-room batch (each room's ray count x
--ray-scale per step) as one batch run with autotuned knobs.

Metric: segment-bounces/s = shoot calls (broadband + octave rays, hit or miss) per second.
  value  -- device time of the engine's kernels (CUDA events on the engine's stream), scene resident.
  e2e    -- through the public C ABI from host buffers: scene upload, trace, histogram download.
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
    """The rooms of a bench workload: the irregular hall (default), the 12-triangle shoebox, the
    500k-triangle arena, or the 64-room batch (ray counts scaled by ray_scale)."""
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


def scene_bytes(scene):
    return int(scene.vertices.nbytes + scene.poly_offsets.nbytes + scene.poly_indices.nbytes +
               scene.absorption.nbytes + scene.scattering.nbytes + scene.transmission.nbytes)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hall", choices=["hall", "shoebox", "batched", "arena", "hall_map"])
    ap.add_argument("--batch", type=int, default=131072, help="primaries per step (single-room workloads)")
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
        args.cpu_sample = {"hall": 3000, "shoebox": 3000, "batched": 400, "arena": 40, "hall_map": 3000}[args.workload]
    if args.ref_sample is None:
        args.ref_sample = {"hall": 200, "shoebox": 200, "batched": 200, "arena": 8, "hall_map": 200}[args.workload]

    if args.impl == "reference":
        return run_reference_arm(args)

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
    B = sum(w.rays for w in rooms_) if batched else args.batch
    # this rank's primaries: steps are consecutive batches; ranks own disjoint ranges
    base = rank * (args.warmup + args.steps) * B
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

    def step_trace(idx, e2e=False):
        kw = dict(seed=args.seed, ray_begin=base + idx * B, kernel_timing=not e2e)
        t0 = time.perf_counter()
        # e2e: the public API from host buffers -- upload the scenes, trace, download the histograms
        ds = tracer.DeviceScene.many([w.scene for w in rooms_]) if e2e else scenes
        out = pinned if e2e else None
        if batched:
            h, s = tracer.trace_batch(rooms_, dscenes=ds, tune=tune, out=out, **kw)
        else:
            mr = map_of(rooms_[0])
            if mr is not None:
                kw["map_receivers"] = mr
            h, s = tracer.trace(rooms_[0], dscene=ds[0], rays=B, out=out, **kw)
            h.pop("map", None)
            h = [h]
        if e2e:
            for d in ds:
                d.close()
        return h, s, time.perf_counter() - t0

    for i in range(args.warmup):
        flush.zero_()
        step_trace(args.steps + i)
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
        _, s, _ = step_trace(i)
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

    # e2e through the C ABI with host buffers (scene upload + histogram download each step)
    e2e = None
    if not args.no_e2e:
        e_steps = max(1, min(args.steps, 3))
        tt, es = 0.0, 0
        h2d = d2h = 0
        for i in range(e_steps):
            h, s, dt = step_trace(i, e2e=True)
            tt += dt
            es += s["segments"]
            h2d = sum(scene_bytes(w.scene) + 88 * len(w.sources) + 32 * len(w.receivers) for w in rooms_)
            d2h = int(sum(v.nbytes for hh in h for v in hh.values()))
        tt = max_over_ranks(dist, tt, device=f"cuda:{local}")
        es = sum_over_ranks(dist, es, device=f"cuda:{local}")
        e2e = {"value": es / tt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": e_steps, "includes": "scene build and upload, trace, histogram download into pinned host "
                                             "buffers"}

    peaks, peak_kind = _peaks()
    agg = {k: sum(s[k] for s in stats) for k in ("segments", "detections", "fp64_retests", "octave_rays",
                                                   "segments_broadband", "segments_phase_b", "segments_phase_c",
                                                   "trace_ms", "shade_ms", "broadband_ms", "waves",
                                                   "bvh_nodes_visited", "tri_tests")}
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
                   "segments_phase_c_frac": agg["segments_phase_c"] / max(1, agg["segments"])},
    }
    traffic_file = os.path.join(ROOT, "profiles", f"{kern}_traffic.json")
    if os.path.exists(traffic_file) and not batched:
        try:
            tr = json.load(open(traffic_file))
            line["roofline"]["traffic"] = tr.get("dram_bytes_per_segment", 0) * seg_oct / max(1, oct_launch)
            line["roofline"]["traffic_source"] = tr.get("source")
        except Exception:
            pass
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
