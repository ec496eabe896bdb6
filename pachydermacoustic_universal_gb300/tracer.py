"""Array-level Python API over the C ABI: device scenes, runs, histograms and stats."""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import _capi
from ._capi import check, dptr, iptr


class DeviceScene:
    """A scene resident on the GPU (pach_scene_create)."""

    def __init__(self, scene, bvh_leaf_max: int = 0, _handle=None):
        L = _capi.lib()
        desc = self._desc(scene, bvh_leaf_max)
        if _handle is not None:
            self.handle = _handle
        else:
            h = C.c_void_p()
            check(L.pach_scene_create(C.byref(desc), C.byref(h)))
            self.handle = h
        self.n_polys = self._o.size - 1

    @classmethod
    def many(cls, scenes, bvh_leaf_max: int = 0, threads: int = 0):
        """Several scenes at once (pach_scenes_create: host builds in parallel)."""
        L = _capi.lib()
        holders = [cls.__new__(cls) for _ in scenes]
        descs = (_capi.SceneDesc * max(1, len(scenes)))()
        for i, (hd, sc) in enumerate(zip(holders, scenes)):
            descs[i] = hd._desc(sc, bvh_leaf_max)
        hs = (C.c_void_p * max(1, len(scenes)))()
        check(L.pach_scenes_create(descs, len(scenes), hs, int(threads)))
        out = []
        for i, (hd, sc) in enumerate(zip(holders, scenes)):
            hd.handle = C.c_void_p(hs[i])
            hd.n_polys = hd._o.size - 1
            out.append(hd)
        return out

    def _desc(self, scene, bvh_leaf_max):
        self._v = np.ascontiguousarray(scene.vertices, dtype=np.float64).reshape(-1)
        self._o = np.ascontiguousarray(scene.poly_offsets, dtype=np.int32)
        self._i = np.ascontiguousarray(scene.poly_indices, dtype=np.int32)
        self._a = np.ascontiguousarray(scene.absorption, dtype=np.float64).reshape(-1)
        self._s = np.ascontiguousarray(scene.scattering, dtype=np.float64).reshape(-1)
        tr = getattr(scene, "transmission", None)
        self._t = np.ascontiguousarray(tr, dtype=np.float64).reshape(-1) if tr is not None else None
        return _capi.SceneDesc(self._v.size // 3, dptr(self._v), self._o.size - 1, iptr(self._o), iptr(self._i),
                               dptr(self._a), dptr(self._s), dptr(self._t), scene.temp_c, scene.rel_humidity,
                               scene.pressure_hpa, scene.air_choice, scene.edge_correction, int(bvh_leaf_max), 0)

    def info(self):
        L = _capi.lib()
        npoly, ntri = C.c_int32(), C.c_int32()
        c, rc = C.c_double(), C.c_double()
        att = np.zeros(8)
        area = np.zeros(self.n_polys)
        check(L.pach_scene_info(self.handle, C.byref(npoly), C.byref(ntri), C.byref(c), C.byref(rc), dptr(att), dptr(area)))
        return {"n_polys": npoly.value, "n_triangles": ntri.value, "sound_speed": c.value, "rho_c": rc.value,
                "air_atten_db_per_m": att, "poly_area": area}

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().pach_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def source_array(sources):
    arr = (_capi.SourceDesc * len(sources))()
    for i, s in enumerate(sources):
        arr[i].origin[:] = [float(x) for x in s.origin]
        arr[i].power_db[:] = [float(x) for x in s.power_db]
        arr[i].kind = int(s.kind)
    return arr


def receiver_array(receivers):
    arr = (_capi.ReceiverDesc * max(1, len(receivers)))()
    for i, r in enumerate(receivers):
        arr[i].origin[:] = [float(x) for x in r.origin]
        arr[i].radius = float(r.radius)
    return arr


@dataclasses.dataclass
class MapReceivers:
    """Mapping receivers (PachMapReceiver): spheres of diameter `increment` centred at `origins`
    [M][3], histograms of `cutoff_ms` ms at 1000 Hz counted from each receiver's direct arrival (one
    bin with time_1pt).  walk 0 reproduces the reference's grid walks, 1 visits every crossed cell."""
    origins: np.ndarray
    increment: float
    cutoff_ms: float
    time_1pt: bool = False
    walk: int = 0
    directional: bool = False

    def desc(self):
        org = np.ascontiguousarray(self.origins, dtype=np.float64).reshape(-1, 3)
        d = _capi.MapDesc()
        d.n_receivers = org.shape[0]
        d.time_1pt = int(bool(self.time_1pt))
        d.origins = dptr(org)
        d.increment = float(self.increment)
        d.cutoff_ms = float(self.cutoff_ms)
        d.walk = int(self.walk)
        d.directional = int(bool(self.directional))
        d._keep = org
        return d

    @property
    def bins(self):
        return 1 if self.time_1pt else int(float(self.cutoff_ms) / 1000.0 * 1000.0)


def make_params(*, rays, cutoff_length_m, hist_cotime_ms, seed=1, oct_range=(0, 7), is_order=-1, sample_rate=1000,
                pure_specular=False, max_broadband_bounces=0, max_segments_per_ray=0, feed_batch=0,
                block_threads=0, blocks_per_sm=0, prim_dirs=None, prim_weights=None, ray_begin=0, wave_kilo_items=0,
                ring_log2=0, kernel_timing=False, ray_sort=0, traversal=0, capture=False, capture_edges_ms=None,
                proposal=None, proposal_mix=0.0, bvh_format=0, map_receivers=None, max_rays=0):
    p = _capi.TraceParams()
    p.seed = seed
    p.ray_count = int(rays)
    p.ray_begin = int(ray_begin)
    p.cutoff_length_m = float(cutoff_length_m)
    p.oct_lo, p.oct_hi = int(oct_range[0]), int(oct_range[1])
    p.is_order = int(is_order)
    p.sample_rate = int(sample_rate)
    p.hist_cotime_ms = float(hist_cotime_ms)
    p.pure_specular = int(bool(pure_specular))
    p.max_broadband_bounces = int(max_broadband_bounces)
    p.max_segments_per_ray = int(max_segments_per_ray)
    p.feed_batch = int(feed_batch)
    p.block_threads = int(block_threads)
    p.blocks_per_sm = int(blocks_per_sm)
    p.wave_kilo_items = int(wave_kilo_items)
    p.ring_log2 = int(ring_log2)
    p.kernel_timing = int(bool(kernel_timing))
    p.ray_sort = int(ray_sort)
    p.traversal = int(traversal)
    p.bvh_format = int(bvh_format)
    p.max_rays = int(max_rays)
    p.prim_dirs = dptr(prim_dirs)
    p.prim_weights = dptr(prim_weights)
    p.capture = int(capture)
    if capture_edges_ms is not None:
        p.capture_edges_ms[:] = [float(x) for x in capture_edges_ms]
    if proposal is not None:
        p.proposal = _capi.fptr(proposal)
        p.n_proposal = int(proposal.shape[0])
        p.proposal_mix = float(proposal_mix)
    if map_receivers is not None:
        md = map_receivers.desc()
        p.map = C.pointer(md)
        p._map_keep = md
    return p


class Run:
    """An asynchronous tracing run (pach_trace_begin ... pach_run_destroy)."""

    def __init__(self, dscene: DeviceScene, sources, receivers, params, keep=()):
        L = _capi.lib()
        self._src = source_array(sources)
        self._rec = receiver_array(receivers)
        self._keep = keep
        self.R = len(receivers)
        self.params = params
        self.T = int(params.sample_rate * params.hist_cotime_ms / 1000.0)
        h = C.c_void_p()
        check(L.pach_trace_begin(dscene.handle, self._src, len(sources), self._rec, len(receivers), C.byref(params),
                                 C.byref(h)))
        self.handle = h

    def poll(self):
        pr = _capi.Progress()
        check(_capi.lib().pach_trace_poll(self.handle, C.byref(pr)))
        return {k: getattr(pr, k) for k, _ in pr._fields_}

    def cancel(self):
        check(_capi.lib().pach_trace_cancel(self.handle))

    def wait(self, timeout_ms=-1):
        check(_capi.lib().pach_trace_wait(self.handle, timeout_ms))

    def histograms(self, scaled=False, out=None):
        """Histograms; out: optional dict of preallocated float64 arrays of these shapes (for example
        views of pinned host memory, which the library's device-to-host copies then use directly)."""
        R, T = self.R, self.T
        shapes = {"energy": (R, 8, T), "pressure": (R, 8, T), "dir_pos": (R, 3, 8, T), "dir_neg": (R, 3, 8, T),
                  "analysis": (R, 3, 8, T)}
        if out is None:
            out = {k: np.zeros(v) for k, v in shapes.items()}
        for k, v in shapes.items():
            a = out[k]
            if a.shape != v or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"out[{k!r}] must be a C-contiguous float64 array of shape {v}")
        E, P, Dp, Dn, An = (out[k] for k in shapes)
        check(_capi.lib().pach_trace_get_histograms(self.handle, int(bool(scaled)), dptr(E), dptr(P), dptr(Dp),
                                                    dptr(Dn), dptr(An), E.size))
        return {"energy": E, "pressure": P, "dir_pos": Dp, "dir_neg": Dn, "analysis": An}

    def filters(self, directional=True, swl=None):
        """Receiver filters from the run's device histograms (Directional_Histogram.Create_Filter,
        Classes_Receivers.cs:1910-1937): [R][7][T + 12287] (omni, then -x +x -y +y -z +z arrivals
        weighted by P Dir_Rec_Neg / E and P Dir_Rec_Pos / E), or [R][1][...] with directional=False;
        swl: the source's 8 band powers (dB), None for 120 dB."""
        kinds = 7 if directional else 1
        out = np.zeros((self.R, kinds, self.T + FILTER_LEN_ADD - FILTER_CUT))
        sw = None if swl is None else np.ascontiguousarray(swl, dtype=np.float64)
        check(_capi.lib().pach_trace_get_filters(self.handle, int(bool(directional)), dptr(sw), dptr(out), out.size))
        return out

    def capture(self):
        """Captured energy (W, unscaled): capture 1 -> [R][4][1536] per emission-direction bin,
        capture 2 -> [primaries][R][4] per primary."""
        if self.params.capture == 2:
            out = np.zeros((self.params.ray_count, self.R, _capi.CAPTURE_WINDOWS), dtype=np.float32)
        else:
            out = np.zeros((self.R, _capi.CAPTURE_WINDOWS, _capi.DIR_BINS), dtype=np.float32)
        check(_capi.lib().pach_trace_get_capture(self.handle, _capi.fptr(out), out.size))
        return out

    def map_histograms(self, scaled=False):
        """Map histograms energy / pressure [M][8][T] (time 0 = each receiver's direct arrival) and
        the direct arrival times [M] (s)."""
        L = _capi.lib()
        sizes = np.zeros(2, dtype=np.int32)
        check(L.pach_trace_get_map(self.handle, 0, None, None, None, iptr(sizes), 0))
        M, T = int(sizes[0]), int(sizes[1])
        E, P, D = np.zeros((M, 8, T)), np.zeros((M, 8, T)), np.zeros(M)
        check(L.pach_trace_get_map(self.handle, int(bool(scaled)), dptr(E), dptr(P), dptr(D), None, E.size))
        out = {"energy": E, "pressure": P, "direct_time": D}
        pm = self.params.map
        if pm and pm.contents.directional:
            Dp, Dn = np.zeros((M, 3, 8, T)), np.zeros((M, 3, 8, T))
            check(L.pach_trace_get_map_directions(self.handle, int(bool(scaled)), dptr(Dp), dptr(Dn), Dp.size))
            out.update(dir_pos=Dp, dir_neg=Dn)
        return out

    def map_parameters(self, decay_depth=30, clarity_ms=80):
        """T_X, EDT, clarity (dB), definition (%) and total energy of every map receiver and band [M][8],
        computed on the device."""
        L = _capi.lib()
        sizes = np.zeros(2, dtype=np.int32)
        check(L.pach_trace_get_map(self.handle, 0, None, None, None, iptr(sizes), 0))
        M = int(sizes[0])
        out = {k: np.zeros((M, 8)) for k in ("t_x", "edt", "clarity", "definition", "energy")}
        check(L.pach_map_parameters(self.handle, int(decay_depth), int(clarity_ms), dptr(out["t_x"]),
                                    dptr(out["edt"]), dptr(out["clarity"]), dptr(out["definition"]),
                                    dptr(out["energy"])))
        return out

    def stats(self):
        s = _capi.Stats()
        check(_capi.lib().pach_trace_get_stats(self.handle, C.byref(s)))
        return s.to_dict()

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().pach_run_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchRun(Run):
    """A batch run over several rooms traced as one wavefront (pach_batch_begin)."""

    def __init__(self, dscenes, workloads, rays, params):
        L = _capi.lib()
        self._src = [source_array(w.sources) for w in workloads]
        self._rec = [receiver_array(w.receivers) for w in workloads]
        descs = (_capi.RoomDesc * len(workloads))()
        for i, w in enumerate(workloads):
            descs[i].scene = dscenes[i].handle.value
            descs[i].sources = self._src[i]
            descs[i].n_sources = len(w.sources)
            descs[i].receivers = self._rec[i]
            descs[i].n_receivers = len(w.receivers)
            descs[i].ray_count = int(rays[i])
            descs[i].cutoff_length_m = float(w.cutoff_length_m)
        self._descs = descs
        self._keep = dscenes
        self.room_receivers = [len(w.receivers) for w in workloads]
        self.R = sum(self.room_receivers)
        self.params = params
        self.T = int(params.sample_rate * params.hist_cotime_ms / 1000.0)
        h = C.c_void_p()
        check(L.pach_batch_begin(descs, len(workloads), C.byref(params), C.byref(h)))
        self.handle = h

    def room_histograms(self, scaled=False, out=None):
        """Histograms split per room (the run's receiver rows in room order)."""
        h = self.histograms(scaled=scaled, out=out)
        out, k = [], 0
        for n in self.room_receivers:
            out.append({name: v[k:k + n] for name, v in h.items()})
            k += n
        return out


def _batch_params(workloads, n, seed, **kw):
    hist_ms = max(w.cutoff_s for w in workloads) * 1000.0
    return make_params(rays=sum(n), cutoff_length_m=workloads[0].cutoff_length_m, hist_cotime_ms=hist_ms, seed=seed,
                       sample_rate=workloads[0].sample_rate, **kw)


TUNE_KNOBS = ("wave_kilo_items", "block_threads", "blocks_per_sm", "traversal")


def autotune(workloads, *, dscenes=None, rays=None, sample_rays=20_000, cache_path=None, force=False, seed=1, **kw):
    """Packet size and block shape for these rooms (pach_autotune); returns a dict with the four knobs
    (TUNE_KNOBS), the measured sample throughput and whether it came from the cache."""
    ds = dscenes or DeviceScene.many([w.scene for w in workloads])
    n = [w.rays for w in workloads] if rays is None else list(rays)
    params = _batch_params(workloads, n, seed, **kw)
    src = [source_array(w.sources) for w in workloads]
    rec = [receiver_array(w.receivers) for w in workloads]
    descs = (_capi.RoomDesc * len(workloads))()
    for i, w in enumerate(workloads):
        descs[i].scene = ds[i].handle.value
        descs[i].sources = src[i]
        descs[i].n_sources = len(w.sources)
        descs[i].receivers = rec[i]
        descs[i].n_receivers = len(w.receivers)
        descs[i].ray_count = int(n[i])
        descs[i].cutoff_length_m = float(w.cutoff_length_m)
    res = _capi.TuneResult()
    path = cache_path.encode() if cache_path else None
    check(_capi.lib().pach_autotune(descs, len(workloads), C.byref(params), int(sample_rays), path, int(bool(force)),
                                    C.byref(res)))
    return {k: getattr(res, k) for k, _ in res._fields_}


def trace_batch(workloads, *, dscenes=None, seed=1, rays=None, scaled=False, tune=None, out=None, **kw):
    """Trace several rooms.Workload as one batch run; returns (per-room histograms, stats).
    tune: a dict from autotune() whose knobs are applied; out: see Run.histograms."""
    ds = dscenes or DeviceScene.many([w.scene for w in workloads])
    n = [w.rays for w in workloads] if rays is None else list(rays)
    if tune:
        for k in TUNE_KNOBS:
            kw.setdefault(k, tune[k])
    params = _batch_params(workloads, n, seed, **kw)
    run = BatchRun(ds, workloads, n, params)
    try:
        run.wait()
        return run.room_histograms(scaled=scaled, out=out), run.stats()
    finally:
        run.close()


def trace(workload, *, dscene=None, seed=1, rays=None, scaled=False, out=None, **kw):
    """Trace a rooms.Workload on the GPU; returns (histograms, stats).  out: see Run.histograms."""
    ds = dscene or DeviceScene(workload.scene)
    n = workload.rays if rays is None else rays
    pd = kw.pop("prim_dirs", None)
    pw = kw.pop("prim_weights", None)
    pr = kw.pop("proposal", None)
    pd = np.ascontiguousarray(pd, dtype=np.float64) if pd is not None else None
    pw = np.ascontiguousarray(pw, dtype=np.float64) if pw is not None else None
    pr = np.ascontiguousarray(pr, dtype=np.float32).reshape(-1, _capi.MLP_OUT) if pr is not None else None
    params = make_params(rays=n, cutoff_length_m=workload.cutoff_length_m, hist_cotime_ms=workload.cutoff_s * 1000.0,
                         seed=seed, sample_rate=workload.sample_rate, prim_dirs=pd, prim_weights=pw, proposal=pr, **kw)
    run = Run(ds, workload.sources, workload.receivers, params, keep=(pd, pw, pr))
    try:
        run.wait()
        h = run.histograms(scaled=scaled, out=out)
        if params.capture:
            h["capture"] = run.capture()
        if kw.get("map_receivers") is not None:
            h["map"] = run.map_histograms(scaled=scaled)
        return h, run.stats()
    finally:
        run.close()


def specular_paths(dscene: DeviceScene, origins, dirs, max_bounces):
    o = np.ascontiguousarray(origins, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    n = o.shape[0]
    poly = np.zeros((n, max_bounces), dtype=np.int32)
    t = np.zeros((n, max_bounces))
    pts = np.zeros((n, max_bounces, 3))
    check(_capi.lib().pach_trace_specular_paths(dscene.handle, n, dptr(o), dptr(d), max_bounces, iptr(poly), dptr(t),
                                                dptr(pts)))
    return poly, t, pts


def shoot_host(scene, origins, dirs):
    """Nearest hits found by the engine's BVH walked on the host (no GPU needed)."""
    v = np.ascontiguousarray(scene.vertices, dtype=np.float64).reshape(-1)
    offs = np.ascontiguousarray(scene.poly_offsets, dtype=np.int32)
    idx = np.ascontiguousarray(scene.poly_indices, dtype=np.int32)
    a = np.ascontiguousarray(scene.absorption, dtype=np.float64).reshape(-1)
    s = np.ascontiguousarray(scene.scattering, dtype=np.float64).reshape(-1)
    desc = _capi.SceneDesc(v.size // 3, dptr(v), offs.size - 1, iptr(offs), iptr(idx), dptr(a), dptr(s), None,
                           scene.temp_c, scene.rel_humidity, scene.pressure_hpa, scene.air_choice,
                           scene.edge_correction, 0, 0)
    o = np.ascontiguousarray(origins, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    n = o.shape[0]
    poly = np.zeros(n, dtype=np.int32)
    t = np.zeros(n)
    check(_capi.lib().pach_scene_shoot_host(C.byref(desc), n, dptr(o), dptr(d), iptr(poly), dptr(t)))
    return poly, t


def convergence_replay(per_rev, mode, distance_m, sound_speed, sample_rate=1000):
    """The engine's convergence checks (pach_convergence_replay) over per-revolution contributions
    per_rev [revs][4][T] (energy, analysis 0..2 of one receiver, band h_oct).  mode 0 SpecMin, 1 Minimum.
    Returns (first revolution after which the check agreed, 1-based, 0 if none; SpecMin's Nmin)."""
    h = np.ascontiguousarray(per_rev, dtype=np.float64)
    stop = C.c_int32()
    nmin = C.c_int64()
    check(_capi.lib().pach_convergence_replay(dptr(h), h.shape[0], h.shape[2], int(sample_rate), int(mode),
                                              float(distance_m), float(sound_speed), C.byref(stop), C.byref(nmin)))
    return stop.value, nmin.value


FILTER_LEN_ADD = 16383   # ETCToFilter output: T + carrier length - 1
FILTER_CUT = 4096        # Create_Filter's Array.Resize(F.Length - 4096)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def etc_to_filter(prms, swl=None, sample_rate=1000):
    """Pach_SP.ETCToFilter on the GPU: prms [8][T] or [n][8][T] band pressure envelopes at sample_rate
    Hz -> [T + 16383] (or [n][T + 16383])."""
    a = _f64(prms)
    one = a.ndim == 2
    a = a[None] if one else a
    if a.ndim != 3 or a.shape[1] != 8:
        raise ValueError("prms must be [8][T] or [n][8][T]")
    n, _, T = a.shape
    out = np.zeros((n, T + FILTER_LEN_ADD))
    check(_capi.lib().pach_etc_to_filter(dptr(a), n, T, dptr(_f64(swl)), int(sample_rate), dptr(out), out.size))
    return out[0] if one else out


def receiver_filters(pressure, energy=None, dir_pos=None, dir_neg=None, swl=None, sample_rate=1000):
    """Create_Filter of R receivers' scaled histograms (pressure/energy [R][8][T], dir_pos/dir_neg
    [R][3][8][T]) on the GPU: [R][7][T + 12287] with the directions, [R][1][T + 12287] without."""
    P = _f64(pressure)
    R, _, T = P.shape
    directional = dir_pos is not None and dir_neg is not None
    E, Dp, Dn = (_f64(energy), _f64(dir_pos), _f64(dir_neg)) if directional else (None, None, None)
    for a, shp in ((E, (R, 8, T)), (Dp, (R, 3, 8, T)), (Dn, (R, 3, 8, T))):
        if a is not None and a.shape != shp:
            raise ValueError(f"histogram shape {a.shape}, expected {shp}")
    out = np.zeros((R, 7 if directional else 1, T + FILTER_LEN_ADD - FILTER_CUT))
    check(_capi.lib().pach_receiver_filters(dptr(E), dptr(P), dptr(Dp), dptr(Dn), R, T, int(sample_rate),
                                            dptr(_f64(swl)), dptr(out), out.size))
    return out


def emit_directions(seed, ray_begin, n, n_sources, kind):
    out = np.zeros((n, 3))
    check(_capi.lib().pach_emit_directions(seed, ray_begin, n, n_sources, kind, dptr(out)))
    return out


def medium_properties(temp_c=20.0, hr=50.0, pa_hpa=1013.25, air_choice=0, edge=0):
    att = np.zeros(8)
    c, rho = C.c_double(), C.c_double()
    check(_capi.lib().pach_medium_properties(temp_c, hr, pa_hpa, air_choice, edge, dptr(att), C.byref(c), C.byref(rho)))
    return att, c.value, rho.value
