"""ctypes wrapper of the CPU FP64 oracle (liboracle built from pach_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by the test suite, by the smoke check and by the CPU-baseline
leg of the benchmark, always as the checker.  The product never imports this module.
Parity is unpinned against the reference itself; see pach_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpach_oracle.so")
_lib = None


class OrcScene(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", C.POINTER(C.c_double)),
                ("n_polys", C.c_int32), ("poly_offsets", C.POINTER(C.c_int32)),
                ("poly_indices", C.POINTER(C.c_int32)),
                ("absorption", C.POINTER(C.c_double)), ("scattering", C.POINTER(C.c_double)),
                ("transmission", C.POINTER(C.c_double)),
                ("temp_c", C.c_double), ("rel_humidity", C.c_double), ("pressure_hpa", C.c_double),
                ("air_choice", C.c_int32), ("edge_correction", C.c_int32)]


class OrcSource(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("power_db", C.c_double * 8), ("kind", C.c_int32), ("pad", C.c_int32)]


class OrcReceiver(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("radius", C.c_double)]


class OrcParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("cutoff_length_m", C.c_double), ("oct_lo", C.c_int32), ("oct_hi", C.c_int32),
                ("is_order", C.c_int32), ("sample_rate", C.c_int32), ("hist_cotime_ms", C.c_double),
                ("pure_specular", C.c_int32), ("grid_domain", C.c_int32), ("brute_force", C.c_int32),
                ("max_broadband_bounces", C.c_int32), ("max_segments_per_ray", C.c_int64)]


class OrcStats(C.Structure):
    _fields_ = [("primaries", C.c_int64), ("segments", C.c_int64), ("segments_broadband", C.c_int64),
                ("segments_phase_b", C.c_int64), ("segments_phase_c", C.c_int64), ("octave_rays", C.c_int64),
                ("end_traces", C.c_int64), ("detections", C.c_int64), ("capped", C.c_int64),
                ("cells_visited", C.c_int64), ("tri_tests", C.c_int64), ("lost_energy", C.c_double), ("initial_energy", C.c_double), ("h_oct", C.c_int32),
                ("bins", C.c_int32), ("cotime_s", C.c_double), ("sound_speed", C.c_double), ("rho_c", C.c_double),
                ("air_atten_db_per_m", C.c_double * 8)]


class OrcMap(C.Structure):
    _fields_ = [("n_receivers", C.c_int32), ("time_1pt", C.c_int32), ("origins", C.POINTER(C.c_double)),
                ("increment", C.c_double), ("cutoff_ms", C.c_double), ("walk", C.c_int32), ("directional", C.c_int32)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ only)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "pach_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.orc_trace_ex.restype = C.c_int
        L.orc_trace_ex.argtypes = [C.POINTER(OrcScene), C.c_int32, C.POINTER(OrcSource), C.c_int32,
                                   C.POINTER(OrcReceiver), C.POINTER(OrcParams), C.c_int64, C.c_int64,
                                   C.c_int32, dp, dp, dp, dp, dp, dp, dp, C.POINTER(OrcStats)]
        L.orc_trace_map.restype = C.c_int
        L.orc_trace_map.argtypes = [C.POINTER(OrcScene), C.c_int32, C.POINTER(OrcSource), C.c_int32,
                                    C.POINTER(OrcReceiver), C.POINTER(OrcMap), C.POINTER(OrcParams), C.c_int64,
                                    C.c_int64, C.c_int32, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp,
                                    C.POINTER(OrcStats)]
        L.orc_map_directions.restype = C.c_int
        L.orc_map_directions.argtypes = [dp, dp, C.c_size_t]
        L.orc_specular_paths.restype = C.c_int
        L.orc_specular_paths.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.c_int32, dp, dp, C.c_int32,
                                         C.POINTER(C.c_int32), dp, dp]
        L.orc_shoot.restype = C.c_int
        L.orc_shoot.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, dp, dp, C.POINTER(C.c_int32), dp, dp]
        L.orc_medium.restype = None
        L.orc_medium.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, dp, dp, dp]
        L.orc_philox.restype = None
        L.orc_philox.argtypes = [C.c_uint32] * 6 + [C.POINTER(C.c_uint32)]
        L.orc_emit_direction.restype = None
        L.orc_emit_direction.argtypes = [C.c_uint64, C.c_int64, C.c_int32, C.c_int32, dp]
        L.orc_schroeder.restype = None
        L.orc_schroeder.argtypes = [dp, C.c_int32, dp]
        L.orc_t_x.restype = C.c_double
        L.orc_t_x.argtypes = [dp, C.c_int32, C.c_int32, C.c_int32]
        L.orc_edt.restype = C.c_double
        L.orc_edt.argtypes = [dp, C.c_int32, C.c_int32]
        for name in ("orc_clarity", "orc_definition"):
            f = getattr(L, name)
            f.restype = C.c_double
            f.argtypes = [dp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32]
        L.orc_center_time.restype = C.c_double
        L.orc_center_time.argtypes = [dp, C.c_int32, C.c_int32, C.c_double, C.c_int32]
        L.orc_strength.restype = C.c_double
        L.orc_strength.argtypes = [dp, C.c_int32, C.c_double, C.c_int32]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class _SceneHolder:
    """Keeps the numpy arrays alive while the C struct points at them."""

    def __init__(self, scene):
        self.v = np.ascontiguousarray(scene.vertices, dtype=np.float64).reshape(-1)
        self.offs = np.ascontiguousarray(scene.poly_offsets, dtype=np.int32)
        self.idx = np.ascontiguousarray(scene.poly_indices, dtype=np.int32)
        self.a = np.ascontiguousarray(scene.absorption, dtype=np.float64).reshape(-1)
        self.s = np.ascontiguousarray(scene.scattering, dtype=np.float64).reshape(-1)
        self.t = np.ascontiguousarray(scene.transmission, dtype=np.float64).reshape(-1)
        self.desc = OrcScene(self.v.size // 3, _dp(self.v), self.offs.size - 1,
                             self.offs.ctypes.data_as(C.POINTER(C.c_int32)),
                             self.idx.ctypes.data_as(C.POINTER(C.c_int32)),
                             _dp(self.a), _dp(self.s), _dp(self.t), scene.temp_c, scene.rel_humidity,
                             scene.pressure_hpa, scene.air_choice, scene.edge_correction)


def medium(temp_c=20.0, hr=50.0, pa_hpa=1013.25, air_choice=0, edge=0):
    att = np.zeros(8)
    c = C.c_double()
    rho = C.c_double()
    lib().orc_medium(temp_c, hr, pa_hpa, air_choice, edge, _dp(att), C.byref(c), C.byref(rho))
    return att, c.value, rho.value


def philox(c0, c1, c2, c3, k0, k1):
    out = (C.c_uint32 * 4)()
    lib().orc_philox(c0, c1, c2, c3, k0, k1, out)
    return list(out)


def emit_direction(seed, ray, n_src, kind):
    d = np.zeros(3)
    lib().orc_emit_direction(seed, ray, n_src, kind, _dp(d))
    return d


def trace(workload, *, seed=1, rays=None, ray_begin=0, threads=0, pure_specular=False, is_order=-1,
          grid_domain=7, brute_force=False, oct_range=(0, 7), prim_dirs=None, prim_weights=None,
          max_broadband_bounces=0, max_segments_per_ray=0, map_receivers=None):
    """Trace primaries [ray_begin, ray_begin+rays) of a rooms.Workload.  Returns RAW histogram sums
    (energy, pressure, dir_pos, dir_neg, analysis) and a stats dict.  map_receivers (an object with
    origins [M][3], increment, cutoff_ms, time_1pt, walk) adds map_energy / map_pressure [M][8][Tm] and
    map_direct [M] (PachMapReceiver)."""
    L = lib()
    sh = _SceneHolder(workload.scene)
    ns = len(workload.sources)
    srcs = (OrcSource * ns)()
    for i, s in enumerate(workload.sources):
        srcs[i].origin[:] = list(s.origin)
        srcs[i].power_db[:] = list(s.power_db)
        srcs[i].kind = s.kind
    nr = len(workload.receivers)
    recs = (OrcReceiver * max(nr, 1))()
    for i, r in enumerate(workload.receivers):
        recs[i].origin[:] = list(r.origin)
        recs[i].radius = r.radius
    n = workload.rays if rays is None else rays
    p = OrcParams(seed, workload.cutoff_length_m, oct_range[0], oct_range[1], is_order, workload.sample_rate,
                  workload.cutoff_s * 1000.0, int(pure_specular), grid_domain, int(brute_force),
                  max_broadband_bounces, max_segments_per_ray)
    T = int(workload.sample_rate * workload.cutoff_s)
    E = np.zeros((nr, 8, T))
    P = np.zeros((nr, 8, T))
    Dp = np.zeros((nr, 3, 8, T))
    Dn = np.zeros((nr, 3, 8, T))
    An = np.zeros((nr, 3, 8, T))
    st = OrcStats()
    pd = np.ascontiguousarray(prim_dirs, dtype=np.float64) if prim_dirs is not None else None
    pw = np.ascontiguousarray(prim_weights, dtype=np.float64) if prim_weights is not None else None
    out = {"energy": E, "pressure": P, "dir_pos": Dp, "dir_neg": Dn, "analysis": An}
    mdesc, mE, mP, mD = None, None, None, None
    if map_receivers is not None:
        m = map_receivers
        morg = np.ascontiguousarray(m.origins, dtype=np.float64).reshape(-1)
        M = morg.size // 3
        Tm = 1 if m.time_1pt else int(float(m.cutoff_ms) / 1000.0 * 1000.0)
        mdesc = OrcMap(M, int(bool(m.time_1pt)), _dp(morg), float(m.increment), float(m.cutoff_ms), int(m.walk),
                       int(bool(getattr(m, "directional", False))))
        mE, mP, mD = np.zeros((M, 8, Tm)), np.zeros((M, 8, Tm)), np.zeros(M)
        out.update(map_energy=mE, map_pressure=mP, map_direct=mD)
    rc = L.orc_trace_map(C.byref(sh.desc), ns, srcs, nr, recs, C.byref(mdesc) if mdesc is not None else None,
                         C.byref(p), ray_begin, ray_begin + n, threads, _dp(pd), _dp(pw), _dp(E), _dp(P), _dp(Dp),
                         _dp(Dn), _dp(An), _dp(mE), _dp(mP), _dp(mD), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"orc_trace failed ({rc})")
    if mdesc is not None and mdesc.directional:
        Dp, Dn = np.zeros((M, 3, 8, Tm)), np.zeros((M, 3, 8, Tm))
        if not L.orc_map_directions(_dp(Dp), _dp(Dn), Dp.size):
            raise RuntimeError("orc_map_directions: no direction histograms")
        out.update(map_dir_pos=Dp, map_dir_neg=Dn)
    stats = {k: getattr(st, k) for k, _ in OrcStats._fields_}
    stats["air_atten_db_per_m"] = list(st.air_atten_db_per_m)
    return out, stats


def specular_paths(scene, origins, dirs, max_bounces, grid_domain=7, brute_force=False):
    L = lib()
    sh = _SceneHolder(scene)
    o = np.ascontiguousarray(origins, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.float64)
    n = o.shape[0]
    poly = np.zeros((n, max_bounces), dtype=np.int32)
    t = np.zeros((n, max_bounces))
    pts = np.zeros((n, max_bounces, 3))
    L.orc_specular_paths(C.byref(sh.desc), grid_domain, int(brute_force), n, _dp(o), _dp(d), max_bounces,
                         poly.ctypes.data_as(C.POINTER(C.c_int32)), _dp(t), _dp(pts))
    return poly, t, pts


def shoot(scene, o, d, grid_domain=7, brute_force=False):
    L = lib()
    sh = _SceneHolder(scene)
    o = np.ascontiguousarray(o, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    poly = C.c_int32()
    t = C.c_double()
    hit = np.zeros(3)
    L.orc_shoot(C.byref(sh.desc), grid_domain, int(brute_force), _dp(o), _dp(d), C.byref(poly), C.byref(t), _dp(hit))
    return poly.value, t.value, hit


# --- room-acoustic parameters (Classes_Math.cs) ---
def schroeder(etc):
    e = np.ascontiguousarray(etc, dtype=np.float64)
    out = np.zeros_like(e)
    lib().orc_schroeder(_dp(e), e.size, _dp(out))
    return out


def t_x(sch, depth=30, fs=1000):
    s = np.ascontiguousarray(sch, dtype=np.float64)
    return lib().orc_t_x(_dp(s), s.size, depth, fs)


def edt(sch, fs=1000):
    s = np.ascontiguousarray(sch, dtype=np.float64)
    return lib().orc_edt(_dp(s), s.size, fs)


def clarity(etc, fs=1000.0, seconds=0.08, start=0.0, pressure=False):
    e = np.ascontiguousarray(etc, dtype=np.float64)
    return lib().orc_clarity(_dp(e), e.size, fs, seconds, start, int(pressure))


def definition(etc, fs=1000.0, seconds=0.05, start=0.0, pressure=False):
    e = np.ascontiguousarray(etc, dtype=np.float64)
    return lib().orc_definition(_dp(e), e.size, fs, seconds, start, int(pressure))


def center_time(etc, fs=1000, direct=0.0, pressure=False):
    e = np.ascontiguousarray(etc, dtype=np.float64)
    return lib().orc_center_time(_dp(e), e.size, fs, direct, int(pressure))


def strength(etc, swl, pressure=False):
    e = np.ascontiguousarray(etc, dtype=np.float64)
    return lib().orc_strength(_dp(e), e.size, swl, int(pressure))


def direct_sound(workload, grid_domain=7):
    """Direct_Sound validity and energy per (receiver, source) (orc_direct): valid [R][S], distance
    [R][S], energy [R][S][8]."""
    L = lib()
    if not hasattr(L.orc_direct, "_declared"):
        L.orc_direct.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.POINTER(OrcSource), C.c_int32,
                                 C.POINTER(OrcReceiver), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.orc_direct.restype = C.c_int
        L.orc_direct._declared = True
    sh = _SceneHolder(workload.scene)
    ns, nr = len(workload.sources), len(workload.receivers)
    srcs = (OrcSource * ns)()
    for i, s in enumerate(workload.sources):
        srcs[i].origin[:] = list(s.origin)
        srcs[i].power_db[:] = list(s.power_db)
        srcs[i].kind = s.kind
    recs = (OrcReceiver * max(nr, 1))()
    for i, r in enumerate(workload.receivers):
        recs[i].origin[:] = list(r.origin)
        recs[i].radius = r.radius
    valid = np.zeros((nr, ns), dtype=np.int32)
    dist = np.zeros((nr, ns))
    energy = np.zeros((nr, ns, 8))
    L.orc_direct(C.byref(sh.desc), grid_domain, ns, srcs, nr, recs, valid.ctypes.data_as(C.POINTER(C.c_int32)),
                 _dp(dist), _dp(energy))
    return valid, dist, energy
