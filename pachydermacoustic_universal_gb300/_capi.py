"""ctypes binding of libpach_gpu.so (include/pach_gpu.h, include/pach_proposal.h).

The library is the product: there is no CPU fallback.  Loading fails loudly when the shared library
is missing and cannot be built, and every tracing entry point fails with PACH_ERR_NO_DEVICE when no
CUDA device is visible.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpach_gpu.so")
_lib = None

STATUS = {0: "PACH_OK", 1: "PACH_ERR_INVALID_ARGUMENT", 2: "PACH_ERR_OUT_OF_MEMORY", 3: "PACH_ERR_CUDA",
          4: "PACH_ERR_TIMEOUT", 5: "PACH_ERR_CANCELLED", 6: "PACH_ERR_BOUNDS", 7: "PACH_ERR_NOT_READY",
          8: "PACH_ERR_NO_DEVICE", 9: "PACH_ERR_GAVE_UP"}
RUN_STATE = {0: "RUNNING", 1: "STOPPED", 2: "FAILED", 3: "CANCELLED"}

MLP_IN, MLP_HIDDEN, MLP_LOBES, MLP_OUT = 12, 256, 32, 160   # include/pach_proposal.h
DIR_BINS, CAPTURE_WINDOWS = 1536, 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_fp = C.POINTER(C.c_float)


class SceneDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", _dp), ("n_polys", C.c_int32), ("poly_offsets", _ip),
                ("poly_indices", _ip), ("absorption", _dp), ("scattering", _dp), ("transmission", _dp),
                ("temp_c", C.c_double), ("rel_humidity", C.c_double), ("pressure_hpa", C.c_double),
                ("air_choice", C.c_int32), ("edge_correction", C.c_int32), ("bvh_leaf_max", C.c_int32),
                ("reserved1", C.c_int32)]


class SourceDesc(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("power_db", C.c_double * 8), ("kind", C.c_int32), ("reserved", C.c_int32)]


class ReceiverDesc(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("radius", C.c_double)]


class MapDesc(C.Structure):
    _fields_ = [("n_receivers", C.c_int32), ("time_1pt", C.c_int32), ("origins", _dp), ("increment", C.c_double),
                ("cutoff_ms", C.c_double), ("walk", C.c_int32), ("directional", C.c_int32)]


class TraceParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("ray_count", C.c_int64), ("ray_begin", C.c_int64), ("cutoff_length_m", C.c_double),
                ("oct_lo", C.c_int32), ("oct_hi", C.c_int32), ("is_order", C.c_int32), ("sample_rate", C.c_int32),
                ("hist_cotime_ms", C.c_double), ("pure_specular", C.c_int32), ("max_broadband_bounces", C.c_int32),
                ("max_segments_per_ray", C.c_int64), ("feed_batch", C.c_int64),
                ("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("wave_kilo_items", C.c_int32), ("ring_log2", C.c_int32),
                ("kernel_timing", C.c_int32), ("ray_sort", C.c_int32),
                ("traversal", C.c_int32), ("capture", C.c_int32),
                ("prim_dirs", _dp), ("prim_weights", _dp),
                ("proposal", C.POINTER(C.c_float)), ("n_proposal", C.c_int32), ("bvh_format", C.c_int32),
                ("proposal_mix", C.c_double), ("capture_edges_ms", C.c_double * 3), ("map", C.POINTER(MapDesc)),
                ("max_rays", C.c_int64)]


class RoomDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("sources", C.POINTER(SourceDesc)), ("n_sources", C.c_int32),
                ("n_receivers", C.c_int32), ("receivers", C.POINTER(ReceiverDesc)), ("ray_count", C.c_int64),
                ("cutoff_length_m", C.c_double)]


class TuneResult(C.Structure):
    _fields_ = [("wave_kilo_items", C.c_int32), ("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("traversal", C.c_int32), ("segments_per_s", C.c_double), ("tune_seconds", C.c_double),
                ("trials", C.c_int32), ("from_cache", C.c_int32)]


class Progress(C.Structure):
    _fields_ = [("state", C.c_int32), ("last_status", C.c_int32), ("rays_done", C.c_int64),
                ("rays_total", C.c_int64), ("end_traces", C.c_int64), ("segments", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("primaries", C.c_int64), ("segments", C.c_int64), ("segments_broadband", C.c_int64),
                ("segments_phase_b", C.c_int64), ("segments_phase_c", C.c_int64), ("octave_rays", C.c_int64),
                ("end_traces", C.c_int64), ("detections", C.c_int64), ("capped", C.c_int64),
                ("fp64_retests", C.c_int64), ("queue_overflows", C.c_int64), ("stack_spills", C.c_int64),
                ("lost_energy", C.c_double), ("initial_energy", C.c_double), ("percent_lost", C.c_double),
                ("h_oct", C.c_int32), ("bins", C.c_int32), ("cotime_s", C.c_double), ("sound_speed", C.c_double),
                ("rho_c", C.c_double), ("air_atten_db_per_m", C.c_double * 8), ("device_ms", C.c_double),
                ("trace_ms", C.c_double), ("shade_ms", C.c_double), ("broadband_ms", C.c_double),
                ("sort_ms", C.c_double),
                ("waves", C.c_int64), ("kernel_launches", C.c_int64), ("peak_live_rays", C.c_int64),
                ("bvh_nodes_visited", C.c_int64), ("tri_tests", C.c_int64),
                ("wall_ms", C.c_double), ("accel", C.c_int32 * 3), ("walk", C.c_int32),
                ("revolutions", C.c_int64), ("converged", C.c_int32), ("check_receivers", C.c_int32 * 2),
                ("reserved2", C.c_int32)]

    def to_dict(self):
        out = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            out[k] = list(v) if hasattr(v, "__len__") else v
        return out


# Every symbol include/pach_gpu.h declares (checked by the CPU test suite).
EXPORTS = ["pach_version", "pach_last_error", "pach_device_count", "pach_scene_create", "pach_scenes_create",
           "pach_scene_destroy",
           "pach_scene_info", "pach_trace_begin", "pach_batch_begin", "pach_autotune", "pach_direct_sound", "pach_trace_poll", "pach_trace_cancel", "pach_trace_wait",
           "pach_trace_get_histograms", "pach_trace_get_filters", "pach_etc_to_filter", "pach_receiver_filters",
           "pach_filters_workspace_bytes", "pach_filters_device", "pach_trace_get_stats", "pach_trace_get_map", "pach_trace_get_map_directions", "pach_map_parameters",
           "pach_etc_parameters",
           "pach_run_destroy", "pach_trace_run",
           "pach_trace_run_noalloc", "pach_convergence_replay", "pach_trace_specular_paths", "pach_scene_shoot_host", "pach_emit_directions", "pach_medium_properties", "pach_medium_attenuation_third_octave", "pach_math_schroeder",
           "pach_math_t_x", "pach_math_edt", "pach_math_clarity", "pach_math_definition", "pach_math_center_time",
           "pach_math_strength", "pach_math_sound_speed",
           # include/pach_proposal.h
           "pach_mlp_param_count", "pach_mlp_create", "pach_mlp_destroy", "pach_mlp_get_params", "pach_mlp_set_params",
           "pach_mlp_set_data", "pach_mlp_loss_grad", "pach_mlp_train", "pach_mlp_forward", "pach_mlp_gemm",
           "pach_direction_bins", "pach_direction_bin", "pach_proposal_sample", "pach_trace_get_capture"]


class PachError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def _declare(L):
    vp = C.c_void_p
    sig = {
        "pach_version": (C.c_char_p, []),
        "pach_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "pach_device_count": (C.c_int, []),
        "pach_scene_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(vp)]),
        "pach_scenes_create": (C.c_int, [C.POINTER(SceneDesc), C.c_int32, C.POINTER(vp), C.c_int32]),
        "pach_scene_destroy": (None, [vp]),
        "pach_scene_info": (C.c_int, [vp, _ip, _ip, _dp, _dp, _dp, _dp]),
        "pach_trace_begin": (C.c_int, [vp, C.POINTER(SourceDesc), C.c_int32, C.POINTER(ReceiverDesc), C.c_int32,
                                       C.POINTER(TraceParams), C.POINTER(vp)]),
        "pach_batch_begin": (C.c_int, [C.POINTER(RoomDesc), C.c_int32, C.POINTER(TraceParams), C.POINTER(vp)]),
        "pach_autotune": (C.c_int, [C.POINTER(RoomDesc), C.c_int32, C.POINTER(TraceParams), C.c_int64, C.c_char_p,
                                    C.c_int32, C.POINTER(TuneResult)]),
        "pach_direct_sound": (C.c_int, [vp, C.POINTER(SourceDesc), C.c_int32, C.POINTER(ReceiverDesc), C.c_int32,
                                        _ip, _dp, _dp]),
        "pach_trace_poll": (C.c_int, [vp, C.POINTER(Progress)]),
        "pach_trace_cancel": (C.c_int, [vp]),
        "pach_trace_wait": (C.c_int, [vp, C.c_int64]),
        "pach_trace_get_histograms": (C.c_int, [vp, C.c_int32, _dp, _dp, _dp, _dp, _dp, C.c_size_t]),
        "pach_trace_get_filters": (C.c_int, [vp, C.c_int32, _dp, _dp, C.c_size_t]),
        "pach_etc_to_filter": (C.c_int, [_dp, C.c_int32, C.c_int32, _dp, C.c_int32, _dp, C.c_size_t]),
        "pach_receiver_filters": (C.c_int, [_dp, _dp, _dp, _dp, C.c_int32, C.c_int32, C.c_int32, _dp, _dp, C.c_size_t]),
        "pach_filters_workspace_bytes": (C.c_size_t, [C.c_int32, C.c_int32]),
        "pach_filters_device": (C.c_int, [vp, vp, vp, vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _dp,
                                          C.c_int32, vp, vp, C.c_size_t, vp]),
        "pach_trace_get_stats": (C.c_int, [vp, C.POINTER(Stats)]),
        "pach_trace_get_map": (C.c_int, [vp, C.c_int32, _dp, _dp, _dp, _ip, C.c_size_t]),
        "pach_trace_get_map_directions": (C.c_int, [vp, C.c_int32, _dp, _dp, C.c_size_t]),
        "pach_map_parameters": (C.c_int, [vp, C.c_int32, C.c_int32, _dp, _dp, _dp, _dp, _dp]),
        "pach_etc_parameters": (C.c_int, [_dp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, _dp, _dp, _dp,
                                          _dp, _dp]),
        "pach_run_destroy": (None, [vp]),
        "pach_trace_run": (C.c_int, [vp, C.POINTER(SourceDesc), C.c_int32, C.POINTER(ReceiverDesc), C.c_int32,
                                     C.POINTER(TraceParams), C.c_int32, _dp, _dp, _dp, _dp, _dp, C.c_size_t,
                                     C.POINTER(Stats)]),
        "pach_trace_run_noalloc": (C.c_int, [vp, C.POINTER(SourceDesc), C.c_int32, C.POINTER(ReceiverDesc), C.c_int32,
                                             C.POINTER(TraceParams), vp, vp, vp, vp, vp, vp, C.POINTER(Stats)]),
        "pach_convergence_replay": (C.c_int, [_dp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                              C.c_double, _ip, C.POINTER(C.c_int64)]),
        "pach_trace_specular_paths": (C.c_int, [vp, C.c_int32, _dp, _dp, C.c_int32, _ip, _dp, _dp]),
        "pach_scene_shoot_host": (C.c_int, [C.POINTER(SceneDesc), C.c_int32, _dp, _dp, _ip, _dp]),
        "pach_emit_directions": (C.c_int, [C.c_uint64, C.c_int64, C.c_int32, C.c_int32, C.c_int32, _dp]),
        "pach_medium_properties": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, _dp, _dp, _dp]),
        "pach_medium_attenuation_third_octave": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                                           _dp, _dp]),
        "pach_math_schroeder": (C.c_int, [_dp, C.c_int32, _dp]),
        "pach_math_t_x": (C.c_double, [_dp, C.c_int32, C.c_int32, C.c_int32]),
        "pach_math_edt": (C.c_double, [_dp, C.c_int32, C.c_int32]),
        "pach_math_clarity": (C.c_double, [_dp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32]),
        "pach_math_definition": (C.c_double, [_dp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32]),
        "pach_math_center_time": (C.c_double, [_dp, C.c_int32, C.c_int32, C.c_double, C.c_int32]),
        "pach_math_strength": (C.c_double, [_dp, C.c_int32, C.c_double, C.c_int32]),
        "pach_math_sound_speed": (C.c_double, [C.c_double]),
        "pach_mlp_param_count": (C.c_int64, []),
        "pach_mlp_create": (C.c_int, [C.c_uint64, C.c_int32, C.POINTER(vp)]),
        "pach_mlp_destroy": (None, [vp]),
        "pach_mlp_get_params": (C.c_int, [vp, _fp, C.c_int64]),
        "pach_mlp_set_params": (C.c_int, [vp, _fp, C.c_int64]),
        "pach_mlp_set_data": (C.c_int, [vp, _fp, _fp, C.c_int32]),
        "pach_mlp_loss_grad": (C.c_int, [vp, _fp, _fp]),
        "pach_mlp_train": (C.c_int, [vp, C.c_int32, C.c_float, C.c_float, _fp]),
        "pach_mlp_forward": (C.c_int, [vp, _fp, C.c_int32, _fp]),
        "pach_mlp_gemm": (C.c_int, [_fp, _fp, C.c_int32, C.c_int32, C.c_int32, _fp]),
        "pach_direction_bins": (C.c_int, [_fp, _fp, C.c_int32]),
        "pach_direction_bin": (C.c_int32, [C.c_double, C.c_double, C.c_double]),
        "pach_proposal_sample": (C.c_int, [_fp, C.c_int32, C.c_double, C.c_uint64, C.c_int64, C.c_int32, _fp, _fp]),
        "pach_trace_get_capture": (C.c_int, [vp, _fp, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib():
    """Load libpach_gpu.so, building it with nvcc when it is missing.  Raises if neither works."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: the CUDA engine was not built")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib().pach_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def check(status):
    if status != 0:
        raise PachError(status, last_error())


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def fptr(a):
    return a.ctypes.data_as(_fp) if a is not None else None


def device_count() -> int:
    return int(lib().pach_device_count())
