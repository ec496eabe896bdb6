"""Learned emission proposal (include/pach_proposal.h).

No counterpart in the reference, whose sources always emit uniformly (GeodesicSource and
RandomSource, Pachyderm_Acoustic_Universal/Classes_Sources.cs:256-265, 390-403).  Here:

* ``ProposalNet``   -- the 12 -> 3 x 256 (GELU) -> 160 network, trained and run by the library's own
  BF16 tensor-core kernels (pach_mlp_*): a mixture of 32 von Mises-Fisher lobes over emission
  directions, conditioned on source xyz, receiver xyz and the room bounds.
* ``collect``       -- training data from the tracer itself: uniform-emission runs with capture on,
  turned into one target distribution over the 1536 emission-direction bins per receiver.
* ``trace_learned`` -- a run that emits from the defensive mixture of the learned lobes and uniform
  emission, weighting each primary by (1 / 4 pi) / q so the histograms stay unbiased.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi, tracer
from ._capi import check, fptr

N_IN, N_OUT, N_LOBES = _capi.MLP_IN, _capi.MLP_OUT, _capi.MLP_LOBES
N_BINS, N_WINDOWS = _capi.DIR_BINS, _capi.CAPTURE_WINDOWS


def param_count() -> int:
    return int(_capi.lib().pach_mlp_param_count())


class ProposalNet:
    """The proposal network on the GPU (pach_mlp)."""

    def __init__(self, seed: int = 1, max_rows: int = 4096):
        h = C.c_void_p()
        check(_capi.lib().pach_mlp_create(int(seed), int(max_rows), C.byref(h)))
        self.handle = h
        self.max_rows = int(max_rows)

    def params(self) -> np.ndarray:
        p = np.zeros(param_count(), dtype=np.float32)
        check(_capi.lib().pach_mlp_get_params(self.handle, fptr(p), p.size))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(_capi.lib().pach_mlp_set_params(self.handle, fptr(p), p.size))

    def set_data(self, cond, target) -> None:
        cond = np.ascontiguousarray(cond, dtype=np.float32).reshape(-1, N_IN)
        target = np.ascontiguousarray(target, dtype=np.float32).reshape(-1, N_BINS)
        if cond.shape[0] != target.shape[0]:
            raise ValueError("cond and target need the same number of rows")
        self._data = (cond, target)
        check(_capi.lib().pach_mlp_set_data(self.handle, fptr(cond), fptr(target), cond.shape[0]))

    def loss_grad(self, with_grad: bool = True):
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(param_count(), dtype=np.float32) if with_grad else None
        check(_capi.lib().pach_mlp_loss_grad(self.handle, fptr(loss), fptr(g)))
        return float(loss[0]), g

    def train(self, steps: int, lr: float = 1e-3, weight_decay: float = 0.0) -> np.ndarray:
        curve = np.zeros(max(1, int(steps)), dtype=np.float32)
        check(_capi.lib().pach_mlp_train(self.handle, int(steps), float(lr), float(weight_decay), fptr(curve)))
        return curve[: int(steps)]

    def forward(self, cond) -> np.ndarray:
        cond = np.ascontiguousarray(cond, dtype=np.float32).reshape(-1, N_IN)
        out = np.zeros((cond.shape[0], N_OUT), dtype=np.float32)
        check(_capi.lib().pach_mlp_forward(self.handle, fptr(cond), cond.shape[0], fptr(out)))
        return out

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().pach_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gemm(A, B) -> np.ndarray:
    """C = bf16(A) . bf16(B)^T through the tensor-core GEMM kernel (diagnostic)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M, K = A.shape
    N = B.shape[0]
    out = np.zeros((M, N), dtype=np.float32)
    check(_capi.lib().pach_mlp_gemm(fptr(A), fptr(B), M, N, K, fptr(out)))
    return out


def direction_bins():
    """Centre directions [1536][3] and solid angles [1536] of the emission-direction bins."""
    d = np.zeros((N_BINS, 3), dtype=np.float32)
    w = np.zeros(N_BINS, dtype=np.float32)
    check(_capi.lib().pach_direction_bins(fptr(d), fptr(w), N_BINS))
    return d, w


def direction_bin(d) -> int:
    return int(_capi.lib().pach_direction_bin(float(d[0]), float(d[1]), float(d[2])))


def condition(workload, receiver: int, source: int = 0) -> np.ndarray:
    lo, hi = workload.scene.bounds()
    s = workload.sources[source].origin
    r = workload.receivers[receiver].origin
    return np.concatenate([np.asarray(s, float), np.asarray(r, float), lo, hi]).astype(np.float32)


def conditions(workload, source: int = 0) -> np.ndarray:
    return np.stack([condition(workload, k, source) for k in range(len(workload.receivers))])


def capture_targets(capture) -> np.ndarray:
    """[R][4][1536] captured energy -> [R][1536] targets: each window's energy share per bin, summed
    over the windows that received energy, normalised to 1."""
    cap = np.asarray(capture, dtype=np.float64)
    tot = cap.sum(axis=2, keepdims=True)
    share = np.divide(cap, tot, out=np.zeros_like(cap), where=tot > 0)
    t = share.sum(axis=1)
    s = t.sum(axis=1, keepdims=True)
    t = np.divide(t, s, out=np.full_like(t, 1.0 / N_BINS), where=s > 0)
    return t.astype(np.float32)


def direction_bins_of(d) -> np.ndarray:
    """Bins of directions d [n][3] (the rule of pach_direction_bin, vectorised)."""
    d = np.asarray(d, dtype=np.float32).reshape(-1, 3)
    a = np.abs(d)
    major = np.where((a[:, 0] >= a[:, 1]) & (a[:, 0] >= a[:, 2]), 0, np.where(a[:, 1] >= a[:, 2], 1, 2))
    m = a[np.arange(d.shape[0]), major]
    sign = d[np.arange(d.shape[0]), major] > 0
    face = 2 * major + np.where(sign, 0, 1)
    ua = np.where(major == 0, 1, 0)          # u: the first of the two other axes (x, y, z order)
    va = np.where(major == 2, 1, 2)          # v: the second
    u = d[np.arange(d.shape[0]), ua] / m
    v = d[np.arange(d.shape[0]), va] / m
    i = np.clip(((u + np.float32(1)) * np.float32(8)).astype(np.int64), 0, 15)
    j = np.clip(((v + np.float32(1)) * np.float32(8)).astype(np.int64), 0, 15)
    return (face * 256 + j * 16 + i).astype(np.int64)


def capture_targets_l2(per_prim, dirs) -> np.ndarray:
    """[N][R][4] per-primary captured energy and the primaries' emission directions [N][3] ->
    [R][1536] targets proportional to sqrt(E[sum_w (e_w / mean e_w)^2 | bin]) x bin solid angle: the
    proposal that minimises the summed relative variance of the windows' energies (the optimal
    importance density for several integrands sharing one sample is proportional to the root of their
    summed squared relative contributions)."""
    e = np.asarray(per_prim, dtype=np.float64)
    mean = e.mean(axis=0)                                   # [R][W]
    rel = np.divide(e, mean[None], out=np.zeros_like(e), where=mean[None] > 0)
    q = (rel ** 2).sum(axis=2)                              # [N][R]
    b = direction_bins_of(dirs)
    cnt = np.bincount(b, minlength=N_BINS).astype(np.float64)
    _, om = direction_bins()
    out = np.zeros((e.shape[1], N_BINS))
    for r in range(e.shape[1]):
        s2 = np.bincount(b, weights=q[:, r], minlength=N_BINS)
        m2 = np.divide(s2, cnt, out=np.zeros(N_BINS), where=cnt > 0)
        t = np.sqrt(m2) * om
        out[r] = t / t.sum() if t.sum() > 0 else 1.0 / N_BINS
    return out.astype(np.float32)


def emission_directions(seed: int, ray_begin: int, n: int, n_sources: int, kind: int) -> np.ndarray:
    """The emission directions the tracer draws for primaries ray_begin .. ray_begin + n - 1."""
    out = np.zeros((n, 3))
    check(_capi.lib().pach_emit_directions(int(seed), int(ray_begin), int(n), int(n_sources), int(kind),
                                           _capi.dptr(out)))
    return out


def collect(workloads, rays: int, seed: int = 1, target: str = "linear", **kw):
    """Trace each workload with uniform emission and capture on; returns (cond [n][12], target [n][1536],
    wall seconds of the traces).  target "l2": per-primary capture and capture_targets_l2; "linear":
    per-bin capture and capture_targets."""
    import time
    conds, targets = [], []
    t0 = time.perf_counter()
    for i, w in enumerate(workloads):
        if target == "l2":
            h, _ = tracer.trace(w, rays=rays, seed=seed + i, capture=2, **kw)
            d = emission_directions(seed + i, 0, rays, len(w.sources), w.sources[0].kind)
            targets.append(capture_targets_l2(h["capture"], d))
        else:
            h, _ = tracer.trace(w, rays=rays, seed=seed + i, capture=1, **kw)
            targets.append(capture_targets(h["capture"]))
        conds.append(conditions(w))
    return np.concatenate(conds), np.concatenate(targets), time.perf_counter() - t0


def sample(raw, mix: float = 0.3, seed: int = 1, ray_begin: int = 0, n: int = 1024):
    """Directions [n][3] and weights [n] the device sampler draws from the defensive mixture."""
    raw = np.ascontiguousarray(raw, dtype=np.float32).reshape(-1, N_OUT)
    d = np.zeros((n, 3), dtype=np.float32)
    w = np.zeros(n, dtype=np.float32)
    check(_capi.lib().pach_proposal_sample(fptr(raw), raw.shape[0], float(mix), int(seed), int(ray_begin), int(n),
                                           fptr(d), fptr(w)))
    return d, w


def trace_learned(workload, raw, mix: float = 0.3, **kw):
    """Trace with emission from the learned lobes raw [R][160] (one mixture per receiver of the
    workload) mixed with uniform emission (probability mix)."""
    return tracer.trace(workload, proposal=np.asarray(raw, dtype=np.float32), proposal_mix=mix, **kw)
