"""CPU checks of the learned-proposal oracle (oracle/mlp_oracle.py) and of the host-side pieces of the
proposal path: the oracle's analytic gradients against finite differences in FP64, its direction bins
against the library's, and the capture-target reduction."""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import mlp_oracle as MO  # noqa: E402
from pachydermacoustic_universal_gb300 import proposal  # noqa: E402


def _problem(seed=3, rows=3):
    rng = np.random.default_rng(seed)
    p = np.zeros(MO.param_count())
    i = 0
    for n, k in MO.LAYERS:
        p[i:i + n * k] = rng.uniform(-1, 1, n * k) * math.sqrt(3.0 / k)
        i += n * k
        p[i:i + n] = rng.normal(0, 0.1, n)
        i += n
    cond = rng.uniform(0, 10, (rows, MO.N_IN))
    target = rng.gamma(0.3, 1.0, (rows, MO.N_BINS))
    target /= target.sum(axis=1, keepdims=True)
    return p, cond, target


def test_row_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    bins = MO.direction_bins()[0]
    out = rng.normal(0, 1, MO.N_OUT)
    out[3::5] = rng.uniform(-1, 3, MO.N_LOBES)   # log kappa inside the clamp
    target = rng.gamma(0.3, 1.0, MO.N_BINS)
    target /= target.sum()
    _, g = MO.row_loss_grad(out, target, bins)
    h = 1e-6
    for j in rng.choice(MO.N_OUT, 40, replace=False):
        e = np.zeros(MO.N_OUT)
        e[j] = h
        fd = (MO.row_loss_grad(out + e, target, bins)[0] - MO.row_loss_grad(out - e, target, bins)[0]) / (2 * h)
        assert g[j] == pytest.approx(fd, rel=1e-5, abs=1e-8), j


def test_network_gradient_matches_finite_differences():
    p, cond, target = _problem()
    bins = MO.direction_bins()[0]
    _, g = MO.loss_grad(p, cond, target, bins, emulate_bf16=False)
    rng = np.random.default_rng(1)
    h = 1e-5
    # directional derivatives along random directions, and single coordinates in every layer
    for _ in range(3):
        v = rng.normal(size=p.size)
        v /= np.linalg.norm(v)
        fd = (MO.loss_grad(p + h * v, cond, target, bins, False)[0] -
              MO.loss_grad(p - h * v, cond, target, bins, False)[0]) / (2 * h)
        assert g @ v == pytest.approx(fd, rel=1e-5)
    offsets = np.cumsum([0] + [n * k + n for n, k in MO.LAYERS])
    for l in range(4):
        for j in rng.integers(offsets[l], offsets[l + 1], 3):
            e = np.zeros(p.size)
            e[j] = h
            fd = (MO.loss_grad(p + e, cond, target, bins, False)[0] -
                  MO.loss_grad(p - e, cond, target, bins, False)[0]) / (2 * h)
            assert g[j] == pytest.approx(fd, rel=1e-4, abs=1e-9), (l, j)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-5, 65504.0, 1.0 + 2 ** -8])
    r = MO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0                 # 1 + 2^-8 is a tie: to even (1.0)
    assert r[2] == 1.0078125                            # above the tie: up
    assert r[5] == 1.0
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_direction_bins_match_library():
    d, om = MO.direction_bins()
    ld, lom = proposal.direction_bins()
    assert np.allclose(d, ld, atol=1e-6)
    assert np.allclose(om, lom, rtol=1e-5)
    assert om.sum() == pytest.approx(4 * math.pi, rel=1e-9)
    rng = np.random.default_rng(5)
    v = rng.normal(size=(2000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for x in v:
        assert proposal.direction_bin(x) == MO.direction_bin(x)
    # every bin centre falls in its own bin
    for b in range(0, MO.N_BINS, 7):
        assert MO.direction_bin(d[b]) == b


def test_capture_targets():
    cap = np.zeros((2, 4, MO.N_BINS), dtype=np.float32)
    cap[0, 0, 10] = 3.0
    cap[0, 0, 11] = 1.0
    cap[0, 2, 500] = 1e-6
    t = proposal.capture_targets(cap)
    assert t.shape == (2, MO.N_BINS)
    # window 0 splits 3:1 between bins 10 and 11, window 2 puts its whole share on bin 500
    assert t[0, 10] == pytest.approx(0.375) and t[0, 11] == pytest.approx(0.125) and t[0, 500] == pytest.approx(0.5)
    assert np.allclose(t[1], 1.0 / MO.N_BINS)         # nothing captured: uniform


def test_mixture_density_normalised():
    rng = np.random.default_rng(2)
    out = rng.normal(0, 1, (2, MO.N_OUT))
    out[:, 3::5] = rng.uniform(-2, 4, (2, MO.N_LOBES))
    d, om = MO.direction_bins()
    # fine quadrature: each bin split into 8 x 8 sub-cells is unnecessary for smooth lobes; the
    # bin-centre rule is accurate to ~1 % for kappa <= 55
    q = MO.mixture_density(out, d, 0.3)
    assert (q * om).sum() == pytest.approx(1.0, rel=2e-2)


def test_vectorised_direction_bins_match_library():
    rng = np.random.default_rng(11)
    v = rng.normal(size=(3000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v[:6] = [[1, 0, 0], [0, -1, 0], [0, 0, 1], [0.5, 0.5, 0.5], [-0.3, 0.3, -0.3], [0, 1e-9, -1]]
    b = proposal.direction_bins_of(v)
    assert all(int(b[i]) == proposal.direction_bin(v[i]) for i in range(len(v)))


def test_second_moment_targets():
    # two primaries in bin A each deliver the window-0 mean x 2 -> relative 2; bin B nothing
    d, _ = MO.direction_bins()
    dirs = np.stack([d[10], d[10], d[20], d[20]])
    cap = np.zeros((4, 1, 4), dtype=np.float32)
    cap[0, 0, 0] = cap[1, 0, 0] = 1.0
    t = proposal.capture_targets_l2(cap, dirs)
    assert t.shape == (1, MO.N_BINS)
    assert t[0, 10] == pytest.approx(1.0) and t[0, 20] == 0.0
