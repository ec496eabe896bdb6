"""GPU checks of the learned emission proposal: the tcgen05 GEMM, the network's loss and gradients
against the FP64 oracle, training, the device sampler's weights, the training capture, and the
unbiasedness and gain of proposal-driven tracing."""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import mlp_oracle as MO  # noqa: E402
from pachydermacoustic_universal_gb300 import proposal, rooms, tracer  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 160, 256), (300, 16, 640), (640, 256, 16),
                                   (1000, 48, 96), (130, 272, 48)])
def test_tensor_core_gemm(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    C = proposal.gemm(A, B)
    ref = MO.bf16(A) @ MO.bf16(B).T  # BF16 products are exact in FP32; only the sum order differs
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def _problem(rows=200, seed=7):
    rng = np.random.default_rng(seed)
    cond = np.concatenate([rng.uniform(1, 9, (rows, 3)), rng.uniform(1, 9, (rows, 3)),
                           np.zeros((rows, 3)), rng.uniform(8, 12, (rows, 3))], axis=1).astype(np.float32)
    target = rng.gamma(0.3, 1.0, (rows, MO.N_BINS))
    target /= target.sum(axis=1, keepdims=True)
    return cond, target.astype(np.float32)


def test_loss_and_gradient_match_oracle():
    net = proposal.ProposalNet(seed=11, max_rows=512)
    cond, target = _problem()
    net.set_data(cond, target)
    loss, g = net.loss_grad()
    p = net.params().astype(np.float64)
    bins = proposal.direction_bins()[0].astype(np.float64)
    ref_loss, ref_g = MO.loss_grad(p, cond, target, bins, emulate_bf16=True)
    assert loss == pytest.approx(ref_loss, rel=2e-3)
    offsets = np.cumsum([0] + [n * k + n for n, k in MO.LAYERS])
    for l, (n, k) in enumerate(MO.LAYERS):
        a, w_end, b_end = offsets[l], offsets[l] + n * k, offsets[l + 1]
        for lo, hi, what in ((a, w_end, "W"), (w_end, b_end, "b")):
            err = np.linalg.norm(g[lo:hi] - ref_g[lo:hi]) / np.linalg.norm(ref_g[lo:hi])
            assert err < 2e-2, (l, what, err)


def test_training_reduces_loss_and_forward_is_consistent():
    net = proposal.ProposalNet(seed=3, max_rows=512)
    rng = np.random.default_rng(9)
    rows = 256
    cond = np.concatenate([rng.uniform(1, 9, (rows, 3)), rng.uniform(1, 9, (rows, 3)),
                           np.zeros((rows, 3)), np.full((rows, 3), 10.0)], axis=1).astype(np.float32)
    # target: a cap of half-angle ~15 degrees around the source -> receiver direction
    dirs, om = MO.direction_bins()
    v = cond[:, 3:6] - cond[:, 0:3]
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    t = np.exp(20.0 * (v @ dirs.T - 1.0)) * om[None, :]
    t /= t.sum(axis=1, keepdims=True)
    net.set_data(cond, t.astype(np.float32))
    l0, _ = net.loss_grad(with_grad=False)
    curve = net.train(400, lr=2e-3)
    l1, _ = net.loss_grad(with_grad=False)
    assert np.all(np.isfinite(curve))
    assert l1 < l0 - 1.0, (l0, l1)
    assert l1 == pytest.approx(curve[-1], abs=0.2)
    # inference through the same kernels agrees with the oracle forward on the trained weights
    out = net.forward(cond[:16])
    ref, _ = MO.forward(net.params().astype(np.float64), cond[:16], emulate_bf16=True)
    assert np.abs(out - ref).max() < 2e-2 * max(1.0, np.abs(ref).max())
    # training resumes after an inference call
    net.train(5, lr=2e-3)


def test_sampler_weights_are_unbiased():
    rng = np.random.default_rng(4)
    raw = rng.normal(0, 1, (3, MO.N_OUT)).astype(np.float32)
    raw[:, 3::5] = rng.uniform(0, 4, (3, MO.N_LOBES))
    n = 400_000
    d, w = proposal.sample(raw, mix=0.3, seed=5, n=n)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    q = MO.mixture_density(raw, d, 0.3)
    assert np.allclose(w, 1.0 / (4 * math.pi) / q, rtol=2e-4)
    # E_q[w] = 1 and E_q[w f] = E_uniform[f] for a cap indicator
    se = w.std() / math.sqrt(n)
    assert abs(w.mean() - 1.0) < 5 * se + 1e-4
    axis = np.array([0.6, 0.0, 0.8])
    f = (d @ axis > math.cos(0.5)).astype(float)
    cap = (1 - math.cos(0.5)) / 2
    est = (w * f).mean()
    assert abs(est - cap) < 5 * (w * f).std() / math.sqrt(n)
    assert np.all(w <= 1.0 / 0.3 + 1e-3)   # the uniform component bounds every weight


def test_capture_accounts_for_every_detection():
    w = rooms.shoebox_c1()
    h, s = tracer.trace(w, rays=2000, seed=3, capture=True)
    cap = h["capture"].astype(np.float64)
    per_rec = cap.sum(axis=(1, 2))
    hist = h["energy"].sum(axis=(1, 2))  # unscaled
    assert np.allclose(per_rec, hist, rtol=1e-4)
    # capture does not change the histograms
    h2, _ = tracer.trace(w, rays=2000, seed=3)
    assert np.allclose(h2["energy"], h["energy"], rtol=1e-12, atol=0)
    # one emission direction for every primary: all capture lands in that direction's bin
    d = np.tile(np.array([[0.3, -0.5, 0.81]]), (500, 1))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    h3, _ = tracer.trace(w, rays=500, seed=3, capture=True, prim_dirs=d)
    b = proposal.direction_bin(d[0])
    c3 = h3["capture"].sum(axis=(0, 1))
    assert c3[b] > 0 and c3.sum() == pytest.approx(c3[b], rel=1e-6)


def test_learned_emission_is_unbiased():
    """Per-band total energy at each receiver with an arbitrary proposal matches uniform emission
    within the seed-to-seed spread (uniform emission on both sides: source kind 2)."""
    w = rooms.shoebox_c1()
    w.sources = [rooms.SourceSpec(s.origin, s.power_db, 2) for s in w.sources]
    rng = np.random.default_rng(8)
    raw = rng.normal(0, 1, (len(w.receivers), MO.N_OUT)).astype(np.float32)
    raw[:, 3::5] = rng.uniform(0, 3, (len(w.receivers), MO.N_LOBES))
    tot_u, tot_l = [], []
    for s in range(6):
        hu, _ = tracer.trace(w, rays=4000, seed=100 + s, scaled=True, oct_range=(3, 4))
        hl, _ = proposal.trace_learned(w, raw, mix=0.3, rays=4000, seed=200 + s, scaled=True, oct_range=(3, 4))
        tot_u.append(hu["energy"].sum(axis=2))
        tot_l.append(hl["energy"].sum(axis=2))
    tu, tl = np.array(tot_u), np.array(tot_l)
    for r in range(len(w.receivers)):
        for o in (3, 4):
            mu, ml = tu[:, r, o].mean(), tl[:, r, o].mean()
            se = math.sqrt(tu[:, r, o].var(ddof=1) / 6 + tl[:, r, o].var(ddof=1) / 6)
            assert abs(mu - ml) < 4 * se + 1e-3 * mu, (r, o, mu, ml, se)


def test_per_primary_capture_matches_bins():
    w = rooms.shoebox_c1()
    h1, _ = tracer.trace(w, rays=1500, seed=4, capture=1)
    h2, _ = tracer.trace(w, rays=1500, seed=4, capture=2)
    per = h2["capture"].astype(np.float64)            # [N][R][4]
    assert per.shape == (1500, len(w.receivers), 4)
    assert np.allclose(per.sum(axis=0), h1["capture"].astype(np.float64).sum(axis=2), rtol=1e-4)
    # each primary's energy lands in its emission-direction bin
    d = proposal.emission_directions(4, 0, 1500, len(w.sources), w.sources[0].kind)
    b = proposal.direction_bins_of(d)
    binned = np.zeros((len(w.receivers), 4, MO.N_BINS))
    for r in range(len(w.receivers)):
        for k in range(4):
            binned[r, k] = np.bincount(b, weights=per[:, r, k], minlength=MO.N_BINS)
    assert np.allclose(binned, h1["capture"], rtol=1e-3, atol=1e-9 * binned.max())
    t = proposal.capture_targets_l2(h2["capture"], d)
    assert t.shape == (len(w.receivers), MO.N_BINS) and np.allclose(t.sum(axis=1), 1.0, atol=1e-5)
