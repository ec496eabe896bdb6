"""Convergence mode's checks (SplitRayTracer with rayCount < 1; TaskAll:783-1107): the engine's host
code (pach_convergence_replay) against the oracle's NumPy restatement (oracle/convergence.py), on
synthetic per-revolution histograms -- the same revolution must stop the run, and SpecMin's Nmin must
agree.  Also the pieces with quirks the checks depend on: SlidingMax's ring buffer and the Envelope."""
import numpy as np
import pytest

from oracle import convergence as OC
from pachydermacoustic_universal_gb300 import tracer


def synthetic_revolutions(rng, revs, T, fs=1000, noise=1.0, spec_ms=300):
    """Per-revolution raw contributions [revs][4][T]: an exponential diffuse decay and a sparse
    specular part before spec_ms, each revolution a noisy draw (gamma noise, mean 1)."""
    t = np.arange(T) / fs
    diffuse = 1e-4 * np.exp(-t / 0.25)
    spec = np.where((t < spec_ms / 1000.0) & (rng.random(T) < 0.05), 3e-4, 0.0)
    out = np.zeros((revs, 4, T))
    for r in range(revs):
        g = rng.gamma(1.0 / noise, noise, size=(3, T)) if noise > 0 else np.ones((3, T))
        a0 = spec * g[0]
        a1 = 0.7 * diffuse * g[1]
        a2 = 0.3 * diffuse * g[2]
        out[r, 1], out[r, 2], out[r, 3] = a0, a1, a2
        out[r, 0] = a0 + a1 + a2
    return out


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("seed", range(6))
def test_engine_checks_stop_where_the_oracle_stops(mode, seed):
    rng = np.random.default_rng(100 + seed)
    T = 1500 + 250 * seed
    per_rev = synthetic_revolutions(rng, 160, T, noise=[0.3, 1.0, 3.0][seed % 3])
    dist, c = 7.0 + seed, 343.0
    stop_e, nmin_e = tracer.convergence_replay(per_rev, mode, dist, c)
    stop_o, chk = OC.replay(per_rev, mode, dist, c, 1000)
    assert stop_e == stop_o
    if mode == 0:
        assert nmin_e == chk.nmin
        assert stop_e == 0 or stop_e * 80 > nmin_e  # SpecMin needs more than Nmin rays counted
    else:
        assert stop_e == 0 or stop_e >= 6         # six stable revolutions in a row


def test_a_check_that_never_settles_never_stops():
    rng = np.random.default_rng(3)
    per_rev = synthetic_revolutions(rng, 40, 1000, noise=1.0)
    per_rev[::2] *= 4.0  # every other revolution four times louder: never within 2 % / 10 %
    for mode in (0, 1):
        assert tracer.convergence_replay(per_rev[:12], mode, 5.0, 343.0)[0] == 0
        assert OC.replay(per_rev[:12], mode, 5.0, 343.0, 1000)[0] == 0


def test_sliding_max_keeps_the_ring_buffer_overwrite():
    # strictly falling input longer than the window: the push overwrites the head slot, so the
    # result is the new sample (a true sliding maximum would give x[i - window + 1])
    x = np.arange(10, 0, -1, dtype=float)
    got = OC.sliding_max(x, 3)
    true_max = [max(x[max(0, i - 2):i + 1]) for i in range(x.size)]
    assert got[:3].tolist() == true_max[:3] == [10.0, 10.0, 10.0]
    assert got[3] == x[3] == 7.0 and true_max[3] == 9.0


def test_minimum_check_needs_six_stable_revolutions():
    T = 1000
    per_rev = np.zeros((12, 4, T))
    per_rev[:, 0, 20:900] = 1.0  # identical revolutions: after the first, the sums grow by 1/n
    # relative change of a cumulative sum after n equal revolutions is 1/n: <= 2 % from n = 50 on
    per_rev = np.concatenate([per_rev] * 10)
    stop_e, _ = tracer.convergence_replay(per_rev, 1, 6.86, 343.0)
    stop_o, _ = OC.replay(per_rev, 1, 6.86, 343.0, 1000)
    assert stop_e == stop_o == 56  # stable from revolution 51 (1/50 is not > 2 %), six in a row: 56
