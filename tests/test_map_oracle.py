"""CPU checks of the oracle's mapping receivers (PachMapReceiver) against hand-computed answers:
one ray bouncing between two parallel walls through a single receiver, with the reference's walks
(walk 0: the broadband phase only sees the legs that run towards +x in a room at positive
coordinates) and with every crossed cell (walk 1).  Tolerance: 1e-12 relative (same FP64 sums)."""
import types

import numpy as np

from oracle import oracle as O
from pachydermacoustic_universal_gb300 import rooms

ALPHA = 0.1


def _box(L=(10.0, 8.0, 4.0)):
    b = rooms._Builder()
    rooms._box_faces(b, (0, 0, 0), L)
    v, offs, idx = b.arrays()
    P = offs.size - 1
    return rooms.SceneArrays(v, offs, idx, np.full((P, 8), ALPHA), np.zeros((P, 8)), np.zeros((P, 8)))


def _workload(scene, src=(2.0, 2.0, 1.5), cutoff_s=2.0):
    return rooms.Workload("box", scene, [rooms.SourceSpec(src)], [], 1, cutoff_s)


def _map(origins, increment=1.0, cutoff_ms=3000.0, time_1pt=False, walk=0):
    return types.SimpleNamespace(origins=np.asarray(origins, float), increment=increment, cutoff_ms=cutoff_ms,
                                 time_1pt=time_1pt, walk=walk)


def _legs_through(x0, xr, L, n_legs):
    """Distances along a ray from x0 moving +x between walls at 0 and L at which it passes xr,
    and the direction (+1/-1) and index of each leg."""
    out = []
    pos, d, dist = x0, 1, 0.0
    for k in range(n_legs):
        wall = L if d > 0 else 0.0
        if min(pos, wall) <= xr <= max(pos, wall):
            out.append((dist + abs(xr - pos), d, k))
        dist += abs(wall - pos)
        pos, d = wall, -d
    return out


def _expected(walk, T_s=1.0):
    att, c, _ = O.medium()
    direct = 3.0 / c                                  # receiver at x = 5, source at x = 2
    r2 = 0.25
    E = np.zeros((8, 3000))
    for dist, d, k in _legs_through(2.0, 5.0, 10.0, 40):
        if dist / c >= T_s + direct:
            break
        if walk == 0 and d < 0:
            continue                                  # the broadband walk returns before visiting
        t = dist / c - direct
        e = (1 - ALPHA) ** k * 10 ** (-0.1 * att * t) / (np.pi * r2)
        E[:, int(t * 1000)] += e
    return E


def test_single_receiver_known_answer_both_walks():
    w = _workload(_box())
    counts = []
    for walk in (0, 1):
        m = _map([(5.0, 2.0, 1.5)], walk=walk)
        h, st = O.trace(w, rays=1, seed=1, pure_specular=True, prim_dirs=np.array([[1.0, 0, 0]]), map_receivers=m,
                        threads=1)
        got = h["map_energy"][0]
        exp = _expected(walk)
        n = 1000                                      # the first second: phase A legs only (44 legs = 1.28 s)
        np.testing.assert_allclose(got[:, :n], exp[:, :n], rtol=1e-12, atol=0)
        counts.append(np.count_nonzero(got[0, :n]))
        np.testing.assert_allclose(h["map_pressure"][0][:, :n], np.sqrt(exp[:, :n]), rtol=1e-12)
        np.testing.assert_allclose(h["map_direct"], [3.0 / O.medium()[1]], rtol=1e-15)
    # 343 m of travel in the first second: 34 legs, every other one towards +x
    assert counts == [18, 35], counts


def test_one_point_histogram_collects_every_arrival():
    w = _workload(_box())
    m = _map([(5.0, 2.0, 1.5), (7.0, 6.0, 2.0)], walk=1)
    h, _ = O.trace(w, rays=50, seed=4, pure_specular=True, map_receivers=m, threads=2)
    m1 = _map([(5.0, 2.0, 1.5), (7.0, 6.0, 2.0)], walk=1, time_1pt=True)
    h1, _ = O.trace(w, rays=50, seed=4, pure_specular=True, map_receivers=m1, threads=2)
    assert h1["map_energy"].shape == (2, 8, 1)
    np.testing.assert_allclose(h1["map_energy"][:, :, 0], h["map_energy"].sum(axis=2), rtol=1e-12)
    assert not h1["map_pressure"].any()


def test_cluster_direct_time_is_zero_and_receivers_are_tested_once():
    scene = _box()
    w = rooms.Workload("box2", scene, [rooms.SourceSpec((2.0, 2.0, 1.5)), rooms.SourceSpec((8.0, 6.0, 1.5))], [], 1, 2.0)
    origins = rooms.audience_plane((1.0, 1.0), (9.0, 7.0), 1.0, 1.0)
    m = _map(origins, walk=1)
    h, _ = O.trace(w, rays=30, seed=2, pure_specular=True, map_receivers=m, threads=2)
    assert np.all(h["map_direct"] == 0)
    # every crossed cell: the map holds exactly what brute-force sphere tests of the same legs give
    # (a receiver listed in several cells is tested once per segment)
    m0 = _map(origins, walk=0)
    h0, _ = O.trace(w, rays=30, seed=2, pure_specular=True, map_receivers=m0, threads=2)
    assert h0["map_energy"].sum() < h["map_energy"].sum()
