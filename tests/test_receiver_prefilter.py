"""The shading pass's cheap receiver test (sphere_near in csrc/device_common.cuh) must accept every
sphere the exact test (sphere_hit, the restatement of Spherical_Receiver.CheckRay's sphere test,
Classes_Receivers.cs:839-849) accepts, or detections would be lost.  Both are restated here in
float32 as the device code computes them, for spheres placed about one radius from random segments
(the hardest cases), at room scales from 1 m to 1 km."""
import numpy as np

f32 = np.float32


def _exact(o, d, c, r2, tseg):
    m = (o - c).astype(f32)
    b = (m * d).sum(1, dtype=f32)
    cc = ((m * m).sum(1, dtype=f32) - r2).astype(f32)
    perp = (m - d * b[:, None]).astype(f32)
    disc = (r2 - (perp * perp).sum(1, dtype=f32)).astype(f32)
    t = -b
    return ~((cc > 0) & (b > 0)) & (disc >= 0) & (t > 0) & (t < tseg)


def _near(o, d, c, r2):
    m = (o - c).astype(f32)
    b = (m[:, 2] * d[:, 2] + m[:, 1] * d[:, 1] + m[:, 0] * d[:, 0]).astype(f32)  # another rounding order
    mm = (m * m).sum(1, dtype=f32)
    return (mm - b * b).astype(f32) <= (f32(1e-5) * mm + r2 + f32(1e-6)).astype(f32)


def test_cheap_receiver_test_is_a_superset_of_the_exact_one():
    rng = np.random.default_rng(11)
    n = 400_000
    for scale in (1.0, 10.0, 100.0, 1000.0):
        o = (rng.uniform(-1, 1, (n, 3)) * scale).astype(f32)
        d = rng.normal(size=(n, 3))
        d = (d / np.linalg.norm(d, axis=1)[:, None]).astype(f32)
        along = rng.uniform(-0.1, 1.1, n) * scale
        r = rng.uniform(0.05, 2.0, n)
        side = rng.normal(size=(n, 3))
        side -= (side * d).sum(1)[:, None] * d
        side /= np.linalg.norm(side, axis=1)[:, None]
        c = (o + d * along[:, None] + side * (r * rng.uniform(0.9, 1.1, n))[:, None]).astype(f32)
        r2 = (r * r).astype(f32)
        tseg = (rng.uniform(0, 1.2, n) * scale).astype(f32)
        hit = _exact(o, d, c, r2, tseg)
        near = _near(o, d, c, r2)
        assert hit.sum() > n // 10
        assert not np.any(hit & ~near), (scale, int(np.sum(hit & ~near)))
        # and it rejects: spheres two radii or more from the line never pass at room scales
        if scale <= 100.0:
            far = (o + d * along[:, None] + side * (2.5 * r)[:, None]).astype(f32)
            assert not np.any(_near(o, d, far, r2) & (r > 0.2))
