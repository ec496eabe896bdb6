"""Seeded synthetic rooms with the shapes of the tracer's benchmark workloads.

No public benchmark scenes exist for this path, so seeded synthetic inputs stand in for them:

* ``shoebox_c1``   -- 10 x 8 x 4 m shoebox, 12 triangles (6 quads split), per-face 8-band
  absorption U[0.05, 0.35], scattering 0.2, one omni source at (2, 2, 1.5) m with 1 W per band
  (120 dB), 3 receivers of radius 0.5 m at seeded interior points.
* ``irregular_hall_c2`` -- 40 x 25 x 15 m shell tessellated to ~18k triangles with seeded vertex
  jitter (sigma 0.2 m), plus 200 random box and prism diffusers (side 0.3-2 m); ~20k triangles;
  per-triangle absorption U[0.02, 0.6] and scattering U[0.05, 0.8] per band; 2 sources, 16
  receivers of radius 0.5 m.
* ``batched_rooms_c3`` -- 64 rooms of log-uniform triangle count in [500, 50k], each a jittered
  shoebox with diffusers, 1-8 sources, 4-32 receivers.
* ``arena_c5`` -- 120 x 90 x 35 m arena shell with tiered seating facets and diffuser panels.

Scenes are returned as plain numpy arrays in the layout of ``pach_scene_desc``
(``include/pach_gpu.h``): a vertex list, polygon offsets into a vertex-index list, and per-polygon
8-band absorption / scattering / transmission.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BANDS = 8
OCTAVE_CENTRES = (62.5, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0)


@dataclass
class SceneArrays:
    vertices: np.ndarray          # (V, 3) float64
    poly_offsets: np.ndarray      # (P+1,) int32
    poly_indices: np.ndarray      # (sum,) int32
    absorption: np.ndarray        # (P, 8) float64
    scattering: np.ndarray        # (P, 8) float64
    transmission: np.ndarray      # (P, 8) float64
    temp_c: float = 20.0
    rel_humidity: float = 50.0
    pressure_hpa: float = 1013.25
    air_choice: int = 0
    edge_correction: int = 0

    @property
    def n_polys(self) -> int:
        return int(self.poly_offsets.shape[0] - 1)

    @property
    def n_triangles(self) -> int:
        counts = np.diff(self.poly_offsets)
        return int(np.sum(np.maximum(counts - 2, 0)))

    def bounds(self):
        return self.vertices.min(axis=0), self.vertices.max(axis=0)


@dataclass
class SourceSpec:
    origin: tuple
    power_db: tuple = (120.0,) * BANDS
    kind: int = 0                 # 0 geodesic, 1 random (theta, phi uniform), 2 uniform sphere


@dataclass
class ReceiverSpec:
    origin: tuple
    radius: float = 0.5


@dataclass
class Workload:
    name: str
    scene: SceneArrays
    sources: list
    receivers: list
    rays: int
    cutoff_s: float
    sample_rate: int = 1000
    extra: dict = field(default_factory=dict)

    @property
    def cutoff_length_m(self) -> float:
        c = 331.0 + 0.6 * self.scene.temp_c
        return self.cutoff_s * c


# ------------------------------------------------------------------------------------------
# builders
# ------------------------------------------------------------------------------------------
class _Builder:
    def __init__(self):
        self.verts: list = []
        self.polys: list = []

    def vertex(self, p) -> int:
        self.verts.append(tuple(float(x) for x in p))
        return len(self.verts) - 1

    def tri(self, a, b, c):
        self.polys.append((a, b, c))

    def quad_tris(self, a, b, c, d):
        """Quad a-b-c-d split into two triangles (a,b,c) and (a,c,d)."""
        self.tri(a, b, c)
        self.tri(a, c, d)

    def arrays(self):
        v = np.asarray(self.verts, dtype=np.float64).reshape(-1, 3)
        offs = np.zeros(len(self.polys) + 1, dtype=np.int32)
        idx = []
        for i, p in enumerate(self.polys):
            offs[i + 1] = offs[i] + len(p)
            idx.extend(p)
        return v, offs, np.asarray(idx, dtype=np.int32)


def _box_faces(b: _Builder, lo, hi):
    """Six faces of an axis-aligned box as 12 triangles; returns the face index of each triangle."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    c = [b.vertex(p) for p in [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
                               (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]]
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]
    face_of = []
    for f, q in enumerate(quads):
        b.quad_tris(c[q[0]], c[q[1]], c[q[2]], c[q[3]])
        face_of += [f, f]
    return face_of


def _interior_points(rng, lo, hi, n, margin, avoid=(), min_sep=1.0, tries=10000):
    pts = []
    lo = np.asarray(lo, float) + margin
    hi = np.asarray(hi, float) - margin
    for _ in range(tries):
        if len(pts) == n:
            break
        p = lo + (hi - lo) * rng.random(3)
        if all(np.linalg.norm(p - np.asarray(a)) >= min_sep for a in list(avoid) + pts):
            pts.append(p)
    if len(pts) < n:
        raise RuntimeError("could not place interior points")
    return [tuple(float(x) for x in p) for p in pts]


def shoebox_c1(seed: int = 1, rays: int = 100_000, scattering: float = 0.2) -> Workload:
    """10 x 8 x 4 m shoebox, 12 triangles, 1 source, 3 receivers, 2 s cutoff."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    face_of = _box_faces(b, (0, 0, 0), (10, 8, 4))
    v, offs, idx = b.arrays()
    face_abs = rng.uniform(0.05, 0.35, size=(6, BANDS))
    absn = face_abs[np.asarray(face_of)]
    scat = np.full((12, BANDS), scattering)
    trans = np.zeros((12, BANDS))
    scene = SceneArrays(v, offs, idx, absn, scat, trans)
    src = SourceSpec((2.0, 2.0, 1.5))
    recs = _interior_points(rng, (0, 0, 0), (10, 8, 4), 3, margin=1.0, avoid=[src.origin], min_sep=1.0)
    return Workload("shoebox_10x8x4_12tri", scene, [src], [ReceiverSpec(r) for r in recs], rays, 2.0)


def proposal_room_c4(seed: int, rays: int = 1_000_000, n_receivers: int = 3) -> Workload:
    """A room drawn like shoebox_c1 for the learned emission proposal: a shoebox of seeded size
    (8-12 x 6-10 x 3-5 m), 12 triangles, per-face absorption U[0.05, 0.35], scattering 0.2, one omni
    source and n_receivers receivers of radius 0.5 m at seeded interior points, 2 s cutoff."""
    rng = np.random.default_rng(1_000_003 * seed + 17)
    size = (rng.uniform(8, 12), rng.uniform(6, 10), rng.uniform(3, 5))
    b = _Builder()
    face_of = _box_faces(b, (0, 0, 0), size)
    v, offs, idx = b.arrays()
    face_abs = rng.uniform(0.05, 0.35, size=(6, BANDS))
    absn = face_abs[np.asarray(face_of)]
    scat = np.full((12, BANDS), 0.2)
    trans = np.zeros((12, BANDS))
    scene = SceneArrays(v, offs, idx, absn, scat, trans)
    src = _interior_points(rng, (0, 0, 0), size, 1, margin=1.0)[0]
    recs = _interior_points(rng, (0, 0, 0), size, n_receivers, margin=1.0, avoid=[src], min_sep=1.5)
    return Workload(f"proposal_room_{seed}", scene, [SourceSpec(src)], [ReceiverSpec(r) for r in recs], rays, 2.0,
                    extra={"size": size})


def _tessellated_shell(b: _Builder, size, target_tris, rng, sigma):
    """Box shell whose 6 faces are grids of quads (2 triangles each), vertices shared along edges
    and jittered in 3-D with N(0, sigma) per unique vertex."""
    L = np.asarray(size, float)
    area = 2 * (L[0] * L[1] + L[0] * L[2] + L[1] * L[2])
    h = math.sqrt(area / (target_tris / 2.0))
    n = [max(1, int(round(L[i] / h))) for i in range(3)]
    key_to_vid = {}
    pos = []

    def vid(i, j, k):
        key = (i, j, k)
        if key not in key_to_vid:
            key_to_vid[key] = len(pos)
            pos.append((L[0] * i / n[0], L[1] * j / n[1], L[2] * k / n[2]))
        return key_to_vid[key]

    tris = []
    # faces: fix one axis at 0 or n
    for axis in range(3):
        u_ax, v_ax = [a for a in range(3) if a != axis]
        for side in (0, n[axis]):
            for iu in range(n[u_ax]):
                for iv in range(n[v_ax]):
                    def g(du, dv):
                        c = [0, 0, 0]
                        c[axis] = side
                        c[u_ax] = iu + du
                        c[v_ax] = iv + dv
                        return vid(*c)
                    a, bb, cc, d = g(0, 0), g(1, 0), g(1, 1), g(0, 1)
                    tris.append((a, bb, cc))
                    tris.append((a, cc, d))
    P = np.asarray(pos, float)
    if sigma > 0:
        P = P + rng.normal(0.0, sigma, size=P.shape)
    base = len(b.verts)
    for p in P:
        b.vertex(p)
    for t in tris:
        b.tri(base + t[0], base + t[1], base + t[2])
    return len(tris)


def _diffuser(b: _Builder, rng, room, kind):
    """A box (12 triangles) or triangular prism (8 triangles) of side U[0.3, 2] m, rotated about z,
    placed against a random wall / floor / ceiling region inside the room."""
    L = np.asarray(room, float)
    s = rng.uniform(0.3, 2.0, size=3)
    # centre near one of the six boundary faces, inside the room
    axis = int(rng.integers(0, 3))
    side = int(rng.integers(0, 2))
    c = rng.uniform(0.15 * L, 0.85 * L)
    c[axis] = (s[axis] * 0.5 + 0.05) if side == 0 else (L[axis] - s[axis] * 0.5 - 0.05)
    th = rng.uniform(0, 2 * math.pi)
    R = np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1]])
    if kind == 0:
        corners = np.array([[x, y, z] for z in (-.5, .5) for y in (-.5, .5) for x in (-.5, .5)]) * s
        # order (x0y0z0, x1y0z0, x0y1z0, x1y1z0, ...) -> box vertex order used below
        pts = [c + R @ p for p in corners]
        ids = [b.vertex(p) for p in pts]
        o = [ids[0], ids[1], ids[3], ids[2], ids[4], ids[5], ids[7], ids[6]]
        for q in [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]:
            b.quad_tris(o[q[0]], o[q[1]], o[q[2]], o[q[3]])
        return 12
    tri2 = np.array([[-.5, -.5], [.5, -.5], [0.0, .5]])
    pts = []
    for z in (-.5, .5):
        for (x, y) in tri2:
            pts.append(c + R @ (np.array([x, y, z]) * s))
    ids = [b.vertex(p) for p in pts]
    b.tri(ids[0], ids[2], ids[1])
    b.tri(ids[3], ids[4], ids[5])
    for k in range(3):
        a0, a1 = ids[k], ids[(k + 1) % 3]
        c0, c1 = ids[3 + k], ids[3 + (k + 1) % 3]
        b.quad_tris(a0, a1, c1, c0)
    return 8


def _jittered_room(rng, size, target_tris, n_diffusers, sigma, abs_rng, scat_rng):
    b = _Builder()
    diff_tris_est = n_diffusers * 10
    shell_target = max(12, target_tris - diff_tris_est)
    _tessellated_shell(b, size, shell_target, rng, sigma)
    for _ in range(n_diffusers):
        _diffuser(b, rng, size, int(rng.integers(0, 2)))
    v, offs, idx = b.arrays()
    P = offs.shape[0] - 1
    absn = rng.uniform(abs_rng[0], abs_rng[1], size=(P, BANDS))
    scat = rng.uniform(scat_rng[0], scat_rng[1], size=(P, BANDS))
    return SceneArrays(v, offs, idx, absn, scat, np.zeros((P, BANDS)))


def irregular_hall_c2(seed: int = 2, rays: int = 1_000_000, target_tris: int = 20_000) -> Workload:
    """40 x 25 x 15 m jittered shell + 200 diffusers (~20k triangles), 2 sources, 16 receivers, 3 s."""
    rng = np.random.default_rng(seed)
    size = (40.0, 25.0, 15.0)
    scene = _jittered_room(rng, size, target_tris, 200, 0.2, (0.02, 0.6), (0.05, 0.8))
    srcs = _interior_points(rng, (0, 0, 0), size, 2, margin=4.0, min_sep=3.0)
    recs = _interior_points(rng, (0, 0, 0), size, 16, margin=4.0, avoid=srcs, min_sep=1.5)
    return Workload("irregular_hall_40x25x15_20ktri", scene, [SourceSpec(s) for s in srcs],
                    [ReceiverSpec(r) for r in recs], rays, 3.0)


def batched_rooms_c3(seed: int = 3, n_rooms: int = 64, max_rays: int = 1_000_000):
    """64 jittered shoebox rooms with diffusers, triangle counts log-uniform in [500, 50k]."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_rooms):
        ntri = int(round(math.exp(rng.uniform(math.log(500), math.log(50_000)))))
        size = (rng.uniform(6, 40), rng.uniform(5, 30), rng.uniform(3, 15))
        ndiff = int(min(200, max(0, (ntri - 200) // 100)))
        scene = _jittered_room(rng, size, ntri, ndiff, 0.05 * min(size) / 3, (0.05, 0.35), (0.1, 0.3))
        nsrc = int(rng.integers(1, 9))
        nrec = int(rng.integers(4, 33))
        margin = min(1.0, 0.2 * min(size))
        srcs = _interior_points(rng, (0, 0, 0), size, nsrc, margin=margin, min_sep=0.5)
        recs = _interior_points(rng, (0, 0, 0), size, nrec, margin=margin, avoid=srcs, min_sep=0.5)
        rays = int(round(math.exp(rng.uniform(math.log(10_000), math.log(max_rays)))))
        out.append(Workload(f"room{r:02d}_{ntri}tri", scene, [SourceSpec(s) for s in srcs],
                            [ReceiverSpec(q) for q in recs], rays, 2.0))
    return out


def arena_c5(seed: int = 5, rays: int = 10_000_000, target_tris: int = 500_000) -> Workload:
    """120 x 90 x 35 m arena: jittered shell, tiered seating facets on the long sides, 2k diffuser
    panels; absorption U[0.02, 0.9]; 4 sources, 64 receivers; 3.5 s."""
    rng = np.random.default_rng(seed)
    size = (120.0, 90.0, 35.0)
    b = _Builder()
    n_panels = 2000
    seat_rows = 40
    seat_target = int(target_tris * 0.35)
    shell_target = target_tris - seat_target - n_panels * 12
    _tessellated_shell(b, size, max(12, shell_target), rng, 0.05)
    # tiered seating: stepped facets (riser + tread) along both long walls, each split into strips
    strips = max(1, seat_target // (2 * seat_rows * 2 * 2))
    for side in (0, 1):
        for r in range(seat_rows):
            y_in = 2.0 + r * 0.8 if side == 0 else size[1] - 2.0 - r * 0.8
            y_out = y_in + (0.8 if side == 0 else -0.8)
            z0, z1 = 0.5 + r * 0.45, 0.5 + (r + 1) * 0.45
            for s in range(strips):
                x0 = 10.0 + (size[0] - 20.0) * s / strips
                x1 = 10.0 + (size[0] - 20.0) * (s + 1) / strips
                riser = [b.vertex(p) for p in [(x0, y_in, z0), (x1, y_in, z0), (x1, y_in, z1), (x0, y_in, z1)]]
                b.quad_tris(*riser)
                tread = [b.vertex(p) for p in [(x0, y_in, z1), (x1, y_in, z1), (x1, y_out, z1), (x0, y_out, z1)]]
                b.quad_tris(*tread)
    for _ in range(n_panels):
        _diffuser(b, rng, size, 0)
    v, offs, idx = b.arrays()
    P = offs.shape[0] - 1
    absn = rng.uniform(0.02, 0.9, size=(P, BANDS))
    scat = rng.uniform(0.05, 0.8, size=(P, BANDS))
    scene = SceneArrays(v, offs, idx, absn, scat, np.zeros((P, BANDS)))
    srcs = [(60.0, 45.0, 2.0), (30.0, 45.0, 3.0), (90.0, 45.0, 3.0), (60.0, 30.0, 10.0)]
    recs = _interior_points(rng, (0, 0, 0), size, 64, margin=3.0, avoid=srcs, min_sep=1.0)
    return Workload("arena_120x90x35_500ktri", scene, [SourceSpec(s) for s in srcs],
                    [ReceiverSpec(r) for r in recs], rays, 3.5)


def audience_plane(lo, hi, height: float, increment: float) -> np.ndarray:
    """Receiver centres [M][3] of a flat audience mesh of increment-sized squares covering [lo, hi] in
    (x, y) at `height`, placed as PachMapReceiver places face receivers with Z displacement
    (Pach_Map_Receiver.cs:107-139): each square's centroid raised by increment / 2."""
    nx = int(round((hi[0] - lo[0]) / increment))
    ny = int(round((hi[1] - lo[1]) / increment))
    xs = lo[0] + (np.arange(nx) + 0.5) * increment
    ys = lo[1] + (np.arange(ny) + 0.5) * increment
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    Z = np.full_like(X, height + increment * 0.5)
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
