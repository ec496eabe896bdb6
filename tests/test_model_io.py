"""CPU checks of the text model reader / writer (model_io.py, after Classes_IO.cs:632-902)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from pachydermacoustic_universal_gb300 import model_io, rooms  # noqa: E402

SAMPLE = """# a box with a partition
[VERTICES]
1 0 0 0
2 4 0 0
3 4 3 0
4 0 3 0
5 2 0 0
6 2 3 0
7 2 3 2.5
8 2 0 2.5
[MATERIALS]
1 floor
ABSORPTION=0.1,0.1,0.12,0.15,0.2,0.2,0.25,0.3
SCATTERING=0.2, 0.2, 0.3
[END]
2 panel
ABSORPTION=0.5,0.5,0.5,0.5,0.5,0.5,0.5,0.5
TRANSMISSION=0.1,0.1,0.05,0.01,0,0,0,0
[END]
[OBJECT 1]
POLY 1,2,3,4
[OBJECT 2]
POLY 5,6,7,8 CURVE=0.1,0.2 FRAME=1,0,0,0,1,0
"""


def test_parse_sample(tmp_path):
    p = tmp_path / "m.txt"
    p.write_text(SAMPLE)
    v, mats, objs = model_io.parse_model(SAMPLE)
    assert len(v) == 8 and v[7] == (2.0, 3.0, 2.5)
    assert mats[0][0] == "floor" and mats[0][2] == [0.2, 0.2, 0.3, 0, 0, 0, 0, 0]
    assert mats[1][3][:4] == [0.1, 0.1, 0.05, 0.01]
    assert objs[0][1] == [[1, 2, 3, 4]] and objs[1][2] == [[0.1, 0.2]]
    scene = model_io.read_model_file(str(p))
    a = scene._arrays
    assert a.n_polys == 2 and a.pressure_hpa == 101325.0 and a.edge_correction == 1
    assert np.allclose(a.absorption[1], 0.5) and np.allclose(a.transmission[1][:2], 0.1)


def test_malformed_curvature_is_rejected():
    bad = SAMPLE.replace("POLY 5,6,7,8 CURVE=0.1,0.2 FRAME=1,0,0,0,1,0", "POLY 5,6,7,8 CURVE=0.1,0.2")
    with pytest.raises(ValueError):
        model_io.parse_model(bad)


def test_round_trip(tmp_path):
    w = rooms.irregular_hall_c2(target_tris=1500)
    p = tmp_path / "hall.txt"
    model_io.write_model_file(str(p), w.scene)
    scene = model_io.read_model_file(str(p))
    a, b = w.scene, scene._arrays
    assert b.n_polys == a.n_polys
    # polygons come back grouped by material: compare as multisets of (vertices, coefficients)
    def key(arr, i):
        ids = arr.poly_indices[arr.poly_offsets[i]:arr.poly_offsets[i + 1]]
        return (tuple(np.round(arr.vertices[ids].ravel(), 12)), tuple(arr.absorption[i]), tuple(arr.scattering[i]),
                tuple(arr.transmission[i]))
    assert sorted(key(a, i) for i in range(a.n_polys)) == sorted(key(b, i) for i in range(b.n_polys))
