"""CPU checks of the map host side: receiver placement (PachMapReceiver.Partition), the .pachm
writer/reader round trip, and the SPL / strength maps as the reference computes them."""
import types

import numpy as np
import pytest

from pachydermacoustic_universal_gb300.mapping import (Get_G_Map, Get_SPL_Map, MapMesh, PachMapReceiver)
from pachydermacoustic_universal_gb300.pachm import read_pachm, write_pachm
from pachydermacoustic_universal_gb300.simulation import GeodesicSource, SourceCluster

SC = types.SimpleNamespace(Sound_speed=lambda arg=0: 343.0, Rho_C=lambda arg=0: 411.6)


def _mesh():
    # two quads and a triangle, tilted so that face and vertex normals differ from +z
    V = [(0, 0, 0), (2, 0, 0), (2, 2, 0.5), (0, 2, 0.5), (4, 0, 0), (4, 2, 0.5), (6, 1, 0.2)]
    F = [(0, 1, 2, 3), (1, 4, 5, 2), (4, 6, 5)]
    return MapMesh(V, F)


def test_receiver_placement_follows_partition():
    src = GeodesicSource([100.0] * 8, (1.0, 1.0, 3.0))
    m = PachMapReceiver(_mesh(), src, 1000, 0.5, SC, 1000.0, False, True, False, False, False)
    cen = np.array([_mesh().Polygon_Vertices(i).mean(axis=0) for i in range(3)])
    np.testing.assert_allclose(m._origins, cen + [0, 0, 0.25])
    np.testing.assert_allclose([r.Direct_Time for r in m.Rec_List],
                               np.linalg.norm(cen + [0, 0, 0.25] - [1, 1, 3], axis=1) / 343.0)
    # face receivers without Z displacement: centroid + the UNIT face normal (not scaled by the increment)
    m2 = PachMapReceiver(_mesh(), src, 1000, 0.5, SC, 1000.0, False, False, False, False, False)
    mesh = _mesh()
    n0 = mesh.Normal(0)
    assert abs(np.linalg.norm(n0) - 1) < 1e-12 and n0[2] > 0
    np.testing.assert_allclose(m2._origins[0], cen[0] + n0)
    # vertex receivers: vertex + vertex normal x increment; Offset_Mesh moves the mesh the same way
    m3 = PachMapReceiver(_mesh(), src, 1000, 0.5, SC, 1000.0, False, False, False, True, True)
    vn = mesh.Vertex_Normals
    np.testing.assert_allclose(m3._origins, mesh.vertices + vn * 0.5)
    np.testing.assert_allclose(m3.Map_Mesh.vertices, mesh.vertices + vn * 0.5)
    # a cluster's receivers have direct time 0 (Map_Receiver ctor)
    cl = SourceCluster([src, GeodesicSource([100.0] * 8, (5.0, 1.0, 3.0))])
    m4 = PachMapReceiver(_mesh(), cl, 1000, 0.5, SC, 1000.0, False, True, False, False, False)
    assert all(r.Direct_Time == 0 for r in m4.Rec_List)


def _filled(seed=0, time_1pt=False, directional=False):
    src = GeodesicSource([100.0] * 8, (1.0, 1.0, 3.0))
    m = PachMapReceiver(_mesh(), src, 1000, 0.5, SC, 500.0, time_1pt, True, directional, False, False)
    rng = np.random.default_rng(seed)
    m._E[:] = rng.random(m._E.shape) * 1e-6
    m._P[:] = np.sqrt(m._E)
    if directional:
        m._Dp[:] = rng.random(m._Dp.shape) * 1e-6
        m._Dn[:] = -rng.random(m._Dn.shape) * 1e-6
    return m


@pytest.mark.parametrize("time_1pt,directional", [(False, False), (True, False), (False, True)])
def test_pachm_round_trip(tmp_path, time_1pt, directional):
    a, b = _filled(1, time_1pt, directional), _filled(2, time_1pt, directional)
    b.Src = (5.0, 1.0, 3.0)
    b.delay_ms = 12.5
    fn = tmp_path / "map.pachm"
    write_pachm(str(fn), [a, b])
    maps = read_pachm(str(fn))
    assert len(maps) == 2
    for src_map, got in zip((a, b), maps):
        np.testing.assert_array_equal(got._E, src_map._E[:, :, :src_map.SampleCT])
        np.testing.assert_array_equal(got._P, src_map._P[:, :, :src_map.SampleCT])
        assert [r.Direct_Time for r in got.Rec_List] == [r.Direct_Time for r in src_map.Rec_List]
        assert got.Src == src_map.Src and got.SrcType == "Geodesic" and got.delay_ms == src_map.delay_ms
        assert got.SampleCT == src_map.SampleCT and got.SampleRate == 1000
        assert got.Directional == directional
        if directional:
            np.testing.assert_array_equal(got._Dp, src_map._Dp)
            np.testing.assert_array_equal(got._Dn, src_map._Dn)
    np.testing.assert_array_equal(maps[0].Map_Mesh.vertices, a.Map_Mesh.vertices)
    assert maps[0].Map_Mesh.faces == a.Map_Mesh.faces
    # the reader places receivers on the (unoffset) face centroids
    np.testing.assert_allclose(maps[0].Rec_List[0].Origin, a.Map_Mesh.Polygon_Vertices(0).mean(axis=0))
    assert maps[0].Rec_List[0].Rho_C == 411.6


def test_spl_map_weights_grow_from_receiver_to_receiver():
    m = _filled(3)
    spl = Get_SPL_Map([m], [500.0, 0.0], 2, [0])
    w = 1.0
    for i in range(m.Count):
        w = np.sqrt(w * 405.0)
        arrival = int(m.Rec_List[i].Direct_Time * 1000)      # each source's histogram starts at its arrival
        e = m._E[i, 2, :m.SampleCT - arrival].sum() * w
        assert abs(spl[i] - 10 * np.log10(e / 1e-12)) < 1e-9
    g = Get_G_Map([m], 2, 100.0, 0)
    np.testing.assert_allclose(g, 10 * np.log10(m._E[:, 2].sum(axis=1) / 1e-12) - 100.0 + 31.0)
