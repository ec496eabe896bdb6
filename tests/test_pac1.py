"""CPU checks of the .pac1 results file (pac1.py): the .NET BinaryWriter encodings and a round trip of
direct-sound and ray-traced sections through the reader that mirrors Read_Pac1."""
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from pachydermacoustic_universal_gb300 import pac1  # noqa: E402
from pachydermacoustic_universal_gb300.simulation import GeodesicSource, Receiver_Bank  # noqa: E402


def test_string_prefix_is_dotnet_7bit():
    import io
    for n, prefix in ((5, b"\x05"), (127, b"\x7f"), (128, b"\x80\x01"), (300, b"\xac\x02")):
        buf = io.BytesIO()
        pac1._Writer(buf).string("a" * n)
        data = buf.getvalue()
        assert data.startswith(prefix) and len(data) == len(prefix) + n
        assert pac1._Reader(data).string() == "a" * n


def test_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    scene = types.SimpleNamespace(Rho_C=lambda arg=0: 413.3, Sound_speed=lambda arg=0: 343.0)
    srcs = [GeodesicSource([120.0 - i for i in range(8)], (2, 2, 1.5)), GeodesicSource([100.0] * 8, (5, 3, 2))]
    pts = [(1.0, 2.0, 3.0), (4.0, 5.0, 1.0), (7.0, 1.0, 2.5)]
    banks, directs = [], []
    for k in range(2):
        b = Receiver_Bank(pts, srcs[k], scene, 1000, 250.0)
        for r in b.Rec_List:
            r._E[:] = rng.random(r._E.shape)
            r._P[:] = rng.random(r._P.shape)
            r._Dp[:] = rng.random(r._Dp.shape)
            r._Dn[:] = -rng.random(r._Dn.shape)
        banks.append(b)
        n = [103, 150, 101]
        d = types.SimpleNamespace(Delay_ms=0.0, Validity=[True, False, True],
                                  Io=[rng.random((8, m)) for m in n],
                                  Dir_Rec_Pos=[rng.random((8, m, 3)).astype(np.float32) for m in n],
                                  Dir_Rec_Neg=[-rng.random((8, m, 3)).astype(np.float32) for m in n])
        d.Time = lambda q, d=d: 0.01 * (q + 1)
        directs.append(d)
    f = str(tmp_path / "out.pac1")
    pac1.write_pac1(f, srcs, directs, banks)
    r = pac1.read_pac1(f)
    assert r["version"] == pac1.VERSION and r["sample_rate"] == 1000 and r["cutoff"] == 250.0
    assert r["sources"] == [tuple(float(x) for x in s.Origin) for s in srcs]
    assert r["receivers"] == pts and r["rho_c"] == [413.3] * 3
    assert len(r["direct"]) == 2 and len(r["ray_traced"]) == 2
    for k in range(2):
        dd = r["direct"][k]
        assert dd["type"] == "Geodesic" and np.array_equal(dd["swl"], srcs[k].SWL())
        for q in range(3):
            assert dd["rec"][q]["validity"] == directs[k].Validity[q]
            assert dd["rec"][q]["time"] == pytest.approx(0.01 * (q + 1))
            assert np.array_equal(dd["rec"][q]["io"], directs[k].Io[q])
            assert np.array_equal(dd["rec"][q]["dir_pos"], directs[k].Dir_Rec_Pos[q])
            assert np.array_equal(dd["rec"][q]["dir_neg"], directs[k].Dir_Rec_Neg[q])
        rt = r["ray_traced"][k]
        assert rt["samples"] == 250 and rt["sample_rate"] == 1000
        for q, rec in enumerate(banks[k].Rec_List):
            got = rt["rec"][q]
            assert got["sound_speed"] == 343.0
            assert np.array_equal(got["energy"], rec._E) and np.array_equal(got["pressure"], rec._P)
            assert np.array_equal(got["dir_pos"], rec._Dp) and np.array_equal(got["dir_neg"], rec._Dn)
