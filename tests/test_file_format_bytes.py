"""Byte-level pins of the result files against the reference writers' field order.

The expected bytes are assembled here one .NET BinaryWriter.Write call at a time, in the order the
reference writes them (paths relative to Pachyderm_Acoustic_Universal/):
  .pac1   Utilities.FileIO.Write_Pac1 (Classes_IO.cs:57-156), Direct_Sound.Write_Data
          (Classes_Direct.cs:61-107), Receiver_Bank.Write_Data (Classes_Receivers.cs:220-339)
  .pachm  Utilities.FileIO.Write_pachm (Classes_IO.cs:263-372)
BinaryWriter encodings: little-endian; Write(string) = 7-bit-group length prefix + UTF-8 bytes;
Write(bool) = 1 byte; Write(int) / Write(UInt32) = 4 bytes; Write(double) = 8; Write(float) = 4.
Value types as the reference declares them: Direct_Sound.Dir_Rec_Pos/Neg are float[][,,]
(Classes_Direct.cs:46), Spherical_Receiver.Directions_Pos/Neg(oct, t, c) return double
(Classes_Receivers.cs:976-999), Delay_ms is a double (Classes_Direct.cs:40), Rec_Type an enum written
as (int), Receiver_Bank.CO_Time returns CutOffTime (Classes_Receivers.cs:166-170).  The version
written is 2.6.0.20, whose Substring(0, 2) = "2." parses as 2 < 2.7: no third-octave flag."""
import struct
import types

import numpy as np

from pachydermacoustic_universal_gb300 import pac1
from pachydermacoustic_universal_gb300.mapping import MapMesh, PachMapReceiver
from pachydermacoustic_universal_gb300.pachm import write_pachm
from pachydermacoustic_universal_gb300.simulation import GeodesicSource, Receiver_Bank


class BW:
    """System.IO.BinaryWriter, call by call."""

    def __init__(self):
        self.b = bytearray()

    def string(self, s):
        data = s.encode("utf-8")
        n = len(data)
        while n >= 0x80:
            self.b.append((n & 0x7F) | 0x80)
            n >>= 7
        self.b.append(n)
        self.b += data

    def int(self, x):
        self.b += struct.pack("<i", int(x))

    def uint(self, x):
        self.b += struct.pack("<I", int(x))

    def double(self, x):
        self.b += struct.pack("<d", float(x))

    def single(self, x):
        self.b += struct.pack("<f", float(x))

    def bool(self, x):
        self.b += b"\x01" if x else b"\x00"


def _tiny_pac1():
    rng = np.random.default_rng(11)
    scene = types.SimpleNamespace(Rho_C=lambda arg=0: 413.3, Sound_speed=lambda arg=0: 343.0)
    src = GeodesicSource([120.0, 119.0, 118.0, 117.0, 116.0, 115.0, 114.0, 113.0], (2.0, 2.0, 1.5))
    pts = [(1.0, 2.0, 3.0), (4.5, 5.0, 1.25)]
    bank = Receiver_Bank(pts, src, scene, 1000, 3.0)  # 3 samples of 1 ms
    for r in bank.Rec_List:
        r._E[:] = rng.random(r._E.shape)
        r._P[:] = rng.random(r._P.shape)
        r._Dp[:] = rng.random(r._Dp.shape)
        r._Dn[:] = -rng.random(r._Dn.shape)
    n = [2, 1]
    d = types.SimpleNamespace(Delay_ms=0.0, Validity=[True, False], Io=[rng.random((8, m)) for m in n],
                              Dir_Rec_Pos=[rng.random((8, m, 3)).astype(np.float32) for m in n],
                              Dir_Rec_Neg=[-rng.random((8, m, 3)).astype(np.float32) for m in n])
    d.Time = lambda q: [0.0125, 0.021][q]
    return src, bank, d


def test_pac1_bytes_follow_write_pac1(tmp_path):
    src, bank, d = _tiny_pac1()
    date = "12/04/2026 09:15:00 AM"
    fn = str(tmp_path / "tiny.pac1")
    pac1.write_pac1(fn, [src], [d], [bank], date=date)
    got = open(fn, "rb").read()

    w = BW()
    w.string(date)                       # 1. DateTime.Now.ToString()
    w.string("2.6.0.20")                 # 2. PachTools.Version()
    w.double(bank.CutOffTime)            # 3. (double)Receiver[0].CO_Time
    w.int(bank.SampleRate)               #    Receiver[0].SampleRate
    w.int(1)                             # 4. SRC.Length
    for x in src.Origin:                 # 4.1-4.3
        w.double(x)
    w.int(len(bank.Rec_List))            # 5. Rec_List.Length
    for r in bank.Rec_List:              # 6. origin x y z, Rho_C
        for x in r.Origin:
            w.double(x)
        w.double(r.Rho_C)
    # 7. Direct_Sound.Write_Data
    w.string("Direct_Sound w sourcedata")
    w.string("Geodesic")                 # type
    for o in range(8):
        w.double(src.SWL(o))
    w.double(d.Delay_ms)
    for q in range(2):
        n = d.Io[q].shape[1]
        w.int(n)                         # Io[q][0].Length
        w.bool(d.Validity[q])
        w.double(d.Time(q))
        for t in range(n):
            for o in range(8):
                w.double(d.Io[q][o, t])
            for o in range(8):
                for a in range(3):
                    w.single(d.Dir_Rec_Pos[q][o, t, a])
                    w.single(d.Dir_Rec_Neg[q][o, t, a])
    # 9. Receiver_Bank.Write_Data
    w.string("Ray-Traced_Data")
    w.int(0)                             # (int)Rec_Type, Stationary
    w.int(bank.SampleRate)
    w.int(bank.SampleCT)
    w.double(bank.CutOffTime)
    for r in bank.Rec_List:
        w.double(r.Sound_Speed)
        for j in range(bank.SampleCT):
            for o in range(8):
                w.double(r._E[o, j])
                w.double(r._P[o, j])
                for a in range(3):
                    w.double(r._Dp[a, o, j])
                for a in range(3):
                    w.double(r._Dn[a, o, j])
    w.string("End")
    assert got == bytes(w.b)
    # literal header bytes: length-prefixed date, then "\x082.6.0.20", then 3.0 as a double, 1000 as an int
    k = 1 + len(date)
    assert got[0] == len(date) and got[k:k + 9] == b"\x082.6.0.20"
    assert got[k + 9:k + 17] == bytes.fromhex("0000000000000840") and got[k + 17:k + 21] == bytes.fromhex("e8030000")
    assert len(got) == len(w.b) == (k + 9 + 8 + 4 + 4 + 24 + 4 + 2 * 32 + (1 + 25) + (1 + 8) + 64 + 8
                                    + 2 * (4 + 1 + 8) + 3 * (64 + 192) + (1 + 15) + 4 + 4 + 4 + 8
                                    + 2 * (8 + 3 * 8 * 64) + (1 + 3))


def _tiny_map(directional):
    V = [(0, 0, 0), (2, 0, 0), (2, 2, 0.5), (0, 2, 0.5), (4, 0, 0)]
    F = [(0, 1, 2, 3), (1, 4, 2)]
    sc = types.SimpleNamespace(Sound_speed=lambda arg=0: 343.0, Rho_C=lambda arg=0: 411.6)
    src = GeodesicSource([100.0] * 8, (1.0, 1.0, 3.0))
    m = PachMapReceiver(MapMesh(V, F), src, 1000, 0.5, sc, 2.0, False, True, directional, False, False)
    rng = np.random.default_rng(5)
    m._E[:] = rng.random(m._E.shape)
    m._P[:] = rng.random(m._P.shape)
    if directional:
        m._Dp[:] = rng.random(m._Dp.shape)
        m._Dn[:] = -rng.random(m._Dn.shape)
    return m


def test_pachm_bytes_follow_write_pachm(tmp_path):
    for directional in (False, True):
        m = _tiny_map(directional)
        fn = str(tmp_path / f"tiny{int(directional)}.pachm")
        write_pachm(fn, [m])
        got = open(fn, "rb").read()
        w = BW()
        w.string("Type;Map_Data" if directional else "Type;Map_Data_NoDir")  # 1. Data_Type()
        w.uint(m.SampleCT)                       # 2. (UInt32)SampleCT
        w.uint(m.SampleRate)                     # 3. (UInt32)SampleRate
        w.uint(2)                                # 4. (UInt32)Rec_Ct (one receiver per face)
        w.string("Version")                      # 4.5
        w.string("2.6.0.20")
        w.string("Mesh Information")             # 5.
        w.string("Mesh Vertices")                # 6.
        w.uint(5)
        w.uint(2)
        for v in m.Map_Mesh.vertices:
            for x in v:
                w.double(x)
        w.string("Mesh Faces")                   # 7. four indices, a triangle repeats its third
        for f in [(0, 1, 2, 3), (1, 4, 2, 2)]:
            for i in f:
                w.uint(i)
        w.string("SourceswLoc")                  # 7.5
        w.int(1)                                 # Rec_List.Length (a plain int)
        for x in m.Src:
            w.double(x)
        w.string(m.SrcType)
        w.double(m.delay_ms)
        w.string("Receiver Hit Data")            # 8.
        w.bool(m.Rec_Vertex)                     # 8a.
        for i in range(2):
            w.uint(i)
            w.double(m.Rec_List[i].Direct_Time)
            w.double(m.Rec_List[i].Rho_C)
            for o in range(8):
                w.uint(o)
                for e in range(m.SampleCT):
                    w.double(m._E[i, o, e])
                    w.double(m._P[i, o, e])
                    if directional:
                        for a in range(3):
                            w.double(m._Dp[i, a, o, e])
                        for a in range(3):
                            w.double(m._Dn[i, a, o, e])
            w.string("End_Receiver_Hits")
        w.string("End_of_File")
        assert got == bytes(w.b), directional
