"""The .pac1 results file of Pachyderm (Utilities.FileIO.Write_Pac1 / Read_Pac1,
Pachyderm_Acoustic_Universal/Classes_IO.cs:57-262; Direct_Sound.Write_Data / Read_Data,
Classes_Direct.cs:61-200; Receiver_Bank.Write_Data / Read_Data, Classes_Receivers.cs:220-424), so the
reference's host opens what the GPU engine computed.

Layout (.NET BinaryWriter: little-endian; strings carry a 7-bit-group length prefix and UTF-8 bytes):
date string, version string, cutoff time (double), sample rate (int), source count (int) and origins
(3 doubles each), receiver count (int) and per receiver origin (3 doubles) and rho c (double); then
per source a "Direct_Sound w sourcedata" section (type string, 8 SWL doubles, Delay_ms, per receiver
sample count, validity, arrival time and per sample 8 energies and 8 x 3 (pos, neg) float direction
pairs) and a "Ray-Traced_Data" section (receiver type, sample rate, sample count, cutoff, per receiver
sound speed and per sample and band energy, pressure, +x +y +z and -x -y -z direction doubles); "End".

The version written is the reference assembly's, 2.6.0.20: the reader then takes the v2.5+ layout
(pressure stored) and no third-octave flag (the writer's own flag test reads only "2." of the version,
so it never writes the flag for 2.x).
"""
from __future__ import annotations

import datetime
import struct

import numpy as np

VERSION = "2.6.0.20"
SOURCE_TYPES = {0: "Geodesic", 1: "PseudoRandom", 2: "Geodesic"}


class _Writer:
    def __init__(self, f):
        self.f = f

    def string(self, s: str):
        b = s.encode("utf-8")
        n = len(b)
        while True:  # 7 bits per byte, high bit = more
            byte = n & 0x7F
            n >>= 7
            self.f.write(bytes([byte | (0x80 if n else 0)]))
            if not n:
                break
        self.f.write(b)

    def double(self, x):
        self.f.write(struct.pack("<d", float(x)))

    def doubles(self, a):
        self.f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())

    def int32(self, x):
        self.f.write(struct.pack("<i", int(x)))

    def uint32(self, x):
        self.f.write(struct.pack("<I", int(x)))

    def boolean(self, x):
        self.f.write(b"\x01" if x else b"\x00")


class _Reader:
    def __init__(self, data: bytes):
        self.b = data
        self.i = 0

    def string(self) -> str:
        n, shift = 0, 0
        while True:
            byte = self.b[self.i]
            self.i += 1
            n |= (byte & 0x7F) << shift
            shift += 7
            if not byte & 0x80:
                break
        s = self.b[self.i:self.i + n].decode("utf-8")
        self.i += n
        return s

    def _unpack(self, fmt, size):
        v = struct.unpack_from(fmt, self.b, self.i)[0]
        self.i += size
        return v

    def double(self):
        return self._unpack("<d", 8)

    def doubles(self, n):
        a = np.frombuffer(self.b, dtype="<f8", count=n, offset=self.i).copy()
        self.i += 8 * n
        return a

    def floats(self, n):
        a = np.frombuffer(self.b, dtype="<f4", count=n, offset=self.i).copy()
        self.i += 4 * n
        return a

    def int32(self):
        return self._unpack("<i", 4)

    def uint32(self):
        return self._unpack("<I", 4)

    def boolean(self):
        return self._unpack("<?", 1)


def write_pac1(filename, sources, direct, banks, cutoff_ms=None, date=None):
    """Write one .pac1 file.  sources: the simulation Source objects (one per result set); direct: a
    Direct_Sound per source (simulation.Direct_Sound, computed); banks: a Receiver_Bank per source
    (filled by SplitRayTracer.Combine_ThreadLocal_Results); date: the date string written first
    (default: now, as DateTime.Now.ToString() writes it in the en-US culture)."""
    if not banks:
        raise ValueError("There is no simulated data to save.")
    rb = banks[0]
    with open(filename, "wb") as f:
        w = _Writer(f)
        w.string(date if date is not None else datetime.datetime.now().strftime("%m/%d/%Y %I:%M:%S %p"))
        w.string(VERSION)
        w.double(rb.CutOffTime if cutoff_ms is None else cutoff_ms)
        w.int32(rb.SampleRate)
        w.int32(len(sources))
        for s in sources:
            for x in s.Origin:
                w.double(x)
        w.int32(len(rb.Rec_List))
        for r in rb.Rec_List:
            for x in r.Origin:
                w.double(x)
            w.double(r.Rho_C)
        for k, s in enumerate(sources):
            d = direct[k]
            w.string("Direct_Sound w sourcedata")
            w.string("Cluster" if hasattr(s, "Sources") else SOURCE_TYPES.get(s.kind, "Geodesic"))
            for o in range(8):
                w.double(s.SWL(o))
            w.double(d.Delay_ms)
            for q in range(len(rb.Rec_List)):
                io = d.Io[q]
                n = io.shape[1]
                w.int32(n)
                w.boolean(d.Validity[q])
                w.double(d.Time(q))
                dirs = np.empty((n, 8, 3, 2), dtype="<f4")
                dirs[..., 0] = np.transpose(d.Dir_Rec_Pos[q], (1, 0, 2))
                dirs[..., 1] = np.transpose(d.Dir_Rec_Neg[q], (1, 0, 2))
                for t in range(n):
                    w.doubles(io[:, t])
                    f.write(dirs[t].tobytes())
            bank = banks[k]
            w.string("Ray-Traced_Data")
            w.int32(0)                         # Receiver_Bank.Type.Stationary
            w.int32(bank.SampleRate)
            w.int32(bank.SampleCT)
            w.double(bank.CutOffTime)
            for r in bank.Rec_List:
                w.double(r.Sound_Speed if hasattr(r, "Sound_Speed") else 343.0)
                T = bank.SampleCT
                rec = np.zeros((T, 8, 8))
                rec[:, :, 0] = r._E[:, :T].T
                rec[:, :, 1] = r._P[:, :T].T
                for c in range(3):
                    rec[:, :, 2 + c] = r._Dp[c, :, :T].T
                    rec[:, :, 5 + c] = r._Dn[c, :, :T].T
                w.doubles(rec)
        w.string("End")


def read_pac1(filename):
    """Read a .pac1 file the way Read_Pac1 does (versions >= 2.2 layout).  Returns a dict with the
    header, per source the direct-sound data and per source the receivers' histograms."""
    r = _Reader(open(filename, "rb").read())
    out = {"date": r.string(), "version": r.string()}
    v = float(out["version"][:3])
    out["cutoff"] = r.double()
    out["sample_rate"] = r.int32()
    if v >= 2.7:
        out["third_octave"] = r.boolean()
    ns = r.int32() if v >= 1.1 else 1
    out["sources"] = [(r.double(), r.double(), r.double()) for _ in range(ns)]
    nr = r.int32()
    out["receivers"], out["rho_c"] = [], []
    for _ in range(nr):
        out["receivers"].append((r.double(), r.double(), r.double()))
        out["rho_c"].append(r.double() if v >= 2.0 else 400.0)
    out["direct"], out["ray_traced"] = [], []
    while True:
        tag = r.string() if r.i < len(r.b) else ""
        if tag in ("End", ""):
            return out
        if tag in ("Direct_Sound", "Direct_Sound w sourcedata"):
            d = {"type": r.string().split(":")[0], "swl": r.doubles(8), "delay_ms": r.double(), "rec": []}
            for _ in range(nr):
                n = r.int32()
                valid = r.boolean()
                tp = r.double()
                io = np.zeros((8, n))
                pos = np.zeros((8, n, 3), dtype=np.float32)
                neg = np.zeros((8, n, 3), dtype=np.float32)
                for t in range(n):
                    io[:, t] = r.doubles(8)
                    pn = r.floats(48).reshape(8, 3, 2)
                    pos[:, t, :] = pn[..., 0]
                    neg[:, t, :] = pn[..., 1]
                d["rec"].append({"validity": valid, "time": tp, "io": io, "dir_pos": pos, "dir_neg": neg})
            out["direct"].append(d)
        elif tag == "Ray-Traced_Data":
            rt = {"type": r.uint32(), "sample_rate": r.int32()}
            T = r.int32()
            rt["samples"] = T
            rt["cutoff"] = r.double()
            rt["rec"] = []
            for _ in range(nr):
                c = r.double()
                a = r.doubles(T * 64).reshape(T, 8, 8)
                rt["rec"].append({"sound_speed": c, "energy": a[:, :, 0].T.copy(), "pressure": a[:, :, 1].T.copy(),
                                  "dir_pos": np.transpose(a[:, :, 2:5], (2, 1, 0)).copy(),
                                  "dir_neg": np.transpose(a[:, :, 5:8], (2, 1, 0)).copy()})
            out["ray_traced"].append(rt)
        else:
            raise ValueError(f"unknown .pac1 section {tag!r}")
