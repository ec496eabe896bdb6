"""Mapping receivers: PachMapReceiver (Pachyderm_Acoustic_Universal/Pach_Map_Receiver.cs) over the
GPU engine.

A map is a mesh of audience surfaces with one small spherical receiver per face (or per vertex);
the tracer detects every segment against the map's receiver grid on the device (pach_map_desc), so
a run with a map fills M x 8 histograms at once.  This module places the receivers as the reference
does, carries the results in the reference's shape (Rec_List, GetEnergyHistogram, Direct_Time,
Rho_C), and provides the parameter maps (Get_SPL_Map, Get_Clarity_Map, Get_Definition_Map,
Get_RT_Map, Get_EDT_Map, Get_G_Map) without coherent superposition -- the decay and clarity maps
are computed on the device, all curves at once (pach_etc_parameters).

Hare's Topology (normals of the map mesh) is not part of the reference tree: a face normal here is
the normalised Newell normal of the face in its vertex order, a vertex normal the normalised sum of
the normals of the faces that use the vertex.
"""
from __future__ import annotations

import numpy as np

from . import _capi
from ._capi import check, dptr
from .tracer import MapReceivers


class MapMesh:
    """The analysis mesh (a Hare Topology of 3- and 4-vertex faces): vertices [V][3], faces as
    vertex-index tuples."""

    def __init__(self, vertices, faces):
        self.vertices = np.array(vertices, dtype=np.float64).reshape(-1, 3)
        self.faces = [tuple(int(i) for i in f) for f in faces]
        for f in self.faces:
            if len(f) not in (3, 4):
                raise ValueError("map faces have 3 or 4 vertices")

    @property
    def Vertex_Count(self):
        return self.vertices.shape[0]

    @property
    def Polygon_Count(self):
        return len(self.faces)

    def Polygon_Vertices(self, i):
        return self.vertices[list(self.faces[i])]

    def Normal(self, i):
        p = self.Polygon_Vertices(i)
        n = np.zeros(3)
        for a, b in zip(p, np.roll(p, -1, axis=0)):   # Newell
            n += np.array([(a[1] - b[1]) * (a[2] + b[2]), (a[2] - b[2]) * (a[0] + b[0]), (a[0] - b[0]) * (a[1] + b[1])])
        ln = np.linalg.norm(n)
        return n / ln if ln > 0 else n

    @property
    def Vertex_Normals(self):
        vn = np.zeros_like(self.vertices)
        for i, f in enumerate(self.faces):
            vn[list(f)] += self.Normal(i)
        ln = np.linalg.norm(vn, axis=1, keepdims=True)
        return np.divide(vn, ln, out=np.zeros_like(vn), where=ln > 0)

    @staticmethod
    def grid(lo, hi, height, increment):
        """A flat rectangle of increment-sized quads at z = height (counter-clockwise seen from above,
        normals +z)."""
        nx = int(round((hi[0] - lo[0]) / increment))
        ny = int(round((hi[1] - lo[1]) / increment))
        xs = lo[0] + np.arange(nx + 1) * increment
        ys = lo[1] + np.arange(ny + 1) * increment
        V = np.array([(x, y, height) for x in xs for y in ys])
        idx = lambda i, j: i * (ny + 1) + j  # noqa: E731
        F = [(idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)) for i in range(nx) for j in range(ny)]
        return MapMesh(V, F)


class Map_Receiver:
    """One map receiver (PachMapReceiver.Map_Receiver, Pach_Map_Receiver.cs:1692-1827): a view into
    its bank's histograms."""

    def __init__(self, bank, index, origin, direct_time, rho_c):
        self._bank = bank
        self.Index = index
        self.Origin = tuple(float(x) for x in origin)
        self.Direct_Time = float(direct_time)
        self.Rho_C = float(rho_c)
        self.Radius = bank.increment * 0.5

    def GetEnergyHistogram(self, Octave):
        E = self._bank._E[self.Index]
        return E[Octave].copy() if Octave < 8 else E.sum(axis=0)

    def Pressure_rms(self, t, Octave):
        return float(self._bank._P[self.Index, Octave, t])

    def Directions_Pos(self, Octave, t):
        """Directional_Histogram.Directions_Pos: the (+x, +y, +z) arrival sums at sample t."""
        return tuple(float(v) for v in self._bank._Dp[self.Index, :, Octave, t])

    def Directions_Neg(self, Octave, t):
        return tuple(float(v) for v in self._bank._Dn[self.Index, :, Octave, t])

    def Energy(self, t, oct):
        return float(self._bank._E[self.Index, oct, t])

    def Combine_Sample(self, sample, Energy_in, Pressure_in, Octave, dir_pos=None, dir_neg=None):
        """Histogram.Combine_Sample / Directional_Histogram.Combine_Sample (Classes_Receivers.cs:1168-1173,
        1750-1772)."""
        if sample >= self._bank._E.shape[2]:
            return
        if self._bank.Directional and sample < 0:
            sample = 0
        self._bank._E[self.Index, Octave, sample] += Energy_in
        self._bank._P[self.Index, Octave, sample] += Pressure_in
        if self._bank.Directional and dir_pos is not None:
            self._bank._Dp[self.Index, :, Octave, sample] += dir_pos
            self._bank._Dn[self.Index, :, Octave, sample] += dir_neg


class PachMapReceiver:
    """Drop-in for PachMapReceiver (Pach_Map_Receiver.cs:34-1834).  Receivers go on the face
    centroids (or the vertices) of Map_Mesh: with Z displacement raised by increment / 2, else offset
    along the face normal by one unit (the reference adds Normal(i) unscaled) or along the vertex
    normal by increment; Offset_Mesh then moves the mesh itself (Partition, 98-159).  Sphere diameter
    = increment, histograms at 1000 Hz of Cutoff_time ms counted from each receiver's direct
    arrival.  walk: 0 the reference's grid walks, 1 every crossed cell (see pach_map_desc)."""

    def __init__(self, Map_MeshIn=None, Src_Pt=None, SampleRate_in=1000, Increment_in=1.0, Sc=None,
                 Cutoff_time=2000.0, Time1Pt=False, Z_displacementIn=True, DirectionalIn=False, RecOnVertex=False,
                 Offset_Mesh=False, walk=0):
        self.Map_Mesh = Map_MeshIn
        self.delay_ms = 0.0
        self.Rec_List = []
        self.Directional = bool(DirectionalIn)
        if Map_MeshIn is None:          # the reading constructor (Read_pachm fills the fields)
            return
        if self.Directional and Time1Pt:
            raise ValueError("a one-point map histogram has no directions")
        self.SWL = Src_Pt.SWL()
        self.Src = tuple(Src_Pt.Origin)
        self.SrcType = Src_Pt.Type()
        self.CutOffTime = float(Cutoff_time)
        self.SampleRate = int(SampleRate_in)
        self.increment = float(Increment_in)
        self.Rec_Vertex = bool(RecOnVertex)
        self.Mesh_Offset = bool(Offset_Mesh)
        self.Z_Displacement = bool(Z_displacementIn)
        self.Time1Pt = bool(Time1Pt)
        self.walk = int(walk)
        self.SampleCT = 1 if self.Time1Pt else int(np.floor(self.CutOffTime * self.SampleRate / 1000))
        self._n_sources = len(Src_Pt.specs())
        self._place(Sc)

    # ---- Partition: receiver placement (Pach_Map_Receiver.cs:98-159)
    def _place(self, Sc):
        M = self.Map_Mesh
        inc = self.increment
        if self.Rec_Vertex:
            base = M.vertices.copy()
        else:
            base = np.array([M.Polygon_Vertices(i).mean(axis=0) for i in range(M.Polygon_Count)])
        if self.Z_Displacement:
            pts = base + np.array([0.0, 0.0, inc * 0.5])
        elif self.Rec_Vertex:
            pts = base + M.Vertex_Normals * inc
        else:
            pts = base + np.array([M.Normal(i) for i in range(M.Polygon_Count)])
        if not self.Z_Displacement and self.Mesh_Offset:
            M.vertices = M.vertices + M.Vertex_Normals * inc
        c = Sc.Sound_speed(0)
        rho_c = Sc.Rho_C(0)
        # Direct_Time (1737-1751): |source - receiver| / c; a SourceCluster leaves it 0
        if self._n_sources == 1:
            direct = np.linalg.norm(pts - np.asarray(self.Src), axis=1) / c
        else:
            direct = np.zeros(len(pts))
        self._origins = pts
        T = 1 if self.Time1Pt else int(self.CutOffTime / 1000.0 * 1000.0)
        self._alloc(len(pts), T)
        self.Rec_List = [Map_Receiver(self, i, p, direct[i], rho_c) for i, p in enumerate(pts)]

    def _alloc(self, M, T):
        self._E = np.zeros((M, 8, T))
        self._P = np.zeros((M, 8, T))
        if self.Directional:
            self._Dp = np.zeros((M, 3, 8, T))
            self._Dn = np.zeros((M, 3, 8, T))

    def map_receivers(self) -> MapReceivers:
        return MapReceivers(self._origins, self.increment, self.CutOffTime, self.Time1Pt, self.walk, self.Directional)

    def _set(self, h):
        """Results of a run (tracer.Run.map_histograms): histograms and the engine's direct arrival times."""
        self._E[:] = h["energy"]
        self._P[:] = h["pressure"]
        if self.Directional:
            self._Dp[:] = h["dir_pos"]
            self._Dn[:] = h["dir_neg"]
        for r, t in zip(self.Rec_List, h["direct_time"]):
            r.Direct_Time = float(t)

    @property
    def Count(self):
        return len(self.Rec_List)

    def Origins(self):
        return [r.Origin for r in self.Rec_List]

    def Data_Type(self):
        return "Type;Map_Data" if self.Directional else "Type;Map_Data_NoDir"

    def MapMesh(self):
        return self.Map_Mesh

    def Duration(self):
        return self._E.shape[2]

    def GetEnergyHistogram(self, Octave, Delay_ms=0.0, Rec_Index=0):
        """Receiver_Bank.GetEnergyHistogram(Octave, Delay_ms, Rec_Index) (Classes_Receivers.cs:432-437)."""
        h = self.Rec_List[Rec_Index].GetEnergyHistogram(Octave)
        pad = int(np.floor(Delay_ms / 1000.0 * self.SampleRate))
        out = np.zeros(pad + h.size)
        out[pad:] = h
        return out

    def AddDirect(self, D, S):
        """AddDirect (Pach_Map_Receiver.cs:322-340): the direct sound's samples into each receiver's
        histogram from sample 0 (the reference's time shift is commented out), where the path is
        unobstructed or screen attenuation is on."""
        for i, rec in enumerate(self.Rec_List):
            if not (D.Validity[i] or D.Screen_atten):
                continue
            # a directional histogram adds the unit vector towards the source to both direction sums
            u = np.subtract(S.Origin, rec.Origin)
            u = u / np.linalg.norm(u)
            for oct in range(8):
                Io = D.Io[i][oct]
                for s in range(Io.size):
                    if s < self.SampleCT:
                        rec.Combine_Sample(s, Io[s], np.sqrt(Io[s]), oct, u, u)

    def Create_Filter(self, VB=None):
        """Receiver_Bank.Create_Filter (Classes_Receivers.cs:626-651) for the map's receivers, on the GPU:
        each Map_Receiver's Histogram.Create_Filter (1175-1184: the pressure filter at 120 dB; none for
        one-point histograms) or, for a directional map, Directional_Histogram.Create_Filter
        (1968-1995: also the six directional filters)."""
        if self._E.shape[2] == 1:
            return None
        from .tracer import receiver_filters
        d = self.Directional
        f = receiver_filters(self._P, self._E, self._Dp if d else None, self._Dn if d else None, swl=None,
                             sample_rate=self.SampleRate)
        self._F = f[:, 0]
        self._Fdir = f[:, 1:] if d else None
        return None

    def GetFilter(self, Rec_Index):
        """Receiver_Bank.GetFilter (Classes_Receivers.cs:454-461): the receiver's filter, or SampleCT
        zeros before Create_Filter."""
        F = getattr(self, "_F", None)
        return np.zeros(self.SampleCT) if F is None else F[Rec_Index].copy()

    def HasFilter(self):
        return getattr(self, "_F", None) is not None

    def Combine_Clones(self, other):
        self._E += other._E
        self._P += other._P
        if self.Directional:
            self._Dp += other._Dp
            self._Dn += other._Dn


# ---------------------------------------------------------------- parameter maps
def _etc(Rec_List, i, Octave, SrcID):
    """IR_Construction.ETCurve(null, null, maps, CutOffTime, SampleRate, Octave, i, SrcID, true)
    (Classes_Math.cs:1351-1394, 1417-1475) for a map: the delayed histograms of the sources summed
    into (int)(CutOffTime * 0.001 * fs) + 16384 + ceil(max delay) bins."""
    m0 = Rec_List[0]
    maxdelay = max(Rec_List[s].delay_ms for s in range(len(Rec_List))) * m0.SampleRate / 1000.0
    H = np.zeros(int(m0.CutOffTime * 0.001 * m0.SampleRate) + 16384 + int(np.ceil(maxdelay)))
    for s in SrcID:
        ir = Rec_List[s].GetEnergyHistogram(Octave, Rec_List[s].delay_ms, i)
        H[:ir.size] += ir
    return H


def _device_parameters(Rec_List, Octave, SrcID, decay_depth=30, clarity_ms=80):
    m0 = Rec_List[0]
    etc = np.ascontiguousarray([_etc(Rec_List, i, Octave, SrcID) for i in range(m0.Count)])
    n, T = etc.shape
    out = {k: np.zeros(n) for k in ("t_x", "edt", "clarity", "definition", "energy")}
    check(_capi.lib().pach_etc_parameters(dptr(etc), n, T, int(m0.SampleRate), int(decay_depth), clarity_ms / 1000.0,
                                          dptr(out["t_x"]), dptr(out["edt"]), dptr(out["clarity"]),
                                          dptr(out["definition"]), dptr(out["energy"])))
    return out


def _no_coherent(flag):
    if flag:
        raise NotImplementedError("coherent superposition needs the reference's filter pipeline (not in this engine)")


def Get_RT_Map(Rec_List, Decay_Depth, Octave, SrcID, Coherent_Superposition=False):
    """Get_RT_Map (Pach_Map_Receiver.cs:1061-1128): T_X of the Schroeder integral per receiver."""
    _no_coherent(Coherent_Superposition)
    return _device_parameters(Rec_List, Octave, SrcID, decay_depth=Decay_Depth)["t_x"]


def Get_EDT_Map(Rec_List, Octave, SrcID, Coherent_Superposition=False):
    """Get_EDT_Map (1200-1269)."""
    _no_coherent(Coherent_Superposition)
    return _device_parameters(Rec_List, Octave, SrcID)["edt"]


def Get_Clarity_Map(Rec_List, C_Cutoff, Octave, SrcID, Coherent_Superposition=False):
    """Get_Clarity_Map (925-991): Clarity at C_Cutoff ms from bin 0 (the map's time zero is the
    direct arrival)."""
    _no_coherent(Coherent_Superposition)
    return _device_parameters(Rec_List, Octave, SrcID, clarity_ms=C_Cutoff)["clarity"]


def Get_Definition_Map(Rec_List, Octave, SrcID, Coherent_Superposition=False):
    """Get_Definition_Map (993-1059): Definition at 50 ms."""
    _no_coherent(Coherent_Superposition)
    return _device_parameters(Rec_List, Octave, SrcID)["definition"]


def Get_G_Map(Rec_List, Octave, SWL, SrcID, Coherent_Superposition=False):
    """Get_G_Map (1271-1329): Strength of one source's histogram, max(0, 10 log10(sum / 1e-12)) - SWL + 31."""
    _no_coherent(Coherent_Superposition)
    m = Rec_List[SrcID]
    tot = m._E[:, Octave].sum(axis=1) if Octave < 8 else m._E.sum(axis=(1, 2))
    with np.errstate(divide="ignore"):
        spl = 10.0 * np.log10(tot / 1e-12)
    spl = np.where(spl < 0, 0.0, spl)
    return spl - SWL + 31.0


def Get_SPL_Map(Rec_List, T_Bounds, Octave, SrcID, Coherent_Superposition=False, ZeroAtDirect=False, mod=None):
    """Get_SPL_Map without coherent superposition (Pach_Map_Receiver.cs:410-540), as the reference
    computes it: the bins summed are [floor(T_Bounds[1]), floor(T_Bounds[0])); each source's weight
    starts at 10^(0/10) = 1 (the mod argument is replaced) and becomes Pressure_Intensity(weight) =
    sqrt(405 weight) anew at every receiver, so it grows from receiver to receiver towards 405; a
    one-bin histogram takes its first sample twice."""
    _no_coherent(Coherent_Superposition)
    m0 = Rec_List[0]
    weight = np.ones(max(SrcID) + 1)
    out = np.zeros(m0.Count)
    T_Max, T_Min = int(np.floor(T_Bounds[0])), int(np.floor(T_Bounds[1]))
    for i in range(m0.Count):
        hist = np.zeros(m0.SampleCT)
        zero = 0
        if ZeroAtDirect:
            z = min(Rec_List[s].Rec_List[i].Direct_Time for s in SrcID)
            zero = int(z * m0.SampleRate)
        for s in SrcID:
            temp = Rec_List[s].GetEnergyHistogram(Octave, Rec_List[s].delay_ms, i)
            weight[s] = np.sqrt(weight[s] * 405.0)
            arrival = int(Rec_List[s].Rec_List[i].Direct_Time * m0.SampleRate) - zero
            for j in range(temp.size):
                t = j + arrival
                if hist.size == 1:
                    hist[0] += temp[j] * weight[s]
                if t >= hist.size:
                    break
                hist[t] += temp[j] * weight[s]
        e = hist[max(T_Min, 0):max(T_Max, 0)].sum() if T_Min < hist.size else 0.0
        spl = 10.0 * np.log10(e / 1e-12) if e > 0 else -np.inf
        out[i] = spl if spl >= 0 else 0.0
    return out
