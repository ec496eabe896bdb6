"""The reference's engine API for the split ray tracer, over the GB300 C ABI.

Names, argument meanings and error behaviour follow Pachyderm_Acoustic_Universal so that a host
written against SplitRayTracer drives this engine unchanged:

* ``Polygon_Scene(Temp, hr, Pa, Air_Choice, EdgeCorrection, IsAcoustic)`` + ``Construct`` +
  ``partition`` -- Classes_Scenes.cs:70-105, 447-630, 727-755 (Pa in hPa, as the Scene ctor).
* ``Basic_Material(abs8)``, ``Lambert_Scattering(scat8)`` -- Classes_Materials.cs:60-200, 4463-4485.
* ``GeodesicSource`` / ``RandomSource`` / ``SourceCluster`` -- Classes_Sources.cs:34-404, 669-740.
* ``Receiver_Bank(points, source, scene, SampleRate, COTime_ms)`` with ``Spherical_Receiver``
  (Radius fixed to 1 m by the ctor, settable) -- Classes_Receivers.cs:139-164, 699-1102.
* ``SplitRayTracer(source, receivers, scene, cutoffTime, octaveRange, isOrder, rayCount)`` with
  ``Begin``, ``ThreadState``, ``ProgressMsg``, ``Combine_ThreadLocal_Results``, ``GetReceiver``,
  ``PercentLost``, ``Conclude_Simulation``, ``Sim_Type`` -- "Classes_Complete_Trace - TaskAll.cs".
  ``cutoffTime`` is a LENGTH in metres (COTime = cutoffTime / c, TaskAll:83).
* ``AcousticalMath`` -- Classes_Math.cs parameter functions.
* ``Receiver_Bank.Create_Filter`` / ``Spherical_Receiver.Create_Filter`` / ``Pach_SP.ETCToFilter`` --
  the receivers' filters (Classes_Receivers.cs:626-663, 1059-1080, 1910-1995; Pach_SP.cs:1584-1680),
  computed on the GPU.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from . import _capi
from ._capi import dptr
from .rooms import SceneArrays, SourceSpec, ReceiverSpec
from .tracer import DeviceScene, Run, make_params


class ThreadState:
    Running = "Running"
    Stopped = "Stopped"


class Basic_Material:
    def __init__(self, ABS):
        a = np.asarray(ABS, dtype=np.float64)
        if a.shape != (8,):
            raise ValueError("Basic_Material takes 8 octave-band absorption coefficients")
        self._abs = a

    def Coefficient_A_Broad(self, Octave=None):
        return self._abs.copy() if Octave is None else float(self._abs[Octave])


class Lambert_Scattering:
    def __init__(self, Scattering):
        s = np.asarray(Scattering, dtype=np.float64)
        if s.shape != (8,):
            raise ValueError("Lambert_Scattering takes 8 octave-band scattering coefficients")
        self._s = s

    def Coefficient(self, octave=None):
        return self._s.copy() if octave is None else float(self._s[octave])


class Polygon_Scene:
    """Scene of planar polygons; ``Construct(Model, Mat, Scat, Trans)`` takes, per object, a list of
    polygons (each an (n, 3) array of points) and the object's material, scattering and transmission."""

    def __init__(self, Temp=20.0, hr=50.0, Pa=1013.25, Air_Choice=0, EdgeCorrection=False, IsAcoustic=True):
        self.temp_c, self.hr, self.pa_hpa = float(Temp), float(hr), float(Pa)
        self.air_choice, self.edge = int(Air_Choice), int(bool(EdgeCorrection))
        self.Valid = False
        self.Partitioned = False
        self._arrays = None
        self._dev = None
        self._info = None

    def Construct(self, Model, Mat, Scat, Trans=None):
        if len(Mat) != len(Model) and len(Scat) != len(Model):
            raise ValueError("The number of material codes must match the numer of objects in the model...")
        verts, offs, idx, ab, sc, tr = [], [0], [], [], [], []
        for i, obj in enumerate(Model):
            for poly in obj:
                p = np.asarray(poly, dtype=np.float64).reshape(-1, 3)
                base = len(verts)
                verts.extend(p.tolist())
                idx.extend(range(base, base + len(p)))
                offs.append(len(idx))
                ab.append(Mat[i].Coefficient_A_Broad())
                sc.append(Scat[i].Coefficient())
                tr.append(np.zeros(8) if Trans is None else np.asarray(Trans[i], dtype=np.float64))
        self._arrays = SceneArrays(np.asarray(verts), np.asarray(offs, np.int32), np.asarray(idx, np.int32),
                                   np.asarray(ab), np.asarray(sc), np.asarray(tr), self.temp_c, self.hr, self.pa_hpa,
                                   self.air_choice, self.edge)
        self.Valid = True

    @classmethod
    def from_arrays(cls, arrays: SceneArrays):
        s = cls(arrays.temp_c, arrays.rel_humidity, arrays.pressure_hpa, arrays.air_choice, arrays.edge_correction)
        s._arrays = arrays
        s.Valid = True
        return s

    def partition(self, *args):
        if not self.Valid:
            raise RuntimeError("Construct the scene before partitioning it")
        self._dev = DeviceScene(self._arrays)
        self._info = self._dev.info()
        self.Partitioned = True

    def _need(self):
        if self._dev is None:
            self.partition()
        return self._info

    def Sound_speed(self, arg=0):
        return self._need()["sound_speed"]

    def Attenuation(self, arg=0):
        return self._need()["air_atten_db_per_m"].copy()

    def Rho_C(self, arg=0):
        return self._need()["rho_c"]

    def SurfaceArea(self, x):
        return float(self._need()["poly_area"][x])

    def Count(self):
        return self._arrays.n_polys

    @property
    def AbsorptionValue(self):
        return [Basic_Material(a) for a in self._arrays.absorption]


class Source:
    kind = 0
    type = ""

    def __init__(self, power_In_db, Source_, ID=0, Third_Octave=False):
        if Third_Octave:
            raise NotImplementedError("third-octave bands are not part of the GPU tracer")
        self.SPL = np.asarray(power_In_db, dtype=np.float64)
        self.Center = tuple(float(x) for x in Source_)
        self.S_ID = ID

    @property
    def Origin(self):
        return self.Center

    @property
    def SoundPower(self):
        return 1e-12 * 10 ** (0.1 * self.SPL)

    def SWL(self, octave=None):
        if octave is None:
            return self.SPL.copy()
        if octave < 8:
            return float(self.SPL[octave])
        return float(10 * np.log10(np.sum(10 ** (0.1 * self.SPL))))

    def Revolution_Period(self):
        return 80

    def Type(self):
        """Source.Type() (Classes_Sources.cs:220-223)."""
        return self.type

    def specs(self):
        return [SourceSpec(self.Center, tuple(self.SPL), self.kind)]


class GeodesicSource(Source):
    kind = 0
    type = "Geodesic"


class RandomSource(Source):
    kind = 1
    type = "PseudoRandom"


class SourceCluster(Source):
    type = "Cluster"

    def __init__(self, sources, id=0, third_octave=False):
        self.Sources = list(sources)
        self.S_ID = id
        spl = np.max([s.SPL for s in self.Sources], axis=0)
        self.SPL = spl
        self.Center = tuple(np.mean([s.Center for s in self.Sources], axis=0))

    def Revolution_Period(self):
        return sum(s.Revolution_Period() for s in self.Sources)

    def specs(self):
        out = []
        for s in self.Sources:
            out.extend(s.specs())
        return out


class Spherical_Receiver:
    def __init__(self, Center, SampleRate, CO_Time_ms, rho_c, Sound_Speed=343.0):
        self.Origin = tuple(float(x) for x in Center)
        self.Sound_Speed = float(Sound_Speed)
        self.Radius = 1.0          # Classes_Receivers.cs:751
        self.SampleRate = SampleRate
        self.CO_Time = CO_Time_ms
        self.Rho_C = rho_c
        T = int(SampleRate * (CO_Time_ms / 1000.0))
        self._E = np.zeros((8, T))
        self._P = np.zeros((8, T))
        self._Dp = np.zeros((3, 8, T))
        self._Dn = np.zeros((3, 8, T))
        self.Reflection_Analysis_Data = np.zeros((3, 8, T))

    def GetEnergyHistogram(self, Octave):
        return self._E[Octave].copy() if Octave < 8 else self._E.sum(axis=0)

    def GetRMSPressureHistogram(self, Octave):
        return self._P[Octave].copy() if Octave < 8 else self._P.sum(axis=0)

    def Directions_Pos(self, Octave, t, c):
        return float(self._Dp[c, Octave, t])

    def Directions_Neg(self, Octave, t, c):
        return float(self._Dn[c, Octave, t])

    def Energy(self, t, oct):
        return float(self._E[:, t].sum()) if oct == 8 else float(self._E[oct, t])

    def Create_Filter(self, SWL=None, dim=None):
        """Directional_Histogram.Create_Filter on the GPU (Classes_Receivers.cs:1059-1071, 1910-1995):
        no argument -- F (pressure) and Fdir[6] (-x +x -y +y -z +z) at 120 dB, kept on the receiver;
        SWL -- the 7 filters returned; SWL and dim -- dim outside 1..6 returns the pressure filter, and
        dim in 1..6 fails as the reference's does (it fills an unallocated array, 1942-1958)."""
        if dim is not None:
            if 1 <= int(dim) <= 6:
                raise RuntimeError("Create_Filter(SWL, Rho_C, dim) for dim 1..6 writes into unallocated "
                                   "arrays in the reference (NullReferenceException)")
            return self._filters(SWL, directional=False)[0]
        if SWL is None:
            f = self._filters(None)
            self.F, self.Fdir = f[0], list(f[1:])
            return None
        return list(self._filters(SWL))

    def _filters(self, SWL, directional=True):
        from .tracer import receiver_filters
        out = receiver_filters(self._P[None], self._E[None], self._Dp[None] if directional else None,
                               self._Dn[None] if directional else None, swl=SWL, sample_rate=self.SampleRate)
        return out[0]

    def Filter3Axis(self):
        """The six directional filters made by Create_Filter() (Classes_Receivers.cs:1073-1080)."""
        return getattr(self, "Fdir", None)

    def HasFilter(self):
        f = getattr(self, "Fdir", None)
        return f is not None and len(f) == 6 and len(f[5]) > 0


class Receiver_Bank:
    def __init__(self, Pt, SrcPT, Sc, SampleRate_in=1000, COTime_in=2000.0, Type=0, third_Oct=False):
        self.SampleRate = int(SampleRate_in)
        self.CutOffTime = float(COTime_in)
        self.SampleCT = int(np.floor(COTime_in * SampleRate_in / 1000))
        self.SWL = SrcPT.SWL()
        rho_c = Sc.Rho_C(0)
        c = Sc.Sound_speed(0)
        self.Rec_List = [Spherical_Receiver(p, self.SampleRate, self.CutOffTime, rho_c, c) for p in Pt]

    def Origins(self):
        return [r.Origin for r in self.Rec_List]

    def Create_Filter(self, SWL=None, Rec_ID=None, dim=None, VB=None):
        """Receiver_Bank.Create_Filter (Classes_Receivers.cs:626-663).  No SWL / Rec_ID: every
        receiver's F and Fdir (120 dB), all receivers in one GPU call; with them: that receiver's 7
        filters, or with dim its Create_Filter(SWL, dim)."""
        if Rec_ID is None:
            from .tracer import receiver_filters
            recs = self.Rec_List
            f = receiver_filters(np.stack([r._P for r in recs]), np.stack([r._E for r in recs]),
                                 np.stack([r._Dp for r in recs]), np.stack([r._Dn for r in recs]),
                                 swl=None, sample_rate=self.SampleRate)
            for r, fr in zip(recs, f):
                r.F, r.Fdir = fr[0], list(fr[1:])
            return None
        return self.Rec_List[Rec_ID].Create_Filter(SWL, dim)

    def Filter_3Axis(self, rec_id):
        return self.Rec_List[rec_id].Filter3Axis()


class Pach_SP:
    """Audio.Pach_SP's filter construction (Pach_SP.cs)."""

    @staticmethod
    def ETCToFilter(Octave_PRMS, SWL, sample_frequency=44100, sample_frequency_out=44100, reuseEdgeForOutside=True):
        """Pach_SP.ETCToFilter (Pach_SP.cs:1584-1680) on the GPU: [8][T] band pressure envelopes at
        sample_frequency -> T + 16383 samples (sample_frequency_out and reuseEdgeForOutside are unused
        there too)."""
        if Octave_PRMS is None or len(Octave_PRMS) != 8:
            raise ValueError("Octave_PRMS must be 8 bands.")
        T = len(Octave_PRMS[0])
        if any(len(b) != T for b in Octave_PRMS[1:]):
            raise ValueError("Inconsistent band lengths.")
        from .tracer import etc_to_filter
        return etc_to_filter(np.asarray(Octave_PRMS, dtype=np.float64), SWL, int(sample_frequency))


class SplitRayTracer:
    """Drop-in for Pachyderm_Acoustic.SplitRayTracer (TaskAll:33-1121), running on the GPU."""

    def __init__(self, sourceIn, receiverIn, roomIn, cutoffTime, octaveRange=(0, 7), isOrderIn=-1, rayCountIn=10000,
                 Vis_Feedback=None, seed=None, **kw):
        # rayCountIn < 1: convergence mode (TaskAll:111-176, 300-330) -- revolutions of Revolution_Period()
        # primaries until the convergence checks agree (0: SpecMin_Convergence_Check, < 0:
        # Minimum_Convergence_Check); the engine picks the checks' receivers as the ctor does
        self.Source = sourceIn
        self.RecMain = receiverIn
        self.Room = roomIn
        self.Raycount = int(rayCountIn)
        self.COTime = float(cutoffTime) / roomIn.Sound_speed(0)   # TaskAll:83
        self._cutoff_len = float(cutoffTime)
        self._oct = (int(octaveRange[0]), int(octaveRange[1]))
        self.IS_Order = int(isOrderIn)
        self._seed = int(time.time_ns() & 0xFFFFFFFFFFFF) if seed is None else int(seed)
        self._kw = kw
        self._run = None
        self._lost_percent = 0.0
        self._stats = None
        self._st = None
        self._ts = 0.0

    def Sim_Type(self):
        return "Stochastic Ray Tracing"

    def Begin(self):
        self._st = time.time()
        self.Room._need()
        specs = self.Source.specs()
        # a PachMapReceiver bank is traced as the run's mapping receivers (pach_map_desc)
        self._is_map = hasattr(self.RecMain, "map_receivers")
        recs = [] if self._is_map else [ReceiverSpec(r.Origin, r.Radius) for r in self.RecMain.Rec_List]
        kw = dict(self._kw)
        if self._is_map:
            kw["map_receivers"] = self.RecMain.map_receivers()
        params = make_params(rays=self.Raycount, cutoff_length_m=self._cutoff_len,
                             hist_cotime_ms=self.RecMain.CutOffTime, seed=self._seed, oct_range=self._oct,
                             is_order=self.IS_Order, sample_rate=self.RecMain.SampleRate, **kw)
        self._run = Run(self.Room._dev, specs, recs, params)

    def ThreadState(self):
        if self._run is None:
            return ThreadState.Stopped
        return ThreadState.Running if self._run.poll()["state"] == 0 else ThreadState.Stopped

    def Conclude_Simulation(self):
        if self._run is not None:
            self._run.cancel()

    @property
    def _currentRay(self):
        return [self._run.poll()["rays_done"]] if self._run else [0]

    @property
    def _rayTotal(self):
        return [self._run.poll()["end_traces"]] if self._run else [0]

    def ProgressMsg(self):
        p = self._run.poll()
        if p["rays_done"] == 0:
            return "Preparing Threads"
        el = time.time() - self._st
        if self.Raycount < 1:  # convergence mode: no total known in advance
            return f"Calculating Ray {p['rays_done']} (sub-ray {p['end_traces']}), until convergence. Press 'Esc' to Cancel..."
        rem = el * (p["rays_total"] - p["rays_done"]) / (p["rays_done"] + 1)
        h, m, s = int(rem // 3600), int(rem % 3600 // 60), int(rem % 60)
        return (f"Calculating Ray {p['rays_done']} of {p['rays_total']} (sub-ray {p['end_traces']}). "
                f"({h} hours,{m} minutes,{s} seconds Remaining.) Press 'Esc' to Cancel...")

    def Combine_ThreadLocal_Results(self):
        self._run.wait()
        if self._is_map:
            self.RecMain._set(self._run.map_histograms(scaled=True))
            self._stats = self._run.stats()
            self._lost_percent = self._stats["percent_lost"]
            self._ts = time.time() - self._st
            return
        h = self._run.histograms(scaled=True)
        for i, rec in enumerate(self.RecMain.Rec_List):
            rec._E[:] = h["energy"][i]
            rec._P[:] = h["pressure"][i]
            rec._Dp[:] = h["dir_pos"][i]
            rec._Dn[:] = h["dir_neg"][i]
            rec.Reflection_Analysis_Data[:] = h["analysis"][i]
        self._stats = self._run.stats()
        self._lost_percent = self._stats["percent_lost"]
        self._ts = time.time() - self._st

    @property
    def GetReceiver(self):
        return self.RecMain

    @property
    def PercentLost(self):
        return self._lost_percent

    @property
    def Stats(self):
        return self._stats

    def close(self):
        if self._run is not None:
            self._run.close()
            self._run = None


class Direct_Sound:
    """Direct sound of point sources (Classes_Direct.cs:232-262, 654-835), visibility rays on the GPU
    (pach_direct_sound).  Io, Time_Pt, Validity and the direction arrays are filled as the reference
    fills them, quirks included: Time_Pt adds Delay_ms to seconds; with ScreenCalc off the direct energy
    enters Io even when the path is blocked (ETCurve adds it only where IsOccluded, i.e. Validity, is
    true); a cluster's Validity is the last member's; negative direction components land in sample 0.
    Screen diffraction (ScreenCalc) and line / surface sources are not modelled."""

    def __init__(self, Src_in, Rec_in, Room_in, Octaves, ScreenCalc=False, SPL_Only=False):
        if ScreenCalc:
            raise NotImplementedError("screen diffraction is not part of the GPU engine")
        self.SPL_Only = bool(SPL_Only)
        self.Delay_ms = 0.0
        self.Src = Src_in
        self.Room = Room_in
        self.Oct_choice = list(Octaves)
        self.C_Sound = Room_in.Sound_speed(0)
        self.SampleFreq = Rec_in.SampleRate
        self.CO_Time = Rec_in.CutOffTime
        self.Receiver = Rec_in.Origins()
        R = len(self.Receiver)
        self.Validity = [False] * R
        self.Io = [None] * R
        self.Time_Pt = np.zeros(R)
        self.Dir_Rec_Pos = [None] * R
        self.Dir_Rec_Neg = [None] * R
        self.Rho_C = [Room_in.Rho_C(0)] * R

    def Begin(self):
        self.Calculate()

    def Calculate(self):
        srcs = self.Src.Sources if isinstance(self.Src, SourceCluster) else [self.Src]
        R, S = len(self.Receiver), len(srcs)
        sa = (_capi.SourceDesc * S)()
        for i, s in enumerate(srcs):
            sa[i].origin[:] = list(s.Center)
            sa[i].power_db[:] = [float(x) for x in s.SPL]
            sa[i].kind = s.kind
        ra = (_capi.ReceiverDesc * max(R, 1))()
        for i, p in enumerate(self.Receiver):
            ra[i].origin[:] = list(p)
            ra[i].radius = 1.0
        valid = np.zeros((R, S), dtype=np.int32)
        dist = np.zeros((R, S))
        energy = np.zeros((R, S, 8))
        self.Room._need()
        _capi.check(_capi.lib().pach_direct_sound(self.Room._dev.handle, sa, S, ra, R,
                                                  valid.ctypes.data_as(C.POINTER(C.c_int32)), dptr(dist), dptr(energy)))
        fs, c = self.SampleFreq, self.C_Sound
        for i in range(R):
            lo, hi = dist[i].min(), dist[i].max()
            self.Time_Pt[i] = lo / c + self.Delay_ms
            samples = 1 if self.SPL_Only else max(int(np.ceil((hi - lo) * fs / c)) + 100, 1)
            Io = np.zeros((8, samples))
            dp = np.zeros((8, samples, 3), dtype=np.float32)
            dn = np.zeros((8, samples, 3), dtype=np.float32)
            for s in range(S):
                self.Validity[i] = bool(valid[i, s])
                L = dist[i, s]
                t = 0 if self.SPL_Only else int(np.floor((L / c - self.Time_Pt[i]) * fs))
                t = min(max(t, 0), samples - 1)
                Io[:, t] += energy[i, s]
                d = (np.asarray(self.Receiver[i]) - np.asarray(srcs[s].Center)) / L
                for oct in range(8):
                    V = d * Io[oct, t]
                    for a in range(3):
                        if -V[a] > 0:
                            dp[oct, t, a] -= np.float32(V[a])
                        else:
                            dn[oct, 0, a] -= np.float32(V[a])
            self.Io[i], self.Dir_Rec_Pos[i], self.Dir_Rec_Neg[i] = Io, dp, dn

    def IsOccluded(self, id):
        return self.Validity[id]

    def Time(self, Rec_ID):
        return float(self.Time_Pt[Rec_ID])

    def Min_Time(self, Rec_ID):
        return float(self.Time_Pt[Rec_ID])

    def EnergyValue(self, octave, Rec_ID):
        return self.Io[Rec_ID].sum(axis=0) if octave > 7 else self.Io[Rec_ID][octave].copy()

    def EnergySum(self, Rec_ID, t):
        return float(self.Io[Rec_ID][:, t].sum()) if t < self.Io[Rec_ID].shape[1] else 0.0


class IR_Construction:
    """IR_Construction.ETCurve (Classes_Math.cs:1351-1475) for one source: the ray histogram delayed by
    the direct sound's Delay_ms, plus the direct sound where it is unobstructed, placed from
    ceil((Delay_ms / 1000 + Time_Pt) fs) (or sample 0 with StartAtZero).  Image-source paths (ISData)
    are not part of this engine and must be None."""

    @staticmethod
    def ETCurve(Direct, ISData, RTData, CO_Time_ms, Sampling_Frequency, Octave, Rec_ID, StartAtZero):
        if ISData is not None:
            raise NotImplementedError("image sources are not part of the GPU engine")
        delay = Direct.Delay_ms if Direct is not None else 0.0
        if RTData is not None:
            h = RTData.Rec_List[Rec_ID].GetEnergyHistogram(Octave)
            pad = int(np.floor(delay / 1000.0 * RTData.SampleRate))
            Histogram = np.zeros(pad + h.size)
            Histogram[pad:] = h
        else:
            Histogram = np.zeros(int((CO_Time_ms + int(delay)) * 0.001 * Sampling_Frequency))
        if Direct is not None and Direct.IsOccluded(Rec_ID):
            start = 0 if StartAtZero else int(np.ceil((delay * 0.001 + Direct.Time(Rec_ID)) * Sampling_Frequency))
            D = Direct.EnergyValue(Octave, Rec_ID)
            n = max(0, min(D.size, Histogram.size - start))
            Histogram[start:start + n] += D[:n]
        return Histogram


class AcousticalMath:
    """Room-acoustic parameters (Classes_Math.cs) computed by the library."""

    @staticmethod
    def SoundSpeed(Air_Temp):
        return _capi.lib().pach_math_sound_speed(float(Air_Temp))

    @staticmethod
    def Sabine(Room, volume):
        """Sabine reverberation time per octave band (Classes_Math.cs:212-228): T60 = 0.161 V /
        (sum S alpha + 4 m V), with m the scene's air attenuation as the reference takes it
        (Room.Attenuation(0), dB/m)."""
        m = Room.Attenuation(0)
        T60 = np.zeros(8)
        for t in range(8):
            TA = sum(Room.SurfaceArea(q) * Room.AbsorptionValue[q].Coefficient_A_Broad(t) for q in range(Room.Count()))
            T60[t] = 0.161 * (volume / (TA + 4 * m[t] * volume))
        return T60

    @staticmethod
    def Eyring(Room, volume):
        """The reference's Eyring time (Classes_Math.cs:246-263): T60 = 0.161 V / (sum S (-ln(1 - alpha))
        + 4 m V), the logarithm taken per surface."""
        m = Room.Attenuation(0)
        T60 = np.zeros(8)
        for t in range(8):
            TA = sum(Room.SurfaceArea(q) * -np.log(1 - Room.AbsorptionValue[q].Coefficient_A_Broad(t))
                     for q in range(Room.Count()))
            T60[t] = 0.161 * volume / (TA + 4 * m[t] * volume)
        return T60

    @staticmethod
    def Schroeder_Integral(etc):
        e = np.ascontiguousarray(etc, dtype=np.float64)
        out = np.zeros_like(e)
        _capi.check(_capi.lib().pach_math_schroeder(dptr(e), e.size, dptr(out)))
        return out

    @staticmethod
    def T_X(Schroeder_Integral, Decay_Depth, sample_f):
        s = np.ascontiguousarray(Schroeder_Integral, dtype=np.float64)
        return _capi.lib().pach_math_t_x(dptr(s), s.size, int(Decay_Depth), int(sample_f))

    @staticmethod
    def EarlyDecayTime(Schroeder_Integral, sample_f):
        s = np.ascontiguousarray(Schroeder_Integral, dtype=np.float64)
        return _capi.lib().pach_math_edt(dptr(s), s.size, int(sample_f))

    @staticmethod
    def Clarity(etc, sample_f, seconds, startTime, pressure):
        e = np.ascontiguousarray(etc, dtype=np.float64)
        return _capi.lib().pach_math_clarity(dptr(e), e.size, float(sample_f), float(seconds), float(startTime),
                                             int(bool(pressure)))

    @staticmethod
    def Definition(etc, sample_f, seconds, StartTime, pressure):
        e = np.ascontiguousarray(etc, dtype=np.float64)
        return _capi.lib().pach_math_definition(dptr(e), e.size, float(sample_f), float(seconds), float(StartTime),
                                                int(bool(pressure)))

    @staticmethod
    def Center_Time(etc, sample_f, Direct_time, pressure):
        e = np.ascontiguousarray(etc, dtype=np.float64)
        return _capi.lib().pach_math_center_time(dptr(e), e.size, int(sample_f), float(Direct_time), int(bool(pressure)))

    @staticmethod
    def Strength(etc, SWL, pressure):
        e = np.ascontiguousarray(etc, dtype=np.float64)
        return _capi.lib().pach_math_strength(dptr(e), e.size, float(SWL), int(bool(pressure)))


def room_parameters(etc, fs=1000, direct_time=0.0):
    """T30, EDT, C80 (dB) and D50 (%) of one energy-time curve, as Pachyderm derives them."""
    sch = AcousticalMath.Schroeder_Integral(etc)
    return {"T30": AcousticalMath.T_X(sch, 30, fs), "EDT": AcousticalMath.EarlyDecayTime(sch, fs),
            "C80": AcousticalMath.Clarity(etc, fs, 0.08, direct_time, False),
            "D50": AcousticalMath.Definition(etc, fs, 0.05, direct_time, False)}
