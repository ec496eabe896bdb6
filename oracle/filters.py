"""FP64 restatement of the receivers' filter construction: Pach_SP.ETCToFilter and the directional
histogram's Create_Filter.

TEST INFRASTRUCTURE ONLY: the checker of the GPU filter kernels (csrc/filters.cu); the product never
imports it.  Paths are relative to Pachyderm_Acoustic_Universal/.

* ETCToFilter (Pach_SP.cs:1584-1680): each of the 8 octave bands' pressure envelope, |P[b][t]| x
  10^((120 - SWL[b]) / 20), is convolved with a band carrier -- GenerateBandLimitedSincPulse
  (Pach_SP.cs:1682-1703), 16384 samples of sinc(bw t) cos(2 pi fc t) at the histogram's own sample
  rate, band edges fc / sqrt 2 .. fc sqrt 2 (fc = 62.5 x 2^b), L1-normalised to 2 / length -- and the
  products are summed; a ninth band at 16 kHz takes the 8 kHz envelope times
  10^(-(a16 - a8) t / fs x 343 / 20), a16 and a8 from the scalar ISO9613_1_attencoef
  (Classes_Medium_Props.cs:193-202) at 293.15 K, 101325 "Pa" and 50 %, whose exponents -1/2, -1/3,
  1/2 and -5/2 are C# integer divisions (0, 0, 0, -2).  The convolutions are FFT_Convolution_double
  (Pach_SP.cs:1948-1975, FFTW, zero padding to a power of two >= T + 16383): exact linear convolution,
  output T + 16383 samples.
* Directional_Histogram.Create_Filter (Classes_Receivers.cs:1910-1937; 1968-1995 with SWL = 120 dB):
  filter 0 from the band pressures, filters 2d + 1 and 2d + 2 (d = x, y, z) from
  P x Dir_Rec_Neg[d] / E and P x Dir_Rec_Pos[d] / E (0 where E = 0); each cut to T + 12287 samples
  (Array.Resize by -4096).  Histogram.Create_Filter (Classes_Receivers.cs:1186-1197) is filter 0 alone.
Parity with the reference itself is unpinned: the reference is C# and FFTW.NET (an external package),
neither runs here; the restatement is pinned to direct convolution in the CPU tests.
"""
from __future__ import annotations

import math

import numpy as np

CARRIER_LEN = 16384
CUT = 4096
RT2 = math.sqrt(2.0)


def iso9613_attencoef_scalar(freq, tk, pa, hr):
    """Classes_Medium_Props.cs:193-202 as written (dB/m), the C# integer-division exponents folded."""
    h = hr * math.pow(10.0, -6.8346 * math.pow(273.16 / tk, 1.261) + 4.6151) / (pa / 101.325)
    frO = (pa / 101.325) * (24 + 4.04 * math.pow(10.0, 4) * h * ((0.02 + h) / (0.391 + h)))
    frN = (pa / 101.325) * math.pow(tk / 293.15, 0) * (9 + 280 * h * math.exp(-4.170 * (math.pow(tk / 293.15, 0) - 1)))
    z = 0.1068 * math.exp(-3352 / tk) * math.pow(frN + freq * freq / frN, -1)
    y = math.pow(tk / 293.15, -2) * (0.01275 * math.exp(-2239.1 / tk) * math.pow(frO + freq * freq / frO, -1) + z)
    return 8.686 * freq * freq * ((1.84 * math.pow(10.0, -11) * math.pow(pa / 101.325, -1) * math.pow(tk / 293.15, 0)) + y)


def band_limited_sinc_pulse(length, fs, fl, fu):
    """GenerateBandLimitedSincPulse (Pach_SP.cs:1682-1703)."""
    fc = (fl + fu) / 2.0
    bw = fu - fl
    t0 = (length - 1) / 2.0
    t = (np.arange(length) - t0) / fs
    x = math.pi * bw * t
    sinc = np.ones(length) if bw == 0 else np.sin(x) / x
    c = sinc * np.cos(2 * math.pi * fc * t)
    norm = 2.0 / (np.abs(c).sum() * length)
    return c * norm if norm > 0 else c


def carriers(fs):
    """[9][16384]: the 8 octave carriers and the 16 kHz one."""
    out = []
    for b in range(8):
        fc = 62.5 * 2.0 ** b
        out.append(band_limited_sinc_pulse(CARRIER_LEN, fs, fc / RT2, fc * RT2))
    out.append(band_limited_sinc_pulse(CARRIER_LEN, fs, 16000.0 / RT2, 16000.0 * RT2))
    return np.array(out)


def hf_attenuation(T, fs):
    """Per-sample factor of the 16 kHz envelope (Pach_SP.cs:1628-1664)."""
    tk = 20 + 273.15
    pa = 101.325 * 1000
    add = iso9613_attencoef_scalar(16000.0, tk, pa, 50.0) - iso9613_attencoef_scalar(8000.0, tk, pa, 50.0)
    dist = np.arange(T) * (1.0 / fs) * 343.0
    return np.power(10.0, -add * dist / 20.0)


def _conv(a, b):
    n = a.size + b.size - 1
    W = 1 << (n - 1).bit_length()
    return np.fft.irfft(np.fft.rfft(a, W) * np.fft.rfft(b, W), W)[:n]


def etc_to_filter(prms, swl, fs, car=None):
    """ETCToFilter of [8][T] band pressure envelopes: T + 16383 samples."""
    prms = np.asarray(prms, dtype=float)
    T = prms.shape[1]
    car = carriers(fs) if car is None else car
    pmod = np.power(10.0, (120.0 - np.asarray(swl, dtype=float)) / 20.0)
    ir = np.zeros(T + CARRIER_LEN - 1)
    for b in range(8):
        ir += _conv(np.abs(prms[b]) * pmod[b], car[b])
    ir += _conv(np.abs(prms[7]) * pmod[7] * hf_attenuation(T, fs), car[8])
    return ir


def direction_envelopes(E, P, Dp, Dn):
    """The 7 envelope sets [7][8][T] of Create_Filter: P, then P Dn[d] / E and P Dp[d] / E per axis."""
    E, P = np.asarray(E, float), np.asarray(P, float)
    out = [P]
    with np.errstate(divide="ignore", invalid="ignore"):
        for d in range(3):
            out.append(np.where(E == 0, 0.0, P * np.asarray(Dn, float)[d] / E))
            out.append(np.where(E == 0, 0.0, P * np.asarray(Dp, float)[d] / E))
    return out


def receiver_filters(E, P, Dp, Dn, swl, fs, directional=True):
    """Create_Filter of one receiver: [7][T + 12287] (directional) or [1][T + 12287]."""
    car = carriers(fs)
    sets = direction_envelopes(E, P, Dp, Dn) if directional else [np.asarray(P, float)]
    return np.array([etc_to_filter(s, swl, fs, car)[:-CUT] for s in sets])
