"""Receiver filters, CPU side: the oracle's restatement of ETCToFilter (oracle/filters.py) pinned to
direct convolution and to the reference's carrier normalisation, and the argument checks of the C ABI
and of the Python mirror, which refuse before any device work (Pach_SP.cs:1584-1703;
Classes_Receivers.cs:1910-1995)."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import filters as F
from pachydermacoustic_universal_gb300 import _capi, tracer
from pachydermacoustic_universal_gb300.simulation import Pach_SP, Spherical_Receiver


def test_fft_convolution_restatement_equals_direct_convolution():
    rng = np.random.default_rng(3)
    for T, fs in ((1, 1000), (57, 1000), (300, 44100)):
        P = rng.random((8, T)) * (rng.random((8, T)) > 0.3)
        swl = rng.uniform(90, 130, 8)
        car = F.carriers(fs)
        pm = 10.0 ** ((120.0 - swl) / 20.0)
        ref = sum(np.convolve(P[b] * pm[b], car[b]) for b in range(8))
        ref = ref + np.convolve(P[7] * pm[7] * F.hf_attenuation(T, fs), car[8])
        got = F.etc_to_filter(P, swl, fs)
        assert got.shape == (T + 16383,)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_carriers_follow_the_reference_pulse():
    fs = 1000
    car = F.carriers(fs)
    assert car.shape == (9, 16384)
    # L1 normalisation to 2 / length (Pach_SP.cs:1698-1700), symmetric about sample 8191.5
    np.testing.assert_allclose(np.abs(car).sum(axis=1) * 16384, 2.0, rtol=1e-12)
    np.testing.assert_allclose(car, car[:, ::-1], rtol=0, atol=1e-18)
    # band 3 (500 Hz): sinc(bw t) cos(2 pi fc t) sample by sample, times one normalising constant
    fl, fu = 500 / math.sqrt(2), 500 * math.sqrt(2)

    def raw(n):
        t = (n - 8191.5) / fs
        return math.sin(math.pi * (fu - fl) * t) / (math.pi * (fu - fl) * t) * math.cos(2 * math.pi * (fl + fu) / 2 * t)

    norm = 2.0 / (sum(abs(raw(n)) for n in range(16384)) * 16384)
    for n in (0, 100, 8191, 9000, 16383):
        assert abs(car[3][n] - raw(n) * norm) <= 1e-12 * abs(raw(n) * norm) + 1e-30


def test_16k_band_attenuation_uses_the_scalar_iso_formula_as_written():
    # 101.325 x 1000 is passed where the formula expects kPa: Pa / 101.325 = 1000
    a8 = F.iso9613_attencoef_scalar(8000.0, 293.15, 101325.0, 50.0)
    a16 = F.iso9613_attencoef_scalar(16000.0, 293.15, 101325.0, 50.0)
    assert 0 < a8 < a16
    ramp = F.hf_attenuation(5, 1000)
    np.testing.assert_allclose(ramp, 10 ** (-(a16 - a8) * np.arange(5) * 0.343 / 20), rtol=1e-14)
    assert ramp[0] == 1.0


def test_direction_envelopes_are_zero_where_energy_is_zero():
    E = np.array([[1.0, 0.0, 2.0]] * 8)
    P = np.array([[2.0, 5.0, 4.0]] * 8)
    Dp = np.ones((3, 8, 3)) * 0.5
    Dn = -np.ones((3, 8, 3))
    sets = F.direction_envelopes(E, P, Dp, Dn)
    assert len(sets) == 7
    np.testing.assert_array_equal(sets[0], P)
    np.testing.assert_array_equal(sets[1][0], [-2.0, 0.0, -2.0])   # P Dir_Rec_Neg / E
    np.testing.assert_array_equal(sets[2][0], [1.0, 0.0, 1.0])     # P Dir_Rec_Pos / E


def _err(call):
    st = call()
    return st, _capi.last_error()


def test_c_abi_refuses_bad_shapes_before_device_work():
    L = _capi.lib()
    out = np.zeros(16)
    x = np.zeros(8)
    dp = _capi.dptr
    st, msg = _err(lambda: L.pach_etc_to_filter(dp(x), 1, 0, None, 1000, dp(out), out.size))
    assert st == 1 and "T < 1" in msg
    st, msg = _err(lambda: L.pach_etc_to_filter(dp(x), 1, 1 << 20, None, 1000, dp(out), out.size))
    assert st == 1 and "2^20" in msg
    st, msg = _err(lambda: L.pach_etc_to_filter(dp(x), 1, 1, None, 0, dp(out), out.size))
    assert st == 1 and "sample rate" in msg
    st, msg = _err(lambda: L.pach_etc_to_filter(dp(x), 1, 1, None, 1000, dp(out), out.size))
    assert st == 1 and "cap" in msg
    st, msg = _err(lambda: L.pach_receiver_filters(None, None, None, None, 1, 1, 1000, None, dp(out), 1 << 20))
    assert st == 1 and "pressure" in msg
    st, msg = _err(lambda: L.pach_filters_device(None, None, None, None, None, 1, 1, 3, 1000, None, 0, None, None, 0,
                                                None))
    assert st == 1 and "kinds" in msg
    assert L.pach_filters_workspace_bytes(0, 10) == 0
    assert L.pach_filters_workspace_bytes(7, 3500) >= 7 * 5 * 32768 * 16


def test_mirror_errors_follow_the_reference():
    with pytest.raises(ValueError, match="8 bands"):
        Pach_SP.ETCToFilter([np.zeros(4)] * 7, [120] * 8, 1000)
    with pytest.raises(ValueError, match="Inconsistent"):
        Pach_SP.ETCToFilter([np.zeros(4)] * 7 + [np.zeros(5)], [120] * 8, 1000)
    rec = Spherical_Receiver((0, 0, 0), 1000, 100.0, 413.0)
    with pytest.raises(RuntimeError, match="unallocated"):
        rec.Create_Filter([120] * 8, 3)
    assert rec.Filter3Axis() is None and not rec.HasFilter()
    with pytest.raises(ValueError, match="shape"):
        tracer.receiver_filters(np.zeros((2, 8, 5)), np.zeros((2, 8, 4)), np.zeros((2, 3, 8, 5)), np.zeros((2, 3, 8, 5)))
