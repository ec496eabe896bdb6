"""Receiver filters on the GPU (csrc/filters.cu) against the FP64 oracle (oracle/filters.py):
Pach_SP.ETCToFilter (Pach_SP.cs:1584-1680) and Directional_Histogram.Create_Filter
(Classes_Receivers.cs:1910-1995), through the C ABI.

Both sides are FP64 transforms of the same sums; the GPU's four-step radix-2 transforms and numpy's
pocketfft round differently, so a filter must match within 1e-11 of its largest magnitude."""
import ctypes as C

import numpy as np
import pytest

from oracle import filters as F
from pachydermacoustic_universal_gb300 import _capi, rooms, tracer
from pachydermacoustic_universal_gb300.simulation import (GeodesicSource, Pach_SP, Polygon_Scene, Receiver_Bank,
                                                          SplitRayTracer)

pytestmark = pytest.mark.gpu
RTOL_MAX = 1e-11


def _close(got, ref):
    ref = np.asarray(ref)
    assert got.shape == ref.shape
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(got - ref).max() / scale
    assert err <= RTOL_MAX, err


@pytest.mark.parametrize("T,fs", [(1, 1000), (37, 1000), (3500, 1000), (16385, 1000), (16386, 1000), (2000, 44100),
                                  (40000, 44100)])
def test_etc_to_filter_matches_oracle(T, fs):
    rng = np.random.default_rng(T)
    P = rng.random((8, T)) * (rng.random((8, T)) > 0.2)
    swl = rng.uniform(80, 130, 8)
    _close(tracer.etc_to_filter(P, swl, fs), F.etc_to_filter(P, swl, fs))


def test_etc_to_filter_batch_and_default_level():
    rng = np.random.default_rng(9)
    P = rng.random((5, 8, 700))
    got = tracer.etc_to_filter(P, None, 1000)
    for i in range(5):
        _close(got[i], F.etc_to_filter(P[i], [120] * 8, 1000))
    _close(Pach_SP.ETCToFilter(list(P[0]), [120] * 8, 1000), got[0])


def _synthetic_histograms(R, T, seed):
    rng = np.random.default_rng(seed)
    E = rng.random((R, 8, T)) * (rng.random((R, 8, T)) > 0.4)
    P = np.sqrt(E * 413.0)
    P[:, :, ::7] += 0.5          # pressure where energy is 0: the directional envelopes stay 0 there
    u = rng.normal(size=(R, 3, 8, T))
    Dp = np.where(u > 0, u, 0.0) * E[:, None]
    Dn = np.where(u < 0, u, 0.0) * E[:, None]
    return E, P, Dp, Dn


def test_receiver_filters_match_oracle():
    E, P, Dp, Dn = _synthetic_histograms(3, 900, 4)
    swl = [100, 105, 110, 115, 120, 125, 118, 112]
    got = tracer.receiver_filters(P, E, Dp, Dn, swl=swl, sample_rate=1000)
    assert got.shape == (3, 7, 900 + 12287)
    for r in range(3):
        ref = F.receiver_filters(E[r], P[r], Dp[r], Dn[r], swl, 1000)
        for k in range(7):
            _close(got[r, k], ref[k])
    omni = tracer.receiver_filters(P, swl=swl, sample_rate=1000)
    assert omni.shape == (3, 1, 900 + 12287)
    np.testing.assert_allclose(omni[:, 0], got[:, 0], rtol=0, atol=1e-12 * np.abs(got[:, 0]).max())


def test_run_filters_equal_filters_of_the_scaled_histograms():
    w = rooms.shoebox_c1()
    w.cutoff_s = 0.5
    ds = tracer.DeviceScene(w.scene)
    run = tracer.Run(ds, w.sources, w.receivers, tracer.make_params(rays=3000, cutoff_length_m=w.cutoff_length_m,
                                                                    hist_cotime_ms=500.0, seed=11))
    run.wait()
    h = run.histograms(scaled=True)
    swl = np.array(w.sources[0].power_db)
    got = run.filters(directional=True, swl=swl)
    ref = tracer.receiver_filters(h["pressure"], h["energy"], h["dir_pos"], h["dir_neg"], swl=swl, sample_rate=1000)
    for r in range(got.shape[0]):
        for k in range(7):
            _close(got[r, k], ref[r, k])
    o = F.receiver_filters(h["energy"][0], h["pressure"][0], h["dir_pos"][0], h["dir_neg"][0], swl, 1000)
    for k in range(7):
        _close(got[0, k], o[k])
    run.close()
    ds.close()


def test_device_form_in_several_passes_equals_one_pass():
    torch = pytest.importorskip("torch")
    E, P, Dp, Dn = _synthetic_histograms(4, 500, 7)
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(v).to(dev) for k, v in dict(E=E, P=P, Dp=Dp, Dn=Dn).items()}
    scale = torch.tensor([1.0, 0.5, 2.0, 0.25], dtype=torch.float64, device=dev)
    L = _capi.lib()
    full = L.pach_filters_workspace_bytes(28, 500)
    one = L.pach_filters_workspace_bytes(1, 500)
    outs = []
    for wsb in (full, one + 1000):
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        out = torch.zeros((4, 7, 500 + 12287), dtype=torch.float64, device=dev)
        st = L.pach_filters_device(t["E"].data_ptr(), t["P"].data_ptr(), t["Dp"].data_ptr(), t["Dn"].data_ptr(),
                                   scale.data_ptr(), 4, 500, 7, 1000, None, 4096, out.data_ptr(), ws.data_ptr(), wsb,
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
        _capi.check(st)
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    ref = tracer.receiver_filters(P * np.array([1.0, 0.5, 2.0, 0.25])[:, None, None], E, Dp, Dn, sample_rate=1000)
    _close(outs[0], ref)


def test_receiver_bank_create_filter_after_a_split_ray_tracer_run():
    w = rooms.shoebox_c1()
    room = Polygon_Scene.from_arrays(w.scene)
    room.partition()
    src = GeodesicSource([120.0] * 8, w.sources[0].origin, 0)
    bank = Receiver_Bank([r.origin for r in w.receivers], src, room, 1000, 400.0)
    rt = SplitRayTracer(src, bank, room, 0.4 * room.Sound_speed(0), [0, 7], -1, 2000, seed=3)
    rt.Begin()
    rt.Combine_ThreadLocal_Results()
    bank.Create_Filter()
    rec = bank.Rec_List[1]
    assert rec.HasFilter() and len(bank.Filter_3Axis(1)) == 6
    ref = F.receiver_filters(rec._E, rec._P, rec._Dp, rec._Dn, [120] * 8, 1000)
    _close(rec.F, ref[0])
    for k in range(6):
        _close(rec.Fdir[k], ref[k + 1])
    seven = bank.Create_Filter([110] * 8, 1)
    assert len(seven) == 7
    _close(seven[0], F.receiver_filters(rec._E, rec._P, rec._Dp, rec._Dn, [110] * 8, 1000)[0])
    _close(bank.Create_Filter([110] * 8, 1, 0), seven[0])
    rt.close()
