"""pach_trace_run_noalloc against the allocating entry point.

Some hosts cannot allocate device memory while they trace -- a host tracing from an audio or plug-in
processing callback, or code whose device memory belongs to another framework's allocator.  For them
the library has pach_trace_run_noalloc: it works in a fixed device array inside the library and writes
into device buffers the caller passes.  This test makes two calls in a row through the C ABI (the
array keeps the previous call's contents, so the second call also checks that the entry point clears
what must start at zero) and compares each with the histograms of pach_trace_begin on the same seed,
within the tolerance of the rerun and shard tests: 1e-9 relative, since only the order of the FP64
atomic additions differs.  The test allocates its buffers itself, with torch, outside the call.  The
first call on a device may load the library's device code (a one-time allocation, which is why a
host makes that call at set-up); from the second call on, the device's free memory and torch's
allocated memory must not move."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_entry_point_matches_the_allocating_one_on_two_calls():
    torch = pytest.importorskip("torch")
    from pachydermacoustic_universal_gb300 import _capi, rooms, tracer

    w = rooms.shoebox_c1()
    n = 800
    torch.cuda.set_device(0)
    ds = tracer.DeviceScene(w.scene)
    ref, st_ref = tracer.trace(w, dscene=ds, rays=n, seed=9)
    R, T = len(w.receivers), int(w.sample_rate * w.cutoff_s)
    params = tracer.make_params(rays=n, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=w.cutoff_s * 1000.0, seed=9)
    src = tracer.source_array(w.sources)
    rec = tracer.receiver_array(w.receivers)
    names = ["energy", "pressure", "dir_pos", "dir_neg", "analysis"]
    sizes = [R * 8 * T, R * 8 * T, R * 24 * T, R * 24 * T, R * 24 * T]
    bufs = [torch.full((s,), 7.0, dtype=torch.float64, device="cuda:0") for s in sizes]  # not zero on purpose
    L = _capi.lib()
    mem_after_first = None
    for call in range(2):
        st = _capi.Stats()
        rc = L.pach_trace_run_noalloc(ds.handle, src, len(w.sources), rec, len(w.receivers), C.byref(params), None,
                                      *[C.c_void_p(b.data_ptr()) for b in bufs], C.byref(st))
        _capi.check(rc)
        torch.cuda.synchronize()
        mem = (torch.cuda.mem_get_info(0)[0], torch.cuda.memory_allocated(0))
        if call == 0:
            mem_after_first = mem
        else:
            assert mem == mem_after_first, ("device memory moved across an allocation-free call", mem_after_first, mem)
        assert st.segments == st_ref["segments"], call
        assert st.primaries == n
        for name, b in zip(names, bufs):
            got = b.cpu().numpy().reshape(ref[name].shape)
            np.testing.assert_allclose(got, ref[name], rtol=1e-9, atol=1e-300, err_msg=f"{name}, call {call}")


def test_noalloc_rejects_sizes_beyond_its_limits():
    pytest.importorskip("torch")
    from pachydermacoustic_universal_gb300 import _capi, rooms, tracer

    w = rooms.shoebox_c1()
    ds = tracer.DeviceScene(w.scene)
    params = tracer.make_params(rays=10, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=2000.0)
    too_many = [rooms.ReceiverSpec((2.0 + 0.01 * i, 3.0, 2.0)) for i in range(300)]
    src = tracer.source_array(w.sources)
    rec = tracer.receiver_array(too_many)
    dummy = C.c_void_p(16)
    rc = _capi.lib().pach_trace_run_noalloc(ds.handle, src, 1, rec, len(too_many), C.byref(params), None,
                                            dummy, dummy, dummy, dummy, dummy, None)
    assert rc == 1 and "256 receivers" in _capi.last_error()


def test_noalloc_rejects_what_the_allocating_entry_point_rejects():
    pytest.importorskip("torch")
    from pachydermacoustic_universal_gb300 import _capi, rooms, tracer

    w = rooms.shoebox_c1()
    ds = tracer.DeviceScene(w.scene)
    params = tracer.make_params(rays=10, cutoff_length_m=w.cutoff_length_m, hist_cotime_ms=2000.0)
    src = tracer.source_array(w.sources)
    rec = tracer.receiver_array([rooms.ReceiverSpec((float("nan"), 3.0, 2.0))])
    dummy = C.c_void_p(16)
    rc = _capi.lib().pach_trace_run_noalloc(ds.handle, src, 1, rec, 1, C.byref(params), None,
                                            dummy, dummy, dummy, dummy, dummy, None)
    msg = _capi.last_error()
    assert rc == 1 and "origin finite" in msg
    with pytest.raises(_capi.PachError) as ei:
        tracer.Run(ds, w.sources, [rooms.ReceiverSpec((float("nan"), 3.0, 2.0))], params)
    assert msg in str(ei.value)
