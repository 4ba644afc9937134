"""pa_resample_plan_noalloc: the resampling plan for callers that cannot
allocate device memory (a host framework that has reserved the device's
memory for its own allocator, or a latency-critical loop that cannot afford
the device-wide synchronisation cudaFree implies).  Its scratch is a fixed
array in the library's device memory instead of cudaMalloc'd buffers.

The test calls it through the C ABI and checks it against the allocating
entry point pa_resample_plan on the same inputs: copy numbers, offsets and
the gather map bit for bit, lnQ and q to the same 1e-12 the stage tests use,
on two calls in a row (the second sees the first call's leftovers in the
shared array).  This file is named to be collected last."""
import ctypes

import numpy as np
import pytest

import paising_gb300 as pa

pytestmark = pytest.mark.gpu


def _energies(oracle, coding, L, R, seed, beta):
    if coding == "ssc":
        s = oracle.ssc_sweep(oracle.ssc_init(L, R, seed, 0), L, 2, beta, seed, 99)
        E, _ = oracle.ssc_energy(s, L)
        return E, None
    w, act = oracle.msc_init(L, R, seed, 0)
    w = oracle.msc_sweep(w, L, 2, beta, seed, 99)
    E, _ = oracle.msc_energy(w, L)
    return E, act


def _plan(fn, torch, E, act, coding, R, Rcap, b0, b1, e_ref, weights, seed, iseq):
    n = len(E)
    Et = torch.from_numpy(E).cuda()
    At = None if act is None else torch.from_numpy(act).cuda()
    roff = torch.empty(n, dtype=torch.int32, device="cuda")
    offs = torch.empty(n, dtype=torch.int32, device="cuda")
    src = torch.empty(Rcap + 1, dtype=torch.int32, device="cuda")
    out = (ctypes.c_double * 3)()
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    st = fn(ptr(Et), ptr(At), coding, R, R, Rcap, b0, b1, e_ref, weights, seed, iseq, ptr(roff), ptr(offs), ptr(src),
            out, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, pa.lib().pa_last_error(None)
    Rn = int(out[2])
    return (roff.cpu().numpy(), offs.cpu().numpy(), src[:Rn].cpu().numpy(), out[0], out[1], Rn)


@pytest.mark.parametrize("coding,weights", [("ssc", pa.WEIGHTS_FP64), ("msc", pa.WEIGHTS_FP32),
                                            ("msc", pa.WEIGHTS_FP64), ("ssc", pa.WEIGHTS_FP32)])
def test_noalloc_plan_matches_allocating_plan(cuda, oracle, coding, weights):
    torch = cuda
    lib = pa.lib()
    c = pa.SSC if coding == "ssc" else pa.MSC
    # two calls in a row with different populations and temperatures
    for R, L, seed, b0 in ((3000, 16, 5, 0.30), (700, 12 if coding == "msc" else 16, 6, 0.55)):
        E, act = _energies(oracle, coding, L, R, seed, b0)
        valid = E if act is None else E[act.astype(bool)]
        e_ref = float(valid.mean()) if weights == pa.WEIGHTS_FP64 else float(valid.min())
        args = (torch, E, act, c, R, 2 * R, b0, b0 + 0.01, e_ref, weights, seed, 1234)
        a = _plan(lib.pa_resample_plan, *args)
        b = _plan(lib.pa_resample_plan_noalloc, *args)
        assert b[5] == a[5]
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(x, y)
        assert b[3] == pytest.approx(a[3], rel=1e-12, abs=1e-14) and b[4] == pytest.approx(a[4], rel=1e-12)


def test_noalloc_rejects_oversize_population(cuda):
    torch = cuda
    n = 262144 + 1
    E = torch.zeros(n, dtype=torch.int32, device="cuda")
    buf = torch.empty(n, dtype=torch.int32, device="cuda")
    out = (ctypes.c_double * 3)()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = pa.lib().pa_resample_plan_noalloc(p(E), None, pa.SSC, n, n, n, 0.1, 0.2, 0.0, pa.WEIGHTS_FP32, 1, 0, p(buf),
                                           p(buf), p(buf), out, None)
    assert st == 1
    assert b"exceeds the maximum" in pa.lib().pa_last_error(None)


def test_noalloc_allocates_no_device_memory(cuda, oracle):
    """What the entry point exists for: it takes no device memory.  After a
    first call (which may load the library's device code), further calls
    leave the device's free memory unchanged to the byte -- also with most of
    that memory held by another allocation, as a caching allocator that has
    reserved the device would hold it."""
    torch = cuda
    lib = pa.lib()
    E, act = _energies(oracle, "msc", 16, 3000, 8, 0.4)
    e_ref = float(E[act.astype(bool)].min())
    args = (torch, E, act, pa.MSC, 3000, 6000, 0.4, 0.41, e_ref, pa.WEIGHTS_FP32, 8, 77)
    first = _plan(lib.pa_resample_plan_noalloc, *args)
    torch.cuda.synchronize()
    # the buffers _plan creates come from torch's cache once it holds them
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(4):
        again = _plan(lib.pa_resample_plan_noalloc, *args)
        assert np.array_equal(again[0], first[0]) and again[5] == first[5]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    hog = torch.empty(max(0, free0 - (4 << 30)), dtype=torch.uint8, device="cuda")
    try:
        free1 = torch.cuda.mem_get_info()[0]
        again = _plan(lib.pa_resample_plan_noalloc, *args)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free1
        assert np.array_equal(again[0], first[0])
    finally:
        del hog
        torch.cuda.empty_cache()
