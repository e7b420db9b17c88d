"""The allocation-free flight entry point, gpis_flights_submit_static.

Callers such as a renderer's frame thread (which must never make the device
synchronize, as cudaMalloc and cudaFree can) or a plugin inside a host that
owns all device memory cannot allocate.  This entry point runs the same flight
kernels with its working memory in a fixed array of the library.  The test
calls it through the C ABI twice in a row -- a primary batch, then the
conditioned secondary batch that reuses the same array -- and checks both
results against gpis_flights_submit with the tolerances of the parity tests.
It lives in its own file so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from gpis_extend_gb300 import abi, runtime, workloads

pytestmark = pytest.mark.gpu

T_TOL = 1e-4 * 1.5


def static_submit(desc, dev, stream):
    lib = abi.load_library()
    soa = dev.soa()
    res = dev.result_soa()
    return lib.gpis_flights_submit_static(ctypes.byref(desc), ctypes.byref(soa), ctypes.byref(res), dev.n,
                                          ctypes.c_void_p(stream.cuda_stream))


def compare(a, b):
    ga, gb = abi.unpack_results(a), abi.unpack_results(b)
    assert np.array_equal(ga["status"], gb["status"])
    assert np.array_equal(ga["hit"], gb["hit"])
    assert np.all(np.abs(ga["t"] - gb["t"]) <= T_TOL)
    miss = ~ga["hit"]
    assert np.all(np.abs(ga["value"][miss] - gb["value"][miss]) <= 1e-5)
    ref = np.linalg.norm(gb["grad"], axis=1)
    assert np.all(np.linalg.norm(ga["grad"] - gb["grad"], axis=1) <= 2e-3 * np.maximum(ref, 1e-6))


MEDIA = {
    # 1D, one octave: the stationary cooperative fast pass and its set-up records
    "sphere_1d": (lambda: workloads.sphere_medium(), workloads.sphere_flights, 1.5),
    # 3D world-space noise: full conditioning records and the generic evaluator
    "sphere_3d": (lambda: workloads.sphere_medium(one_d=False), workloads.sphere_flights, 1.5),
    # 1D, three octaves, nonstationary length scale: the octave fast pass
    "torus_octaves": (lambda: workloads.torus_plane_medium(), workloads.torus_flights, 2.0),
}


@pytest.mark.parametrize("kind", sorted(MEDIA))
def test_static_entry_matches_context_entry_twice(kind):
    import torch
    from gpis_extend_gb300 import build
    build.build()
    assert torch.cuda.is_available()
    stream = torch.cuda.current_stream()
    make_desc, make_flights, half = MEDIA[kind]
    desc = make_desc()
    n = 2048 if kind == "sphere_3d" else 8192
    prim = make_flights(n, desc, index_offset=12345)
    with runtime.Context(desc) as ctx:
        ref1 = ctx.trace_host(prim)
        sec, _ = workloads.secondary_flights(prim, ref1, desc, half=half)
        ref2 = ctx.trace_host(sec)
    # first call: primary flights; second call: conditioned secondaries (the
    # conditioning records of the working array are rewritten by this call)
    for batch, ref in ((prim, ref1), (sec, ref2)):
        dev = runtime.DeviceFlights(batch)
        assert static_submit(desc, dev, stream) == abi.GPIS_OK, abi.load_library().gpis_last_error()
        torch.cuda.synchronize()
        compare(dev.results(), ref)


def test_static_entry_rejects_oversized_batches():
    import torch
    desc = workloads.sphere_medium()
    lib = abi.load_library()
    soa = abi.FlightSoA()
    res = abi.ResultSoA()
    rc = lib.gpis_flights_submit_static(ctypes.byref(desc), ctypes.byref(soa), ctypes.byref(res),
                                        abi.STATIC_MAX_FLIGHTS + 1,
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == abi.GPIS_ERANGE
    assert b"65536" in lib.gpis_last_error()
