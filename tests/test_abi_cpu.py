"""CPU-side checks of the C ABI library: it builds for sm_103a, loads without a
GPU, exports every symbol include/gpis.h declares, and its host-only entry
points (defaults, JSON medium parsing, flight seeds) agree with the reference
semantics.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from gpis_extend_gb300 import abi, build, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.load_library()


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gpis_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_medium_defaults_match(lib):
    d = abi.MediumDesc()
    lib.gpis_medium_desc_init(ctypes.byref(d))
    ref = abi.medium_defaults()
    assert bytes(d) == bytes(ref)
    assert ctypes.sizeof(abi.MediumDesc) % 8 == 0


def test_medium_from_json(lib):
    js = b'''{"type": "sparse_conv_noise", "sigma_a": 0.2, "sigma_s": 0.8,
      "correlation_context": "renewal+", "1D_sampling": true, "1D_sampling_scheme": "MIS",
      "step_size": 0.01, "min_step": 8, "seed": 1, "impulse_density": 8,
      "1D_gradient_correlationXY": true,
      "gaussian_process": {"type": "standard",
         "mean": {"type": "spherical", "center": [0, 0, 0], "radius": 1.0},
         "covariance": {"type": "squared_exponential", "sigma": 0.05, "lengthScale": 0.1}}}'''
    d = abi.MediumDesc()
    assert lib.gpis_medium_desc_from_json(js, ctypes.byref(d)) == 0
    assert abs(d.sigma - 0.05) < 1e-7 and abs(d.length_scale - 0.1) < 1e-7
    assert d.one_d_sampling == 1 and d.sampling_scheme == abi.SCHEME_MIS and d.correlation_xy == 1
    assert d.correlation_context == abi.CTX_RENEWAL_PLUS and d.seed == 1 and d.impulse_density == 8
    assert d.mean_kind == abi.MEAN_SPHERE and d.mean_params[3] == 1.0
    # the reference rejects a missing correlation context ("goldfish")
    assert lib.gpis_medium_desc_from_json(b'{"type": "sparse_conv_noise"}', ctypes.byref(d)) == abi.GPIS_EINVAL
    assert b"goldfish" in lib.gpis_last_error()
    assert lib.gpis_medium_desc_from_json(b'{"correlation_context": "renewal", "intersect_method": "mean"}',
                                          ctypes.byref(d)) == abi.GPIS_ENOTSUP
    assert lib.gpis_medium_desc_from_json(b'{not json', ctypes.byref(d)) == abi.GPIS_EINVAL
    # torus union plane via csg
    js = b'''{"correlation_context": "renewal", "gaussian_process": {"type": "csg",
       "left": {"mean": {"type": "torus", "major_radius": 1.0, "minor_radius": 0.35}},
       "right": {"mean": {"type": "linear", "reference_point": [0, -0.5, 0], "direction": [0, 1, 0]}}}}'''
    assert lib.gpis_medium_desc_from_json(js, ctypes.byref(d)) == 0, lib.gpis_last_error()
    assert d.mean_kind == abi.MEAN_TORUS_PLANE and abs(d.mean_params[5] + 0.5) < 1e-7


def test_flight_seeds_agree(lib):
    d = workloads.sphere_medium()
    pss = (ctypes.c_uint32 * 4)(17, 3, 0, 1)
    a, b = ctypes.c_uint32(), ctypes.c_uint32()
    lib.gpis_flight_seeds(ctypes.byref(d), pss, 1, ctypes.byref(a), ctypes.byref(b))
    ns, nm = workloads.pss_seeds(d, np.array([[17, 3, 0, 1]], np.uint32), 1)
    assert (a.value, b.value) == (int(ns[0]), int(nm[0]))


def test_ctx_create_fails_loudly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    d = workloads.sphere_medium()
    h = ctypes.c_void_p()
    rc = lib.gpis_ctx_create(ctypes.byref(d), 1, ctypes.byref(h))
    assert rc == abi.GPIS_ENODEV and not h.value


def test_static_entry_rejects_misaligned_streams_before_launch(lib):
    # a stream pointer offset by 4 bytes (a sub-slice of a float buffer) is refused
    # with GPIS_EINVAL before the entry point touches the device; the addresses are
    # never dereferenced
    d = workloads.sphere_medium()
    soa = abi.FlightSoA()
    res = abi.ResultSoA()
    soa.origin_near = 0x10000
    soa.dir_far = 0x20000 + 4
    soa.seeds = 0x30000
    soa.prev = 0x40000
    res.rec = 0x50000
    rc = lib.gpis_flights_submit_static(ctypes.byref(d), ctypes.byref(soa), ctypes.byref(res), 128, None)
    assert rc == abi.GPIS_EINVAL
    assert b"16-byte" in lib.gpis_last_error()
