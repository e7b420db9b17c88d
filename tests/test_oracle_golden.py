"""Pins of the oracle (CPU restatement) against the reference.

* Bit-exact against golden vectors written by the reference's own hash, PCG,
  Box-Muller and tangent-frame code (tests/golden/reference_primitives.json).
* The known answers of src/gpu/tests/RaySegmentBatchTest.cpp (plane mean,
  Renewal+ continuity, 73 seeded noise values) and of
  src/gpu/tests/SeSplat1DTest.cpp, re-expressed on the oracle.
"""
import json
import os

import numpy as np
import pytest

from gpis_extend_gb300 import abi, hashing
from oracle import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_primitives.json")))


def f32(bits):
    return np.array([bits], np.uint32).view(np.float32)[0]


def f64(bits):
    return np.array([int(bits)], np.uint64).view(np.float64)[0]


def test_xxhash32_matches_reference():
    for x, h in GOLD["xxhash32_1"]:
        assert oracle.lib().gor_xxhash32_1(x) == h
    for x, y, h in GOLD["xxhash32_2"]:
        assert oracle.lib().gor_xxhash32_2(x, y) == h
    for a, b, c, d, h in GOLD["xxhash32_4"]:
        assert oracle.lib().gor_xxhash32_4(a, b, c, d) == h
    # the numpy host hash used for flight seeds agrees too
    x = np.array([r[0] for r in GOLD["xxhash32_1"]], np.uint32)
    assert np.array_equal(hashing.xxhash32_1(x), np.array([r[1] for r in GOLD["xxhash32_1"]], np.uint32))
    g4 = np.array(GOLD["xxhash32_4"], np.uint64).astype(np.uint32)
    assert np.array_equal(hashing.xxhash32_4(g4[:, 0], g4[:, 1], g4[:, 2], g4[:, 3]), g4[:, 4])
    g2 = np.array(GOLD["xxhash32_2"], np.uint64).astype(np.uint32)
    assert np.array_equal(hashing.xxhash32_2(g2[:, 0], g2[:, 1]), g2[:, 2])


def test_pcg_stream_matches_reference():
    for row in GOLD["pcg_next1d"]:
        state = int(row[0])
        f, _ = oracle.pcg_stream(state, 12)
        assert list(f.view(np.uint32)) == row[1:]


def test_cell_impulses_1d_bit_exact():
    for cell, seed, flat in GOLD["cell1d"]:
        pos, w = oracle.cell_1d(cell, seed, 8)
        ref = np.array(flat, np.uint32).reshape(8, 2)
        assert np.array_equal(pos.view(np.uint32), ref[:, 0])
        assert np.array_equal(w.view(np.uint32), ref[:, 1])


def test_cell_impulses_3d_bit_exact_in_pinned_order():
    """next3D order as g++ evaluates Vec3f(next1D(), next1D(), next1D()): right to left."""
    for i, j, k, seed, flat in GOLD["cell3d"]:
        pos, w = oracle.cell_3d(i, j, k, seed, 8, order=0)
        ref = np.array(flat, np.uint32).reshape(8, 4)
        assert np.array_equal(pos.view(np.uint32), ref[:, :3])
        assert np.array_equal(w.view(np.uint32), ref[:, 3])


def test_box_muller_matches_reference():
    for row in GOLD["normal4"]:
        z = oracle.normal_pairs(row[0], 2)
        ref = np.array([f64(b) for b in row[1:]])
        assert np.allclose(z, ref, rtol=4e-16, atol=0), (z, ref)


def test_tangent_frame_matches_reference():
    """The frame enters through the 1D coordinate; checked via the oracle's gradient
    transport: toGlobal(e_z) of the frame must equal the normalised direction."""
    for row in GOLD["tangent_frame"]:
        v = np.array(row[:3], np.uint32).view(np.float32)
        t = np.array(row[3:6], np.uint32).view(np.float32)
        b = np.array(row[6:9], np.uint32).view(np.float32)
        n = np.array(row[9:12], np.uint32).view(np.float32)
        # restate the float32 construction in numpy with the reference operation order
        n2 = _normalize_f32(v)
        sign = np.float32(np.copysign(np.float32(1.0), n2[2]))
        a = np.float32(-1.0) / (sign + n2[2])
        bb = n2[0] * n2[1] * a
        t2 = _normalize_f32(np.array([np.float32(1.0) + sign * n2[0] * n2[0] * a, sign * bb, -sign * n2[0]], np.float32))
        b2 = _normalize_f32(np.array([bb, sign + n2[1] * n2[1] * a, -n2[1]], np.float32))
        assert np.array_equal(n2.view(np.uint32), n.view(np.uint32))
        assert np.array_equal(t2.view(np.uint32), t.view(np.uint32))
        assert np.array_equal(b2.view(np.uint32), b.view(np.uint32))


def _normalize_f32(v):
    v = np.asarray(v, np.float32)
    s = v[0] * v[0]
    s = np.float32(s + v[1] * v[1])
    s = np.float32(s + v[2] * v[2])
    inv = np.float32(1.0) / np.sqrt(np.float32(s))
    return (v * inv).astype(np.float32)


def plane_grid_medium(amplitude, step=0.05):
    """The 8^3 plane grid of RaySegmentBatchTest.cpp:26-42: mean = x - 2.5."""
    vox = np.zeros((8, 8, 8), np.float32)
    vox[:, :, :] = np.arange(8, dtype=np.float32)[None, None, :] - 2.5
    grid = abi.make_mean_grid(vox)
    d = abi.make_medium(sigma=amplitude, length_scale=1.0, kernel_scale=3.0, impulse_density=3.0,
                        one_d_sampling=1, correlation_context=abi.CTX_RENEWAL_PLUS,
                        step_size=step, min_step=8)
    return abi.attach_grid(d, grid)


def ray_batch(origins, dirs, near, far, jitter, noise_seeds, normal_seeds, first, prev=None):
    n = len(origins)
    b = abi.FlightBatch(n)
    b.origin_near[:, :3] = origins
    b.origin_near[:, 3] = near
    b.dir_far[:, :3] = dirs
    b.dir_far[:, 3] = far
    b.seeds[:, 0] = noise_seeds
    b.seeds[:, 1] = normal_seeds
    b.seeds[:, 2] = abi.FLAG_FIRST_SCATTER if first else 0
    b.set_jitter(np.full(n, jitter, np.float32))
    if prev is not None:
        b.prev[:] = prev
    return b


def plane_known_answer_batch(n=513):
    i = np.arange(n)
    dirs = np.where((i % 2 == 0)[:, None], [[1, 0, 0]], [[-1, 0, 0]]).astype(np.float32)
    return ray_batch(np.tile([0.0, 3.0, 3.0], (n, 1)), dirs, 0.0, 5.0, 0.2,
                     123 + i, 456 + i, True)


def test_oracle_plane_known_answer():
    """RaySegmentBatchTest.cpp:82-119: hit at t=2.5+-0.01 with grad.x=1+-0.002 for +x
    rays; miss with t=5 and value -2.5+-1e-5 for -x rays (amplitude 0)."""
    d = plane_grid_medium(0.0)
    r = abi.unpack_results(oracle.trace_flights(d, plane_known_answer_batch()))
    even = np.arange(513) % 2 == 0
    assert np.all(r["status"] == abi.FLIGHT_OK)
    assert np.all(r["hit"][even]) and not np.any(r["hit"][~even])
    assert np.all(np.abs(r["t"][even] - 2.5) <= 0.01)
    assert np.all(np.abs(r["grad"][even, 0] - 1.0) <= 0.002)
    assert np.all(r["t"][~even] == 5.0)
    assert np.all(np.abs(r["value"][~even] + 2.5) <= 1e-5)


def test_oracle_renewal_plus_continuity():
    """RaySegmentBatchTest.cpp:121-142: a conditioned segment of length 1e-3 keeps
    the birth value 0.9 within 0.005."""
    d = plane_grid_medium(0.1)
    b = ray_batch([[3.0, 3.0, 3.0]], [[1, 0, 0]], 0.0, 0.001, 0.2, [123], [456], False,
                  prev=[[0.9, 1.2, 0.0, 0.0]])
    r = abi.unpack_results(oracle.trace_flights(d, b))
    assert r["status"][0] == abi.FLIGHT_OK and not r["hit"][0]
    assert abs(r["value"][0] - 0.9) <= 0.005


def test_oracle_seeded_noise_known_answer():
    """RaySegmentBatchTest.cpp:144-175: value at x=5.001 = 2.501 + 0.2 * noise(seed)
    within 3e-5 over 73 seeds; the FP64 field agrees with the reference sum to 2e-6."""
    d = plane_grid_medium(0.2)
    seeds = np.array([r[0] for r in GOLD["se_noise_1d_seeds"]], np.uint32)
    expect = np.array([f64(r[1]) for r in GOLD["se_noise_1d_seeds"]])
    n = len(seeds)
    b = ray_batch(np.tile([5.0, 3.0, 3.0], (n, 1)), np.tile([1, 0, 0], (n, 1)), 0.0, 0.001, 0.2,
                  seeds, np.full(n, 456), True)
    r = abi.unpack_results(oracle.trace_flights(d, b))
    assert np.all(r["status"] == abi.FLIGHT_OK) and not np.any(r["hit"])
    assert np.all(np.abs(r["value"] - (2.501 + 0.2 * expect)) <= 3e-5)
    for s, e in zip(seeds, expect):
        out = oracle.field(d, [5, 3, 3], [1, 0, 0], [5.001, 3, 3], [s, 456, 1, 0], double_mode=True)
        assert abs(out[0] - e) <= 2e-6


def test_oracle_se_splat_expectation():
    """SeSplat1DTest.cpp:31-84 inputs; the FP64 expectation used for the GPU splat."""
    i = np.arange(1025)
    q = ((i % 31) - 15).astype(np.float32) * np.float32(0.1)
    c = ((i % 7) - 3).astype(np.float32) * np.float32(0.2)
    q[0] = c[0]
    v, dv = oracle.se_splat_1d(q, c, 0.7)
    delta = q.astype(np.float64) - c
    assert np.allclose(v, np.exp(-delta ** 2 / (2 * 0.7 * 0.7)), atol=1e-15)
    assert v[0] == 1.0 and dv[0] == 0.0


def test_flight_seeds_formula():
    d = abi.make_medium(seed=1, correlation_context=abi.CTX_RENEWAL_PLUS)
    pss = np.array([[5, 9, 0, 3]], np.uint32)
    from gpis_extend_gb300 import workloads
    ns, nm = workloads.pss_seeds(d, pss, 1)
    a, b = oracle.flight_seeds(d, pss[0], 1)
    assert (int(ns[0]), int(nm[0])) == (a, b)
    h = oracle.lib().gor_xxhash32_4(5, 9, 0, 3) + oracle.lib().gor_xxhash32_1(1)
    assert a == (1 + h) & 0xFFFFFFFF and b == (h + 1) & 0xFFFFFFFF
    # Global memory zeroes the bounce word of the noise seed only
    g = abi.make_medium(seed=1, correlation_context=abi.CTX_GLOBAL)
    a2, b2 = oracle.flight_seeds(g, pss[0], 1)
    assert a2 == (1 + oracle.lib().gor_xxhash32_4(5, 9, 0, 0) + oracle.lib().gor_xxhash32_1(1)) & 0xFFFFFFFF
    assert b2 == b
