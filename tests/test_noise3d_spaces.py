"""3D noise outside the stationary world form: isotropic ray space
(isotropic_3D_sampling, evaluateNoise3DIsotropicRayNormalized), the brute-force
nonstationary length scale and the multi-resolution grid, in world and in
isotropic space (evaluateNoise3D, SparseConvolutionNoise.cpp:142-165, 308-377;
conditioning3D, :498-574).

CPU: the oracle's conditioning meets the birth value and the birth gradient of
the 3D field at the origin, its float and FP64 evaluations agree, and the
unconditioned normalized noise has unit variance.  GPU: noise values within 1e-5
of the FP64 anchor, the precise evaluator bit-exact with the oracle's float
evaluation on >= 99 % of points, and flights against the oracle with the bars of
the stationary parity tests."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle

MEDIA = {
    "iso": lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL_PLUS, isotropic_3d_sampling=1),
    "iso_aniso": lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL_PLUS, isotropic_3d_sampling=1,
                                                 aniso=(1.0, 0.6, 1.4)),
    "ns": lambda: workloads.torus_plane_medium(nonstationary=True, octaves=1, one_d_sampling=0),
    "ns_iso": lambda: workloads.torus_plane_medium(nonstationary=True, octaves=1, one_d_sampling=0,
                                                   isotropic_3d_sampling=1),
    "mr": lambda: workloads.torus_plane_medium(nonstationary=True, octaves=1, one_d_sampling=0, multires=1),
    "mr_iso": lambda: workloads.torus_plane_medium(nonstationary=True, octaves=1, one_d_sampling=0, multires=1,
                                                   isotropic_3d_sampling=1),
}


def points(n, rng, half=1.2):
    o = rng.uniform(-half, half, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    seeds = np.zeros((n, 4), np.uint32)
    seeds[:, 0] = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    seeds[:, 1] = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    prev = np.zeros((n, 4), np.float32)
    prev[:, 0] = rng.normal(scale=0.02, size=n)
    prev[:, 1:] = rng.normal(size=(n, 3))
    return o, d, seeds, prev


@pytest.mark.parametrize("name", sorted(MEDIA))
def test_oracle_conditioning_meets_birth_state_3d(name):
    desc = MEDIA[name]()
    rng = np.random.default_rng(sum(map(ord, name)))
    o, d, seeds, prev = points(60, rng)
    for i in range(len(o)):
        f = oracle.field(desc, o[i], d[i], o[i], seeds[i], prev[i])
        assert abs(f[4] - prev[i, 0]) <= 2e-6 * (1 + abs(prev[i, 0])), (i, f[4], prev[i, 0])
        g = oracle.gradient(desc, o[i], d[i], o[i], 0.0, seeds[i], prev[i])
        assert np.abs(g - prev[i, 1:]).max() <= 1e-5 * (1 + np.abs(prev[i, 1:]).max()), (i, g, prev[i, 1:])


@pytest.mark.parametrize("name", sorted(MEDIA))
def test_oracle_float_mode_matches_fp64_3d(name):
    desc = MEDIA[name]()
    rng = np.random.default_rng(7 + len(name))
    o, d, seeds, prev = points(40, rng)
    seeds[:20, 2] = abi.FLAG_FIRST_SCATTER
    for i in range(len(o)):
        p = (o[i] + 0.07 * d[i]).astype(np.float32)
        a = oracle.field(desc, o[i], d[i], p, seeds[i], prev[i])
        b = oracle.field(desc, o[i], d[i], p, seeds[i], prev[i], double_mode=True)
        assert abs(a[0] - b[0]) <= 1e-5 * max(1.0, abs(b[0])), (i, a[0], b[0])
        assert np.abs(a[1:4] - b[1:4]).max() <= 2e-5 * max(1.0, np.abs(b[1:4]).max()), (i, a[1:4], b[1:4])


@pytest.mark.parametrize("name", ["iso", "mr_iso"])
def test_oracle_unconditioned_noise_has_unit_variance_3d(name):
    """The normalisation of isotropic-space noise: over independent realizations the
    normalized noise has mean 0 and variance 1 (within sampling error)."""
    desc = MEDIA[name]()
    rng = np.random.default_rng(3)
    o, d, seeds, prev = points(1500, rng)
    seeds[:, 2] = abi.FLAG_FIRST_SCATTER
    v = np.array([oracle.field(desc, o[i], d[i], o[i], seeds[i], prev[i])[0] for i in range(len(o))])
    assert abs(v.mean()) < 0.12 and 0.8 < v.var() < 1.2, (v.mean(), v.var())


def test_json_accepts_isotropic_3d_sampling():
    import ctypes
    from gpis_extend_gb300 import build
    build.build()
    lib = abi.load_library()
    js = b'''{"correlation_context": "renewal", "1D_sampling": false, "isotropic_3D_sampling": true,
       "gaussian_process": {"mean": {"type": "spherical", "center": [0, 0, 0], "radius": 1.0},
       "covariance": {"type": "squared_exponential", "sigma": 0.05, "lengthScale": 0.1}}}'''
    d = abi.MediumDesc()
    assert lib.gpis_medium_desc_from_json(js, ctypes.byref(d)) == 0, lib.gpis_last_error()
    assert d.isotropic_3d_sampling == 1 and d.one_d_sampling == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MEDIA))
def test_gpu_noise3d_spaces_vs_fp64(name):
    """Noise value within 1e-5 (and gradient within 2e-4) of the oracle's FP64
    evaluation of the same impulse set, unconditioned and conditioned."""
    from gpis_extend_gb300 import build, runtime
    build.build()
    desc = MEDIA[name]()
    rng = np.random.default_rng(100 + len(name))
    n = 400
    o, d, seeds, prev = points(n, rng)
    seeds[: n // 2, 2] = abi.FLAG_FIRST_SCATTER
    t = rng.uniform(0.0, 0.4, n)
    p = (o.astype(np.float64) + d * t[:, None]).astype(np.float32)
    with runtime.Context(desc) as ctx:
        out = ctx.debug_field(o, p, d, seeds, prev)
    for i in range(n):
        ref = oracle.field(desc, o[i], d[i], p[i], seeds[i], prev[i], double_mode=True)
        assert abs(out[i, 0] - ref[0]) <= 1e-5 * max(1.0, abs(ref[0])), (name, i, out[i, 0], ref[0])
        assert np.abs(out[i, 1:4] - ref[1:4]).max() <= 2e-4 * max(1.0, np.abs(ref[1:4]).max()), (name, i)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MEDIA))
def test_gpu_precise_field_3d_spaces_matches_oracle(name):
    """The precise evaluator against the oracle's float field value, unconditioned
    and conditioned (origins included): bit-exact on >= 99 % of the points, within
    8 ulp of the field scale on all."""
    from gpis_extend_gb300 import build, runtime
    build.build()
    desc = MEDIA[name]()
    rng = np.random.default_rng(200 + len(name))
    n = 600
    o, d, seeds, prev = points(n, rng)
    seeds[: n // 2, 2] = abi.FLAG_FIRST_SCATTER
    t = rng.uniform(0.0, 0.4, n)
    t[n // 2: n // 2 + n // 8] = 0.0
    p = (o.astype(np.float64) + d * t[:, None]).astype(np.float32)
    with runtime.Context(desc) as ctx:
        out = ctx.debug_field(o, p, d, seeds, prev)
    ref = np.array([oracle.field(desc, o[i], d[i], p[i], seeds[i], prev[i])[4] for i in range(n)], np.float32)
    exact = out[:, 6] == ref
    ulp = np.spacing(np.maximum(np.abs(ref), np.float32(desc.sigma)))
    err = np.abs(out[:, 6].astype(np.float64) - ref) / ulp
    print(name, "bit-exact", exact.mean(), "max ulp", err.max())
    assert np.all(err <= 8), (name, err.max())
    assert exact.mean() >= 0.99, (name, exact.mean())


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MEDIA))
def test_gpu_flights_3d_spaces_vs_oracle(name):
    """Primary flights and the conditioned secondaries at their hits on both paths."""
    from gpis_extend_gb300 import build, runtime
    from test_gpu_parity import flights_vs_oracle
    build.build()
    desc = MEDIA[name]()
    sphere = name.startswith("iso")
    make, half = (workloads.sphere_flights, 1.5) if sphere else (workloads.torus_flights, 2.0)
    prim = make(1 << 12, desc)
    with runtime.Context(desc) as ctx:
        rec = ctx.trace_host(prim)
        rec_cpu, st = flights_vs_oracle(desc, prim, rec, scene=half)
        assert st["hits"] > 100
        sec, _ = workloads.secondary_flights(prim, rec_cpu, desc, half=half)
        rec2 = ctx.trace_host(sec)
        flights_vs_oracle(desc, sec, rec2, scene=half)
