"""1D specular next-event estimation (neeGrad / neePDF, SparseConvolutionNoise.cpp:662-821).

CPU: the oracle's PDF outside the transverse law equals the density of the
gradients its own sampler draws (the uncorrelated branch of evaluateGradientNoise1D),
and neeGrad lies on the gradient plane: its along-ray derivative is the field's.
The transverse-law branch is pinned in test_oracle_transverse.py against the
reference's analytic expectation.  GPU: gpis_nee_host against the oracle on the
hits of primary and conditioned secondary flights: PDF within 1e-3 relative on
>= 99.9 % of queries (all within 1e-2 relative or 1e-6 absolute), gradient within
1e-4 relative."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle


def frame(n):
    n = np.asarray(n, np.float64)
    n = n / np.linalg.norm(n)
    a = np.array([1.0, 0, 0]) if abs(n[0]) < 0.9 else np.array([0, 1.0, 0])
    t = np.cross(a, n)
    t /= np.linalg.norm(t)
    return t, np.cross(n, t), n


@pytest.mark.parametrize("sigma,ell", [(0.04, 0.05), (0.02, 0.2)])
def test_oracle_nee_pdf_uncorrelated_branch(sigma, ell):
    d = abi.make_medium(sigma=sigma, length_scale=ell, kernel_scale=3.0, impulse_density=10.0,
                        seed=17429, correlation_context=abi.CTX_RENEWAL_PLUS, one_d_sampling=1,
                        sampling_scheme=abi.SCHEME_MIS, correlation_xy=0,
                        mean_kind=abi.MEAN_HOMOGENEOUS, mean_params=(0.0,))
    rd = (np.array([1, 2, 3], np.float32) / np.float32(np.sqrt(14.0))).astype(np.float32)
    T, B, _ = frame(rd)
    origin = np.zeros(3, np.float32)
    t = np.float32(0.7 * ell)
    p = (rd * t).astype(np.float32)
    # world transverse variance: sigma^2 (sqrt2 / l)^2 * 1/2
    v = sigma * sigma / (ell * ell)
    n_ok = 0
    for i in range(400):
        a, b = oracle.flight_seeds(d, [5, 9, i, 1], 29)
        s = [a, b, abi.FLAG_FIRST_SCATTER, 0]
        g = oracle.gradient(d, origin, rd, p, float(t), s, (0, 0, 0, 0)).astype(np.float64)
        if float(g @ rd) >= -0.02:
            continue
        res = np.array([g @ T, g @ B])
        nrm = (g / np.linalg.norm(g)).astype(np.float32)
        cosine = abs(float(nrm.astype(np.float64) @ rd))
        density = np.exp(-(res @ res) / (2 * v)) / (2 * np.pi * v)
        want = density * float(g @ g) / (4 * cosine * cosine)
        pdf, ng = oracle.nee(d, origin, rd, p, nrm, float(t), s, (0, 0, 0, 0))
        assert abs(pdf - want) <= 2e-4 * max(1.0, want), (i, pdf, want)
        assert np.allclose(ng, g, rtol=1e-4, atol=1e-6 * np.linalg.norm(g))
        n_ok += 1
    assert n_ok > 100


@pytest.mark.parametrize("ns", [False, True])
def test_oracle_nee_gradient_on_plane(ns):
    desc = workloads.torus_plane_medium(nonstationary=ns, octaves=1) if ns else workloads.sphere_medium()
    rng = np.random.default_rng(4)
    for i in range(200):
        o = rng.uniform(-1.2, 1.2, 3).astype(np.float32)
        d = rng.normal(size=3)
        d = (d / np.linalg.norm(d)).astype(np.float32)
        p = (o + 0.3 * d).astype(np.float32)
        nrm = rng.normal(size=3)
        nrm -= 1.5 * abs(nrm @ d) * d
        nrm = (nrm / np.linalg.norm(nrm)).astype(np.float32)
        s = [int(rng.integers(2 ** 32)), int(rng.integers(2 ** 32)), 0 if i % 2 else abi.FLAG_FIRST_SCATTER, 0]
        prev = [0.0, *rng.normal(size=3)]
        _, g = oracle.nee(desc, o, d, p, nrm, 0.3, s, prev)
        fg = oracle.gradient(desc, o, d, p, 0.3, s, prev)
        a, b = float(g.astype(np.float64) @ d), float(fg.astype(np.float64) @ d)
        assert abs(a - b) <= 1e-4 * max(1.0, abs(b)), (i, a, b)
        assert np.allclose(np.cross(g, nrm), 0, atol=1e-5 * max(1.0, np.linalg.norm(g)))


def nee_queries(desc, batch, rec, seed):
    """Hits of a traced batch with a random normal facing the ray (dot(n, -d) > 0)."""
    r = abi.unpack_results(rec)
    idx = np.nonzero(r["hit"] & (r["status"] == abi.FLIGHT_OK))[0]
    sub = batch.subset(idx)
    o = sub.origin_near[:, :3].astype(np.float64)
    d = sub.dir_far[:, :3].astype(np.float64)
    t = r["t"][idx].astype(np.float64)
    p = (o + d * t[:, None]).astype(np.float32)
    rng = np.random.default_rng(seed)
    light = rng.normal(size=(len(idx), 3))
    light /= np.linalg.norm(light, axis=1, keepdims=True)
    light[np.sum(light * d, axis=1) > 0] *= -1
    h = -d + light
    h /= np.linalg.norm(h, axis=1, keepdims=True)
    return sub, p, r["t"][idx].astype(np.float32), h.astype(np.float32)


def compare_nee(desc, sub, p, t, nrm, out):
    n = sub.n
    pdf_c = np.zeros(n)
    g_c = np.zeros((n, 3))
    for i in range(n):
        pdf_c[i], g_c[i] = oracle.nee(desc, sub.origin_near[i, :3], sub.dir_far[i, :3], p[i], nrm[i],
                                      float(t[i]), sub.seeds[i], sub.prev[i])
    pdf_g = out[:, 0].astype(np.float64)
    assert np.all(np.isfinite(pdf_g))
    err = np.abs(pdf_g - pdf_c)
    rel_ok = err <= 1e-3 * np.maximum(pdf_c, 1e-9)
    assert rel_ok.mean() >= 0.999, np.sort(err / np.maximum(pdf_c, 1e-9))[-8:]
    assert np.all((err <= 1e-2 * pdf_c) | (err <= 1e-6))
    gn = np.linalg.norm(g_c, axis=1)
    gerr = np.linalg.norm(out[:, 1:] - g_c, axis=1)
    assert np.mean(gerr <= 1e-4 * np.maximum(gn, 1e-3)) >= 0.999
    return int((pdf_c > 0).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["sphere_xy", "sphere", "torus_ns", "torus_ns_xy", "torus_mr", "torus_mr_xy",
                                  "torus_oct", "torus_oct_xy"])
def test_gpu_nee_vs_oracle(case):
    from gpis_extend_gb300 import runtime
    if case.startswith("sphere"):
        desc = workloads.sphere_medium(sampling_scheme=abi.SCHEME_MIS, correlation_xy=int(case.endswith("xy")))
    else:
        desc = workloads.torus_plane_medium(nonstationary=True, octaves=3 if case.startswith("torus_oct") else 1,
                                            sampling_scheme=abi.SCHEME_MIS, correlation_xy=int(case.endswith("xy")),
                                            multires=int(case.startswith("torus_mr")))
    prim = workloads.sphere_flights(1 << 11, desc)
    with runtime.Context(desc) as ctx:
        rec = oracle.trace_flights(desc, prim)
        sub, p, t, nrm = nee_queries(desc, prim, rec, 1)
        out = ctx.nee(sub, p, t, nrm)
        positive = compare_nee(desc, sub, p, t, nrm, out)
        sec, _ = workloads.secondary_flights(prim, rec, desc)
        rec2 = oracle.trace_flights(desc, sec)
        sub2, p2, t2, nrm2 = nee_queries(desc, sec, rec2, 2)
        out2 = ctx.nee(sub2, p2, t2, nrm2)
        positive += compare_nee(desc, sub2, p2, t2, nrm2, out2)
    assert positive > 100


@pytest.mark.gpu
def test_gpu_nee_rejects_3d_and_bad_inputs():
    from gpis_extend_gb300 import runtime
    d3 = workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL)
    prim = workloads.sphere_flights(64, d3)
    p = prim.origin_near[:, :3].copy()
    nrm = -prim.dir_far[:, :3].copy()
    with runtime.Context(d3) as ctx:
        out = ctx.nee(prim, p, np.zeros(64, np.float32), nrm)
    assert np.all(np.isnan(out[:, 0]))
    d1 = workloads.sphere_medium()
    prim = workloads.sphere_flights(64, d1)
    p = prim.origin_near[:, :3].copy()
    p[3, 1] = np.inf
    nrm = -prim.dir_far[:, :3].copy()
    with runtime.Context(d1) as ctx:
        out = ctx.nee(prim, p, np.zeros(64, np.float32), nrm)
        assert np.isnan(out[3, 0]) and np.sum(np.isnan(out[:, 0])) == 1
        empty = abi.FlightBatch(0)
        assert ctx.nee(empty, np.zeros((0, 3)), np.zeros(0), np.zeros((0, 3))).shape == (0, 4)
