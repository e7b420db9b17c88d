"""Renewal+ transverse-gradient law and 1D NEE density of the oracle.

Re-expresses tests/SparseTransverseGradientTest.cpp:24-96 of the reference on
the oracle: unconditioned moments, exact birth-gradient recovery, closed-form
transverse variance and mean, an independent dense-GP conditional (restated
here from the squared-exponential covariance and its derivatives), empirical
moments over 12000 sampled gradients and the NEE density of sampled normals.
"""
import numpy as np
import pytest

from gpis_extend_gb300 import abi
from oracle import oracle

CASES = [(0.04, 0.05), (0.02, 0.2), (0.08, 0.4)]
DIRS = [np.array([0, 0, 1], np.float32),
        (np.array([1, 2, 3], np.float32) / np.float32(np.sqrt(np.float32(14.0)))).astype(np.float32)]


def f32normalize(v):
    v = np.asarray(v, np.float32)
    s = np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
    return (v * (np.float32(1.0) / np.sqrt(s))).astype(np.float32)


def frame(n_in):
    n = f32normalize(n_in)
    sign = np.float32(np.copysign(1.0, n[2]))
    a = np.float32(-1.0) / (sign + n[2])
    b = n[0] * n[1] * a
    t = f32normalize([np.float32(1.0) + sign * n[0] * n[0] * a, sign * b, -sign * n[0]])
    bt = f32normalize([b, sign + n[1] * n[1] * a, -n[1]])
    return t, bt, n


def to_global(F, v):
    t, b, n = F
    return (t * np.float32(v[0]) + b * np.float32(v[1]) + n * np.float32(v[2])).astype(np.float32)


def to_local(F, v):
    return np.array([np.dot(F[0], v), np.dot(F[1], v), np.dot(F[2], v)])


def medium(sigma, ell):
    return abi.make_medium(sigma=sigma, length_scale=ell, kernel_scale=3.0, impulse_density=10.0,
                           seed=17429, correlation_context=abi.CTX_RENEWAL_PLUS, one_d_sampling=1,
                           sampling_scheme=abi.SCHEME_MIS, correlation_xy=1,
                           mean_kind=abi.MEAN_HOMOGENEOUS, mean_params=(0.0,))


def seeds_for(desc, pss, first):
    a, b = oracle.flight_seeds(desc, pss, 29)
    return [a, b, abi.FLAG_FIRST_SCATTER if first else 0, 0]


def dense_gp_transverse_variance(sigma, ell, origin, q_point, tangent, bitangent, rd):
    """Conditional variance of d/dtangent f(q) given f, and its gradient along
    (tangent, bitangent, rd) at the origin, for k = sigma^2 exp(-|x-y|^2 / (2 l^2))."""
    s2, l2 = sigma * sigma, ell * ell

    def k(x, y):
        d = x - y
        return s2 * np.exp(-d @ d / (2 * l2))

    def k_f_du(x, y, u):           # cov(f(x), d/du f(y))
        return k(x, y) * ((x - y) @ u) / l2

    def k_du_dv(x, y, u, v):       # cov(d/du f(x), d/dv f(y))
        d = x - y
        return k(x, y) * (u @ v / l2 - (d @ u) * (d @ v) / (l2 * l2))

    o = np.asarray(origin, np.float64)
    dirs = [None, np.asarray(tangent, np.float64), np.asarray(bitangent, np.float64), np.asarray(rd, np.float64)]
    K = np.zeros((4, 4))
    for i in range(4):
        for j in range(4):
            if dirs[i] is None and dirs[j] is None:
                K[i, j] = k(o, o)
            elif dirs[i] is None:
                K[i, j] = k_f_du(o, o, dirs[j])
            elif dirs[j] is None:
                K[i, j] = k_f_du(o, o, dirs[i])
            else:
                K[i, j] = k_du_dv(o, o, dirs[i], dirs[j])
    q = np.asarray(q_point, np.float64)
    u = dirs[1]
    cross = np.zeros(4)
    for j in range(4):
        if dirs[j] is None:
            cross[j] = -k_f_du(o, q, u)       # cov(d/du f(q), f(o)) = d/dq_u k(q, o)
        else:
            cross[j] = k_du_dv(q, o, u, dirs[j])
    prior = s2 / l2
    return prior - cross @ np.linalg.solve(K, cross)


@pytest.mark.parametrize("sigma,ell", CASES)
@pytest.mark.parametrize("di", [0, 1])
def test_transverse_law(sigma, ell, di):
    rd = DIRS[di]
    d = medium(sigma, ell)
    F = frame(rd)
    origin = np.zeros(3, np.float32)
    g0 = to_global(F, [0.3, -0.2, -0.8])
    pss = [3, 7, 1, 2]
    prev = [0.0, *g0]
    ok, mu, var = oracle.transverse_moments(d, origin, rd, origin, seeds_for(d, pss, True), prev)
    assert ok and np.all(mu == 0) and var == 0.5
    s = seeds_for(d, pss, False)
    assert oracle.sampling_scheme(d, origin, origin, s) == abi.SCHEME_UNI
    rec = oracle.gradient(d, origin, rd, origin, 0.0, s, prev)
    assert np.linalg.norm(rec.astype(np.float64) - g0) < 2e-6
    lc = np.float32(np.float32(ell) * np.sqrt(np.float32(2.0)) / np.float32(2.0))
    linv = np.float32(1.0) / lc
    for q in (0.0, 1e-7, 0.1, 0.7, 1.0, 3.0, 12.0):
        p = (rd * np.float32(q * ell)).astype(np.float32)
        ok, mu, var = oracle.transverse_moments(d, origin, rd, p, s, prev)
        assert ok
        assert abs(var - 0.5 * (-np.expm1(-q * q))) <= 3e-7
        actual = (linv * to_global(F, [np.float32(mu[0]), np.float32(mu[1]), 0.0]) * np.float32(sigma))
        expected = to_global(F, [0.3, -0.2, 0.0]) * np.float32(np.exp(-0.5 * q * q))
        assert np.linalg.norm(actual.astype(np.float64) - expected) < 1e-6
        dense = dense_gp_transverse_variance(sigma, ell, origin, p, F[0], F[1], rd)
        assert abs(var * 2 * sigma * sigma / (ell * ell) - dense) <= 3e-6 * max(1.0, abs(dense))


@pytest.mark.parametrize("sigma,ell", CASES)
@pytest.mark.parametrize("di", [0, 1])
def test_transverse_sampling_and_nee_pdf(sigma, ell, di):
    rd = DIRS[di]
    d = medium(sigma, ell)
    F = frame(rd)
    origin = np.zeros(3, np.float32)
    g0 = to_global(F, [0.3, -0.2, -0.8])
    prev = [0.0, *g0]
    t = np.float32(0.7 * ell)
    p = (rd * t).astype(np.float32)
    ok, mu, var = oracle.transverse_moments(d, origin, rd, p, seeds_for(d, [3, 7, 1, 2], False), prev)
    v = var * 2 * sigma * sigma / (ell * ell)
    expected = np.array([np.exp(-0.245) * 0.3, np.exp(-0.245) * -0.2])
    trials = 12000
    ssum = np.zeros(2)
    ssq = np.zeros(2)
    pdfs = 0
    for i in range(trials):
        s = seeds_for(d, [3, 7, i, 2], False)
        g = oracle.gradient(d, origin, rd, p, float(t), s, prev)
        loc = to_local(F, g)
        res = np.array([loc[0] - expected[0], loc[1] - expected[1]], np.float64)
        ssum += res
        ssq += res * res
        if i < 300 and loc[2] < -0.02:
            nrm = (g / np.float32(np.linalg.norm(g.astype(np.float64)))).astype(np.float32)
            cosine = abs(float(np.dot(nrm.astype(np.float64), rd)))
            density = np.exp(-(res @ res) / (2 * v)) / (2 * np.pi * v)
            exp_pdf = density * float(g.astype(np.float64) @ g) / (4 * cosine * cosine)
            pdf, _ = oracle.nee(d, origin, rd, p, nrm, float(t), s, prev)
            assert abs(pdf - exp_pdf) <= 2e-4 * max(1.0, exp_pdf), (i, pdf, exp_pdf)
            pdfs += 1
    for axis in range(2):
        assert abs(ssum[axis] / trials) <= 0.035 * np.sqrt(v)
        assert abs(ssq[axis] / trials - v) <= 0.05 * v
    assert pdfs > 40
