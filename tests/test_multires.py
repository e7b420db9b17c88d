"""The multi-resolution grid of a nonstationary length scale (kernelScaleLevelRatio
and the two-level blend, SparseConvolutionNoise.cpp:101-111, 156-165, 244-295,
379-417, 576-656, 687-808).

CPU: the blend is the level-weighted sum of two stationary fields at the level
length scales with the levels' seed offsets; the level weights have unit total
variance; the conditioned field meets the birth value (and the birth gradient
under Renewal+); NEE on a mirror GP surface is unbiased against the plain
estimator; unsupported combinations are refused.  GPU: the flights, field,
NEE and a mirror render against the oracle (the field, flight and NEE bars are
in test_nonstationary and test_nee, which run this medium too)."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle
from test_nonstationary import birth_points


def mr_medium(**kw):
    return workloads.torus_plane_medium(nonstationary=True, octaves=1, multires=1, **kw)


def test_oracle_level_weights():
    desc = mr_medium()
    rng = np.random.default_rng(1)
    for p in rng.uniform(-1.5, 1.5, (200, 3)).astype(np.float32):
        info, seeds = oracle.level_ratio(desc, p)
        ls = 0.11 + 0.09 * np.sin(3.0 * p[0]) * np.cos(2.0 * p[2])
        assert info[0] <= ls * (1 + 1e-6) and ls <= info[1] * (1 + 1e-6)
        assert np.isclose(info[1] / info[0], 2.5, rtol=1e-6)
        assert abs(info[2] ** 2 + info[3] ** 2 - 1.0) < 1e-6
        assert seeds[1] == (int(seeds[0]) + 1) & 0xFFFFFFFF
        # the level index of scale 2.5^L is L: the offsets are small negative integers here
        assert -6 <= np.int32(seeds[0]) <= -1


def test_oracle_blend_of_stationary_levels():
    """Unconditioned, the noise is w_low n(l_low, seed + L_low) + w_high n(l_high, seed + L_high)
    with n the stationary field of length scale l; the coordinates differ by float
    rounding only (l_inv p / s against (1 / l) p)."""
    desc = mr_medium()
    rng = np.random.default_rng(3)
    o, d, seeds, prev = birth_points(120, rng)
    seeds[:, 2] = abi.FLAG_FIRST_SCATTER
    for i in range(len(o)):
        p = (o[i] + 0.3 * d[i]).astype(np.float32)
        info, lseed = oracle.level_ratio(desc, p)
        total = oracle.field(desc, o[i], d[i], p, seeds[i], prev[i])[0]
        parts = []
        for s, off in zip(info[:2], lseed):
            st = workloads.torus_plane_medium(nonstationary=False, octaves=1, length_scale=float(s))
            sd = seeds[i].copy()
            sd[0] = (int(sd[0]) + int(off)) & 0xFFFFFFFF
            parts.append(oracle.field(st, o[i], d[i], p, sd, prev[i])[0])
        assert abs(total - (info[2] * parts[0] + info[3] * parts[1])) <= 1e-4, (i, total, parts, info)


@pytest.mark.parametrize("context,xy", [(abi.CTX_RENEWAL_PLUS, 0), (abi.CTX_RENEWAL_PLUS, 1), (abi.CTX_RENEWAL, 0)])
def test_oracle_conditioning_meets_birth(context, xy):
    desc = mr_medium(context=context, correlation_xy=xy)
    rng = np.random.default_rng(7 + xy)
    o, d, seeds, prev = birth_points(150, rng)
    for i in range(len(o)):
        f = oracle.field(desc, o[i], d[i], o[i], seeds[i], prev[i])
        assert abs(f[4] - prev[i, 0]) <= 2e-6 * (1 + abs(prev[i, 0]))
        if context != abi.CTX_RENEWAL_PLUS:
            continue
        g = oracle.gradient(desc, o[i], d[i], o[i], 0.0, seeds[i], prev[i]).astype(np.float64)
        want = prev[i, 1:].astype(np.float64)
        if xy:
            assert np.abs(g - want).max() <= 2e-4 * (1 + np.abs(want).max())
        else:
            assert abs(g @ d[i] - want @ d[i]) <= 2e-4 * (1 + abs(want @ d[i]))


def test_oracle_rejects_unsupported():
    with pytest.raises(abi.GpisError):          # octaves on the grid
        oracle.field(workloads.torus_plane_medium(nonstationary=True, octaves=3, multires=1),
                     [0, 0, 0], [0, 0, 1], [0, 0, 0.1], [1, 2, 1, 0])
    with pytest.raises(abi.GpisError):          # ls(p) reaches 0
        oracle.field(mr_medium(ls_params=(0.1, 0.1, 3.0, 2.0)), [0, 0, 0], [0, 0, 1], [0, 0, 0.1], [1, 2, 1, 0])
    # a stationary covariance ignores the flag (_multiResolutionGrid needs a nonstationary kernel)
    st = workloads.torus_plane_medium(nonstationary=False, octaves=1)
    st_mr = workloads.torus_plane_medium(nonstationary=False, octaves=1, multires=1)
    a = oracle.field(st, [0, 0, 0], [0, 0, 1], [0.3, 0.1, 0.2], [1, 2, 1, 0])
    b = oracle.field(st_mr, [0, 0, 0], [0, 0, 1], [0.3, 0.1, 0.2], [1, 2, 1, 0])
    assert np.array_equal(a, b)


def test_oracle_nee_unbiased_on_the_grid():
    """neePDF's multi-resolution law (:776-808) is the density of the blended
    gradient: NEE and plain mirror renders agree in the mean."""
    means = {}
    for kind in ("torus_mr", "torus_mr_nee"):
        desc = workloads.render_medium(kind)
        m = []
        for seed in range(6):
            sc = workloads.render_scene(width=16, height=16, spp=96, phase="mirror", max_bounces=2,
                                        sampler_seed=200 + seed, box_half=2.0)
            m.append(oracle.render(desc, sc)[0].mean())
        means[kind] = np.array(m, np.float64)
    uni, nee = means["torus_mr"], means["torus_mr_nee"]
    se = np.sqrt(uni.var(ddof=1) / len(uni) + nee.var(ddof=1) / len(nee))
    assert abs(uni.mean() - nee.mean()) <= 4 * se, (uni, nee)


@pytest.mark.gpu
def test_gpu_multires_render_matches_restatement():
    from gpis_extend_gb300 import runtime
    desc = workloads.render_medium("torus_mr_nee")
    sc = workloads.render_scene(width=32, height=32, spp=4, max_bounces=4, phase="conductor", box_half=2.0)
    with runtime.Context(desc) as ctx:
        g, gs = ctx.render(sc)
    c, cs = oracle.render(desc, sc)
    close = np.all(np.abs(g - c) <= 1e-3 * np.abs(c) + 1e-7, axis=2)
    print("multires pixels within 1e-3", close.mean(), "means", g.mean(), c.mean(), gs, cs)
    assert close.mean() >= 0.99
    assert abs(g.mean() - c.mean()) <= 0.005 * c.mean()
    for k in ("distance_flights", "shadow_flights", "medium_events"):
        assert abs(gs[k] - cs[k]) <= 0.01 * cs[k] + 2, k
    assert gs["nee_queries"] > 0
