"""Medium::sampleDistance / Medium::transmittance semantics
(GaussianProcessMedium.cpp:222-440) through gpis_medium_sample_distance /
gpis_medium_transmittance, against the oracle's restatement of the same state
machines.  CPU tests pin the oracle's edge semantics; GPU tests run two chained
bounces (primary, then the conditioned query from every hit along the mirror
direction) and shadow rays, and compare samples and updated states."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle

T_TOL = 1e-4 * 1.5


def make_rays(batch):
    r = np.zeros(batch.n, abi.RAY_DTYPE)
    r["pos"] = batch.origin_near[:, :3]
    r["dir"] = batch.dir_far[:, :3]
    r["near_t"] = batch.origin_near[:, 3]
    r["far_t"] = batch.dir_far[:, 3]
    return r


def make_states(n, pss, scene_seed=1):
    s = np.zeros(n, abi.STATE_DTYPE)
    s["pss"] = pss
    s["scene_seed"] = scene_seed
    s["first_scatter"] = 1
    return s


# ---- CPU: oracle edge semantics -------------------------------------------------

def test_oracle_distance_edge_cases():
    d = workloads.sphere_medium()
    rays = np.zeros(4, abi.RAY_DTYPE)
    rays["dir"] = [0, 0, 1]
    rays["pos"] = [0, 0, -1.4]
    rays["near_t"] = [0.5, 0.0, 0.0, 0.0]
    rays["far_t"] = [0.5, 1.0, np.inf, 1.0]           # far <= near: exits at maxT
    st = make_states(4, np.array([[i, 0, 0, 0] for i in range(4)], np.uint32))
    st["bounce"][3] = d.max_bounces                   # bounce limit: Failed
    s = oracle.medium_sample_distance(d, rays, st, np.full(4, 0.5, np.float32))
    assert s["status"][0] == 1 and s["exited"][0] == 1 and s["t"][0] == 0.5 and st["bounce"][0] == 0
    assert s["status"][1] == 1 and s["exited"][1] == 0 and 0.3 < s["t"][1] < 0.5   # hits the unit sphere near z=-1
    assert st["first_scatter"][1] == 0 and st["bounce"][1] == 1 and st["last_val"][1] == 0.0
    assert abs(st["info_t"][1] - s["t"][1]) < 1e-7
    assert np.allclose(s["weight"][1], 0.8)          # sigma_s / sigma_t
    assert s["status"][2] == 1                        # an infinite far is clamped to near + 2000
    assert s["status"][3] == 0
    # a ray that misses: exits at far with the gradient of the end point and lastVal = f(far)
    rays2 = np.zeros(1, abi.RAY_DTYPE)
    rays2["pos"] = [0, 1.4, -1.4]
    rays2["dir"] = [0, 0, 1]
    rays2["far_t"] = 2.8
    st2 = make_states(1, np.array([[9, 9, 0, 0]], np.uint32))
    s2 = oracle.medium_sample_distance(d, rays2, st2, np.array([0.25], np.float32))
    assert s2["exited"][0] == 1 and s2["t"][0] == np.float32(2.8) and st2["last_val"][0] > 0
    assert np.linalg.norm(s2["aniso"][0]) > 0.5 and st2["bounce"][0] == 1


def test_oracle_absorption_only_medium():
    d = workloads.sphere_medium()
    d.sigma_s = 0.0
    d.sigma_a = 1.0
    rays = np.zeros(2, abi.RAY_DTYPE)
    rays["pos"] = [[0, 0, -1.4], [0, 1.4, -1.4]]
    rays["dir"] = [0, 0, 1]
    rays["far_t"] = 2.8
    st = make_states(2, np.array([[1, 2, 0, 0], [3, 4, 0, 0]], np.uint32))
    s = oracle.medium_sample_distance(d, rays, st, np.full(2, 0.5, np.float32))
    assert np.all(s["exited"] == 1) and np.allclose(s["t"], 2.8)
    assert np.all(s["weight"][0] == 0.0) and np.all(s["weight"][1] == 1.0)   # transmittance weight
    assert np.all(st["bounce"] == 0)


def test_oracle_transmittance():
    d = workloads.sphere_medium()
    rays = np.zeros(3, abi.RAY_DTYPE)
    rays["pos"] = [[0, 0, -1.4], [0, 1.4, -1.4], [0, 0, 0]]
    rays["dir"] = [0, 0, 1]
    rays["far_t"] = [2.8, 2.8, 0.0]
    st = make_states(3, np.array([[i, 1, 0, 0] for i in range(3)], np.uint32))
    tr = oracle.medium_transmittance(d, rays, st, np.full(3, 0.5, np.float32))
    assert list(tr) == [0.0, 1.0, 1.0]
    assert st["first_scatter"][0] == 0 and st["first_scatter"][1] == 1 and st["bounce"][0] == 0


def test_json_max_bounces():
    import ctypes
    from gpis_extend_gb300 import build
    build.build()
    lib = abi.load_library()
    d = abi.MediumDesc()
    assert lib.gpis_medium_desc_from_json(b'{"correlation_context": "renewal", "max_bounces": 7}',
                                          ctypes.byref(d)) == 0
    assert d.max_bounces == 7
    lib.gpis_medium_desc_init(ctypes.byref(d))
    assert d.max_bounces == 1024


# ---- GPU: adapter vs oracle --------------------------------------------------------

def compare_samples(g, c, gs, cs):
    assert np.array_equal(g["status"], c["status"])
    ok = (g["status"] == 1) & (c["status"] == 1)
    agree = g["exited"][ok] == c["exited"][ok]
    assert agree.mean() >= 0.9999
    sel = np.nonzero(ok)[0][agree]
    dt = np.abs(g["t"][sel] - c["t"][sel])
    assert np.mean(dt <= T_TOL) >= 0.9999
    close = sel[dt[np.arange(len(sel))] <= 1e-6]
    rel = np.linalg.norm(g["aniso"][close] - c["aniso"][close], axis=1) / np.maximum(
        1e-6, np.linalg.norm(c["aniso"][close], axis=1))
    assert np.mean(rel <= 2e-3) >= 0.999
    assert np.array_equal(g["gp_id"][sel], c["gp_id"][sel])
    assert np.array_equal(g["sampling_scheme"][sel], c["sampling_scheme"][sel])
    assert np.allclose(g["weight"][sel], c["weight"][sel])
    for k in ("first_scatter", "bounce"):
        assert np.mean(gs[k][sel] == cs[k][sel]) >= 0.9999
    assert np.mean(np.abs(gs["info_t"][sel] - cs["info_t"][sel]) <= 2 * T_TOL) >= 0.9999


@pytest.mark.gpu
@pytest.mark.parametrize("one_d", [True, False])
def test_gpu_sample_distance_chain_vs_oracle(one_d):
    from gpis_extend_gb300 import runtime
    ctxname = abi.CTX_RENEWAL_PLUS if one_d else abi.CTX_RENEWAL
    d = workloads.sphere_medium(one_d=one_d, context=ctxname, sampling_scheme=abi.SCHEME_MIS)
    n = 1 << 12 if one_d else 1 << 9
    prim = workloads.sphere_flights(n, d)
    rays = make_rays(prim)
    jit = prim.jitter.copy()
    st_g = make_states(n, prim.pss)
    st_c = st_g.copy()
    with runtime.Context(d) as ctx:
        sg = ctx.sample_distance(0, rays, st_g, jit)
        sc = oracle.medium_sample_distance(d, rays, st_c, jit)
        compare_samples(sg, sc, st_g, st_c)
        # second bounce from the oracle's hits along the mirror direction, with the
        # oracle's states (identical inputs on both paths)
        hit = (sc["status"] == 1) & (sc["exited"] == 0)
        idx = np.nonzero(hit)[0]
        r2 = np.zeros(len(idx), abi.RAY_DTYPE)
        dirs = rays["dir"][idx].astype(np.float64)
        nrm = sc["aniso"][idx].astype(np.float64)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        refl = dirs - 2 * np.sum(dirs * nrm, axis=1, keepdims=True) * nrm
        refl /= np.linalg.norm(refl, axis=1, keepdims=True)
        p = sc["p"][idx].astype(np.float64)
        _, tmax = workloads.clip_to_cube(np.clip(p, -1.5, 1.5), refl, 1.5)
        r2["pos"] = p.astype(np.float32)
        r2["dir"] = refl.astype(np.float32)
        r2["far_t"] = np.maximum(tmax, 1e-3).astype(np.float32)
        s2 = st_c[idx].copy()
        s2["pss"][:, 3] += 1
        s2c = s2.copy()
        j2 = workloads.counter_float32_unit(99, np.arange(len(idx), dtype=np.uint64), 0)
        g2 = ctx.sample_distance(0, r2, s2, j2)
        c2 = oracle.medium_sample_distance(d, r2, s2c, j2)
        compare_samples(g2, c2, s2, s2c)
        # shadow rays from the second-bounce states toward +y
        r3 = r2.copy()
        r3["dir"] = [0.0, 1.0, 0.0]
        r3["far_t"] = 1.5 - np.clip(r2["pos"][:, 1], -1.5, 1.5)
        s3g, s3c = s2.copy(), s2.copy()
        tg = ctx.transmittance(0, r3, s3g, j2)
        tc = oracle.medium_transmittance(d, r3, s3c, j2)
        assert np.mean(tg == tc) >= 0.9999
        assert np.mean(s3g["first_scatter"] == s3c["first_scatter"]) >= 0.9999
