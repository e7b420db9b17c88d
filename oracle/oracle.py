"""ctypes wrapper of the oracle (oracle/gpis_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker.  Builds
oracle/_build/libgpis_oracle.so on first use (gcc, a few seconds).
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

from gpis_extend_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpis_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (no reference sources needed)."""
    src = [os.path.join(HERE, "gpis_oracle.c"), os.path.join(HERE, "pt_oracle.c"), os.path.join(HERE, "gpis_oracle.h"),
           os.path.join(os.path.dirname(HERE), "include", "gpis.h")]
    stale = not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in src)
    if force or stale:
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            u32, vp, c_int = ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int
            P = ctypes.POINTER
            M = P(abi.MediumDesc)
            sigs = {
                "gor_xxhash32_1": (u32, [u32]),
                "gor_xxhash32_2": (u32, [u32, u32]),
                "gor_xxhash32_4": (u32, [u32, u32, u32, u32]),
                "gor_pcg_stream": (None, [ctypes.c_uint64, u32, vp, vp]),
                "gor_normal_pair": (None, [ctypes.c_uint64, u32, vp]),
                "gor_cell_1d": (None, [u32, u32, u32, vp, vp]),
                "gor_cell_3d": (None, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, u32, u32, u32, vp, vp]),
                "gor_field": (c_int, [M, vp, vp, vp, vp, vp, c_int, vp]),
                "gor_gradient": (c_int, [M, vp, vp, vp, ctypes.c_float, vp, vp, vp]),
                "gor_trace_flights": (c_int, [M, c_int, P(abi.FlightSoA), P(abi.ResultSoA), u32, c_int]),
                "gor_flight_seeds": (None, [M, vp, u32, vp, vp]),
                "gor_transverse_moments": (c_int, [M, vp, vp, vp, vp, vp, c_int, vp, vp]),
                "gor_nee": (c_int, [M, vp, vp, vp, vp, ctypes.c_float, vp, vp, vp, vp]),
                "gor_level_ratio": (c_int, [M, vp, vp, vp]),
                "gor_sampling_scheme": (c_int, [M, vp, vp, vp]),
                "gor_se_splat_1d": (None, [vp, vp, u32, ctypes.c_float, vp, vp]),
                "gor_medium_sample_distance": (c_int, [M, vp, vp, vp, vp, u32]),
                "gor_medium_transmittance": (c_int, [M, vp, vp, vp, vp, u32]),
                "gor_render": (c_int, [M, ctypes.POINTER(abi.SceneDesc), vp, vp, u32, u32]),
                "gor_render_span": (c_int, [M, ctypes.POINTER(abi.SceneDesc), vp, vp, u32, u32, u32]),
            }
            for k, (r, a) in sigs.items():
                f = getattr(L, k)
                f.restype = r
                f.argtypes = a
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


def _f3(v):
    return np.ascontiguousarray(v, np.float32).reshape(-1)


def trace_flights(media, batch, n_threads=0):
    """Float-mode flights on the CPU; returns the (n, 8) result records."""
    if isinstance(media, abi.MediumDesc):
        media = [media]
    arr = (abi.MediumDesc * len(media))(*media)
    rec = abi.new_results(batch.n)
    rc = lib().gor_trace_flights(arr, len(media), ctypes.byref(batch.soa()),
                                 ctypes.byref(abi.result_soa(rec)), batch.n, n_threads)
    if rc:
        raise abi.GpisError(f"oracle trace failed: {rc}", rc)
    return rec


def field(desc, origin, direction, p, seeds, prev=(0, 0, 0, 0), double_mode=False):
    o, d, q = _f3(origin), _f3(direction), _f3(p)
    s = np.ascontiguousarray(seeds, np.uint32)
    pv = np.ascontiguousarray(prev, np.float32)
    out = np.zeros(6, np.float64)
    rc = lib().gor_field(ctypes.byref(desc), _p(o), _p(d), _p(q), _p(s), _p(pv), int(double_mode), _p(out))
    if rc:
        raise abi.GpisError(f"oracle field failed: {rc}", rc)
    return out


def gradient(desc, origin, direction, p, t_segment, seeds, prev=(0, 0, 0, 0)):
    o, d, q = _f3(origin), _f3(direction), _f3(p)
    s = np.ascontiguousarray(seeds, np.uint32)
    pv = np.ascontiguousarray(prev, np.float32)
    out = np.zeros(3, np.float32)
    rc = lib().gor_gradient(ctypes.byref(desc), _p(o), _p(d), _p(q), float(t_segment), _p(s), _p(pv), _p(out))
    if rc:
        raise abi.GpisError(f"oracle gradient failed: {rc}", rc)
    return out


def transverse_moments(desc, origin, direction, p, seeds, prev, conditioning=True):
    o, d, q = _f3(origin), _f3(direction), _f3(p)
    s = np.ascontiguousarray(seeds, np.uint32)
    pv = np.ascontiguousarray(prev, np.float32)
    mean = np.zeros(2, np.float64)
    var = np.zeros(1, np.float64)
    ok = lib().gor_transverse_moments(ctypes.byref(desc), _p(o), _p(d), _p(q), _p(s), _p(pv),
                                      int(conditioning), _p(mean), _p(var))
    return bool(ok), mean, float(var[0])


def nee(desc, origin, direction, p, normal, t_segment, seeds, prev):
    o, d, q, nr = _f3(origin), _f3(direction), _f3(p), _f3(normal)
    s = np.ascontiguousarray(seeds, np.uint32)
    pv = np.ascontiguousarray(prev, np.float32)
    pdf = np.zeros(1, np.float32)
    g = np.zeros(3, np.float32)
    rc = lib().gor_nee(ctypes.byref(desc), _p(o), _p(d), _p(q), _p(nr), float(t_segment), _p(s),
                       _p(pv), _p(pdf), _p(g))
    if rc:
        raise abi.GpisError(f"oracle nee failed: {rc}", rc)
    return float(pdf[0]), g


def level_ratio(desc, p):
    """Multi-resolution levels at p: ((low scale, high scale, low weight, high weight),
    (low seed offset, high seed offset))."""
    q = _f3(p)
    info = np.zeros(4, np.float32)
    seeds = np.zeros(2, np.uint32)
    rc = lib().gor_level_ratio(ctypes.byref(desc), _p(q), _p(info), _p(seeds))
    if rc:
        raise abi.GpisError(f"oracle level_ratio failed: {rc}", rc)
    return info, seeds


def sampling_scheme(desc, origin, p, seeds):
    o, q = _f3(origin), _f3(p)
    s = np.ascontiguousarray(seeds, np.uint32)
    return lib().gor_sampling_scheme(ctypes.byref(desc), _p(o), _p(q), _p(s))


def cell_1d(cell, seed, impulses):
    pos = np.zeros(impulses, np.float32)
    w = np.zeros(impulses, np.float32)
    lib().gor_cell_1d(cell & 0xFFFFFFFF, seed & 0xFFFFFFFF, impulses, _p(pos), _p(w))
    return pos, w


def cell_3d(i, j, k, seed, impulses, order=0):
    pos = np.zeros((impulses, 3), np.float32)
    w = np.zeros(impulses, np.float32)
    lib().gor_cell_3d(i, j, k, seed & 0xFFFFFFFF, impulses, order, _p(pos), _p(w))
    return pos, w


def pcg_stream(state, n):
    f = np.zeros(n, np.float32)
    r = np.zeros(n, np.uint32)
    lib().gor_pcg_stream(state, n, _p(f), _p(r))
    return f, r


def normal_pairs(state, pairs):
    out = np.zeros(2 * pairs, np.float64)
    lib().gor_normal_pair(state, pairs, _p(out))
    return out


def flight_seeds(desc, pss, scene_seed):
    p = np.ascontiguousarray(pss, np.uint32)
    a = np.zeros(1, np.uint32)
    b = np.zeros(1, np.uint32)
    lib().gor_flight_seeds(ctypes.byref(desc), _p(p), scene_seed, _p(a), _p(b))
    return int(a[0]), int(b[0])


def se_splat_1d(q, c, scale):
    q = np.ascontiguousarray(q, np.float32)
    c = np.ascontiguousarray(c, np.float32)
    v = np.zeros(len(q), np.float64)
    d = np.zeros(len(q), np.float64)
    lib().gor_se_splat_1d(_p(q), _p(c), len(q), float(scale), _p(v), _p(d))
    return v, d


def medium_sample_distance(desc, rays, states, jitter):
    """rays: RAY_DTYPE array; states: STATE_DTYPE array (updated in place)."""
    samples = np.zeros(len(rays), abi.SAMPLE_DTYPE)
    jit = np.ascontiguousarray(jitter, np.float32)
    rc = lib().gor_medium_sample_distance(ctypes.byref(desc), _p(rays), _p(states), _p(jit), _p(samples), len(rays))
    if rc:
        raise abi.GpisError(f"oracle sample distance failed: {rc}", rc)
    return samples


def medium_transmittance(desc, rays, states, jitter):
    tr = np.zeros(len(rays), np.float32)
    jit = np.ascontiguousarray(jitter, np.float32)
    rc = lib().gor_medium_transmittance(ctypes.byref(desc), _p(rays), _p(states), _p(jit), _p(tr), len(rays))
    if rc:
        raise abi.GpisError(f"oracle transmittance failed: {rc}", rc)
    return tr


def render(desc, scene, n_threads=0):
    """The path tracer restatement: returns (image (h, w, 3) float32, counts dict).
    Rows are split over a thread pool (the C code releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    h, w = scene.height, scene.width
    img = np.zeros((h, w, 3), np.float32)
    n_threads = n_threads or os.cpu_count() or 1
    chunks = [(r, min(h, r + max(1, h // (4 * n_threads)))) for r in range(0, h, max(1, h // (4 * n_threads)))]
    counts = np.zeros((len(chunks), 4), np.uint64)
    L = lib()

    def run(k):
        r0, r1 = chunks[k]
        rc = L.gor_render(ctypes.byref(desc), ctypes.byref(scene), _p(img), _p(counts[k]), r0, r1 - r0)
        if rc:
            raise abi.GpisError(f"oracle render failed: {rc}", rc)

    with ThreadPoolExecutor(n_threads) as ex:
        list(ex.map(run, range(len(chunks))))
    c = counts.sum(axis=0)
    return img, {"distance_flights": int(c[0]), "shadow_flights": int(c[1]), "medium_events": int(c[2]),
                 "failed": int(c[3])}


def render_band(desc, scene, row0, rows, n_threads=0, span=16):
    """Rows [row0, row0 + rows) of the restatement's image, each row split into spans
    of `span` pixels over a thread pool (a band of a large image at full spp);
    returns (rows, counts dict)."""
    from concurrent.futures import ThreadPoolExecutor
    h, w = scene.height, scene.width
    img = np.zeros((h, w, 3), np.float32)
    n_threads = n_threads or os.cpu_count() or 1
    jobs = [(r, c) for r in range(row0, row0 + rows) for c in range(0, w, span)]
    counts = np.zeros((len(jobs), 4), np.uint64)
    L = lib()

    def run(k):
        r, c = jobs[k]
        rc = L.gor_render_span(ctypes.byref(desc), ctypes.byref(scene), _p(img), _p(counts[k]), r, c, span)
        if rc:
            raise abi.GpisError(f"oracle render failed: {rc}", rc)

    with ThreadPoolExecutor(n_threads) as ex:
        list(ex.map(run, range(len(jobs))))
    c = counts.sum(axis=0)
    return img[row0:row0 + rows], {"distance_flights": int(c[0]), "shadow_flights": int(c[1]),
                                   "medium_events": int(c[2]), "failed": int(c[3])}


def render_rows(desc, scene, row0, rows, n_threads=0):
    """Rows [row0, row0 + rows) of the restatement's image of the full scene (the CPU
    baseline's bounded sample); returns (rows, counts dict)."""
    from concurrent.futures import ThreadPoolExecutor
    h, w = scene.height, scene.width
    img = np.zeros((h, w, 3), np.float32)
    n_threads = n_threads or os.cpu_count() or 1
    counts = np.zeros((rows, 4), np.uint64)
    L = lib()

    def run(k):
        rc = L.gor_render(ctypes.byref(desc), ctypes.byref(scene), _p(img), _p(counts[k]), row0 + k, 1)
        if rc:
            raise abi.GpisError(f"oracle render failed: {rc}", rc)

    with ThreadPoolExecutor(n_threads) as ex:
        list(ex.map(run, range(rows)))
    c = counts.sum(axis=0)
    return img[row0:row0 + rows], {"distance_flights": int(c[0]), "shadow_flights": int(c[1]),
                                   "medium_events": int(c[2]), "failed": int(c[3])}


def compare_flights(rec_gpu, rec_cpu, sigma, scene_scale, t_tol_rel=1e-4, value_tol=1e-5, grad_tol=2e-3):
    """Parity statistics of two sets of flight records of the same inputs (the GPU's
    and this oracle's): the bars of the flight path, counted rather than asserted.

    * status agreement, hit / miss (transmittance 0/1) agreement;
    * hits on both sides: |dt| <= t_tol_rel * scene_scale; hits outside it that are
      back-off cases (one side returned t = 0 after the reference refinement's x0.9
      back-off reached 0.01, SparseConvolutionNoiseMedium.cpp:309-330) and the rest;
    * misses on both sides: t equal, the value at farT within value_tol of the noise
      scale sigma (relative above sigma);
    * gradients of hits with |dt| <= 1e-6: relative L2 <= grad_tol.
    """
    g, c = abi.unpack_results(rec_gpu), abi.unpack_results(rec_cpu)
    n = len(g["hit"])
    agree = g["hit"] == c["hit"]
    both = agree & g["hit"]
    dt = np.abs(g["t"][both].astype(np.float64) - c["t"][both])
    t_tol = t_tol_rel * scene_scale
    bad = dt > t_tol
    backoff = (g["t"][both] == 0) | (c["t"][both] == 0)
    miss = agree & ~g["hit"]
    s = max(float(sigma), 1e-6)
    vtol = value_tol * s * np.maximum(1.0, np.abs(c["value"][miss]) / s)
    v_ok = np.abs(g["value"][miss].astype(np.float64) - c["value"][miss]) <= vtol
    close_t = both.copy()
    close_t[both] = dt <= 1e-6
    gg, cg = g["grad"][close_t], c["grad"][close_t]
    rel = np.linalg.norm(gg - cg, axis=1) / np.maximum(1e-6, np.linalg.norm(cg, axis=1))
    hits = int(both.sum())
    return {
        "flights": int(n),
        "status_agreement": float((g["status"] == c["status"]).mean()) if n else 1.0,
        "hit_agreement": float(agree.mean()) if n else 1.0,
        "hit_disagreements": int((~agree).sum()),
        "hits": hits,
        "t_tol": t_tol,
        "hits_within_t_tol": float(1.0 - bad.mean()) if hits else 1.0,
        "t_outliers": int(bad.sum()),
        "t_outliers_backoff": int((bad & backoff).sum()),
        "t_outliers_other": int((bad & ~backoff).sum()),
        "max_dt_non_backoff": float(dt[~backoff].max()) if (~backoff).any() else 0.0,
        "misses": int(miss.sum()),
        "miss_t_equal": float((g["t"][miss] == c["t"][miss]).mean()) if miss.any() else 1.0,
        "miss_value_within_tol": float(v_ok.mean()) if miss.any() else 1.0,
        "normals_compared": int(close_t.sum()),
        "normals_within_tol": float((rel <= grad_tol).mean()) if close_t.any() else 1.0,
    }
