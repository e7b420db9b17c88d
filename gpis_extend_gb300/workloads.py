"""Seeded synthetic flight workloads.

The sphere workload: origins uniform on a radius-3 sphere, each aimed at a
uniform point of the unit ball, clipped to the cube |x|,|y|,|z| <= 1.5 (the
bounding primitive that carries the medium), through the field whose mean is
the signed distance to the unit sphere.  The same generator feeds the GPU
path, the oracle and the benchmark, so every consumer sees identical inputs.

Random numbers come from a counter-based generator: value(seed, index, dim)
is a splitmix64 finaliser of a linear combination of the three, so any
subset of flights can be regenerated independently.
"""
import numpy as np

from . import abi

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(x):
    x = x.astype(np.uint64)
    x ^= x >> np.uint64(30)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(27)
    x *= np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    return x


def counter_uniform(seed, index, dim):
    """U[0,1) doubles (53-bit) from (seed, index, dim)."""
    with np.errstate(over="ignore"):
        idx = np.asarray(index, np.uint64)
        x = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)
             + idx * np.uint64(0xD1B54A32D192ED03)
             + np.uint64(dim) * np.uint64(0x8CB92BA72F3D8DD7)
             + np.uint64(0x632BE59BD9B4E019))
        x = _mix64(x)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def counter_float32_unit(seed, index, dim):
    """U[0,1) float32 values from 24 high bits (never rounds up to 1)."""
    u = counter_uniform(seed, index, dim)
    return (np.floor(u * 16777216.0) / 16777216.0).astype(np.float32)


def _unit_sphere(u, v):
    z = 1.0 - 2.0 * u
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * v
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=-1)


def clip_to_cube(o, d, half):
    """Slab intersection of rays o + t d with the cube [-half, half]^3 (float64)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        t0 = (-half - o) * inv
        t1 = (half - o) * inv
    tmin = np.max(np.minimum(t0, t1), axis=-1)
    tmax = np.min(np.maximum(t0, t1), axis=-1)
    return tmin, tmax


def sphere_medium(one_d=True, context=abi.CTX_RENEWAL_PLUS, sigma=0.05, length_scale=0.1,
                  impulse_density=8.0, seed=1, step_size=0.01, min_step=8, **kw):
    """The stationary SE field over the unit-sphere SDF: sigma 0.05, l 0.1, localScale 3,
    8 impulses per cell, cell hash seeded 1; 1D sampling with Renewal+ by default
    (the batched-flight microbenchmark), 3D world-space noise with Renewal for the
    image configuration."""
    params = dict(sigma=sigma, length_scale=length_scale, kernel_scale=3.0,
                  impulse_density=impulse_density, seed=seed, one_d_sampling=int(one_d),
                  correlation_context=context, step_size=step_size, min_step=min_step,
                  mean_kind=abi.MEAN_SPHERE, mean_params=(0, 0, 0, 1), sigma_s=0.8, sigma_a=0.2)
    params.update(kw)
    return abi.make_medium(**params)


def torus_plane_medium(nonstationary=True, octaves=3, context=abi.CTX_RENEWAL_PLUS, **kw):
    """The nonstationary field over the union SDF of a torus (R 1, r 0.35, about the
    y axis) and the plane y = -0.5: length scale 0.11 + 0.09 sin(3x) cos(2z)
    (0.02 to 0.2; the cells follow the supremum 0.2), three octaves halving the
    length scale with std 0.04 / 0.02 / 0.01, 1D sampling with Renewal+.
    nonstationary=False keeps the length scale at 0.2; octaves=1 keeps one
    realization with std 0.04."""
    params = dict(sigma=0.04, length_scale=1.0 if nonstationary else 0.2, kernel_scale=3.0,
                  impulse_density=8.0, seed=1, one_d_sampling=1, correlation_context=context,
                  step_size=0.005, min_step=8, mean_kind=abi.MEAN_TORUS_PLANE,
                  mean_params=(0, 0, 0, 1.0, 0.35, -0.5), sigma_s=0.8, sigma_a=0.2)
    if nonstationary:
        params.update(ls_kind=abi.LS_SINCOS, ls_params=(0.11, 0.09, 3.0, 2.0), ls_max=0.2)
    if octaves > 1:
        params.update(n_octaves=octaves, octave_sigma=[0.04 / 2 ** k for k in range(octaves)],
                      octave_scale=[0.5 ** k for k in range(octaves)],
                      octave_seed=[0x1F123BB5 * k for k in range(octaves)])
    params.update(kw)
    return abi.make_medium(**params)


def pss_seeds(desc, pss, scene_seed=1):
    """Vectorised noise/normal seeds (computeSeed / prepareGpisSegment formulas)."""
    from .hashing import xxhash32_4, xxhash32_1
    pss = np.asarray(pss, np.uint32)
    w = pss[:, 3].copy()
    if desc.correlation_context == abi.CTX_GLOBAL:
        w[:] = 0
    scene = xxhash32_1(np.full(len(pss), scene_seed, np.uint32))
    with np.errstate(over="ignore"):
        noise = np.full(len(pss), desc.seed, np.uint32)
        if not desc.single_realization:
            noise = noise + xxhash32_4(pss[:, 0], pss[:, 1], pss[:, 2], w) + scene
        normal = xxhash32_4(pss[:, 0], pss[:, 1], pss[:, 2], pss[:, 3]) + scene + np.uint32(1)
    return noise.astype(np.uint32), normal.astype(np.uint32)


def sphere_flights(n, desc, seed=7, half=1.5, bounce=0, scene_seed=1, index_offset=0):
    """Primary flights of the sphere workload: returns a FlightBatch of n flights.

    Origin = entry point of the ray into the cube, nearT = 0, farT = chord length;
    jitter from the same counter stream; path coordinates pss = (i mod 2048,
    i div 2048, 0, bounce)."""
    i = np.arange(n, dtype=np.uint64) + np.uint64(index_offset)
    o = 3.0 * _unit_sphere(counter_uniform(seed, i, 0), counter_uniform(seed, i, 1))
    tgt = _unit_sphere(counter_uniform(seed, i, 2), counter_uniform(seed, i, 3))
    tgt *= np.cbrt(counter_uniform(seed, i, 4))[:, None]
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d32 = d.astype(np.float32)
    tmin, tmax = clip_to_cube(o, d, half)
    entry = (o + d * tmin[:, None]).astype(np.float32)
    # pull the entry point onto the cube face exactly where rounding pushed it outside
    entry = np.clip(entry, -half, half).astype(np.float32)
    b = abi.FlightBatch(n)
    b.origin_near[:, :3] = entry
    b.origin_near[:, 3] = 0.0
    b.dir_far[:, :3] = d32
    b.dir_far[:, 3] = (tmax - tmin).astype(np.float32)
    pss = np.stack([(i % 2048).astype(np.uint32), (i // 2048).astype(np.uint32),
                    np.zeros(n, np.uint32), np.full(n, bounce, np.uint32)], axis=1)
    ns, nm = pss_seeds(desc, pss, scene_seed)
    b.seeds[:, 0] = ns
    b.seeds[:, 1] = nm
    b.seeds[:, 2] = abi.FLAG_FIRST_SCATTER
    b.set_jitter(counter_float32_unit(seed, i, 5))
    b.pss = pss
    b.index_offset = int(index_offset)
    return b


def torus_flights(n, desc, seed=11, half=2.0, bounce=0, scene_seed=1, index_offset=0):
    """Primary flights through the torus-union-plane field (bounded by the cube +-2):
    origins uniform on a radius-4 sphere, directions toward uniform points of the box
    [-1.4, 1.4] x [-0.6, 0.4] x [-1.4, 1.4] around the torus and the plane; the rest
    as sphere_flights."""
    i = np.arange(n, dtype=np.uint64) + np.uint64(index_offset)
    o = 4.0 * _unit_sphere(counter_uniform(seed, i, 0), counter_uniform(seed, i, 1))
    tgt = np.stack([2.8 * counter_uniform(seed, i, 2) - 1.4, counter_uniform(seed, i, 3) - 0.6,
                    2.8 * counter_uniform(seed, i, 4) - 1.4], axis=1)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmin, tmax = clip_to_cube(o, d, half)
    entry = np.clip((o + d * tmin[:, None]).astype(np.float32), -half, half).astype(np.float32)
    b = abi.FlightBatch(n)
    b.origin_near[:, :3] = entry
    b.origin_near[:, 3] = 0.0
    b.dir_far[:, :3] = d.astype(np.float32)
    b.dir_far[:, 3] = (tmax - tmin).astype(np.float32)
    pss = np.stack([(i % 2048).astype(np.uint32), (i // 2048).astype(np.uint32),
                    np.zeros(n, np.uint32), np.full(n, bounce, np.uint32)], axis=1)
    ns, nm = pss_seeds(desc, pss, scene_seed)
    b.seeds[:, 0] = ns
    b.seeds[:, 1] = nm
    b.seeds[:, 2] = abi.FLAG_FIRST_SCATTER
    b.set_jitter(counter_float32_unit(seed, i, 5))
    b.pss = pss
    b.index_offset = int(index_offset)
    return b


def secondary_flights(primary, rec, desc, seed=7, half=1.5, scene_seed=1):
    """Conditioned secondary flights from the hits of a primary pass: origin = hit
    point, direction = mirror reflection about the sampled normal, prevValue = 0,
    prevGradient = sampled gradient (Renewal+ birth), bounce = 1.  Returns
    (batch, index of the primary flight of each secondary flight)."""
    res = abi.unpack_results(rec)
    ok = res["hit"] & (res["status"] == abi.FLIGHT_OK)
    g = res["grad"].astype(np.float64)
    gn = np.linalg.norm(g, axis=1)
    ok &= np.isfinite(gn) & (gn > 1e-12)
    idx = np.nonzero(ok)[0]
    o = primary.origin_near[idx, :3].astype(np.float64)
    d = primary.dir_far[idx, :3].astype(np.float64)
    t = res["t"][idx].astype(np.float64)
    p = o + d * t[:, None]
    nrm = g[idx] / gn[idx, None]
    r = d - 2.0 * np.sum(d * nrm, axis=1, keepdims=True) * nrm
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    p = np.clip(p, -half, half)
    _, tmax = clip_to_cube(p, r, half)
    b = abi.FlightBatch(len(idx))
    b.origin_near[:, :3] = p.astype(np.float32)
    b.origin_near[:, 3] = 0.0
    b.dir_far[:, :3] = r.astype(np.float32)
    b.dir_far[:, 3] = np.maximum(tmax, 1e-4).astype(np.float32)
    i = idx.astype(np.uint64) + np.uint64(getattr(primary, "index_offset", 0))
    pss = np.stack([(i % 2048).astype(np.uint32), (i // 2048).astype(np.uint32),
                    np.zeros(len(idx), np.uint32), np.ones(len(idx), np.uint32)], axis=1)
    ns, nm = pss_seeds(desc, pss, scene_seed)
    b.seeds[:, 0] = ns
    b.seeds[:, 1] = nm
    b.seeds[:, 2] = 0
    b.set_jitter(counter_float32_unit(seed, i, 6))
    b.prev[:, 0] = 0.0
    b.prev[:, 1:4] = res["grad"][idx]
    b.pss = pss
    return b, idx


def render_medium(kind="sphere_3d"):
    """Media of the image workloads (sigma_a = 0, so sigma_s / sigma_t = 1 and the
    Lambert albedo carries the surface colour):
    sphere_3d  the unit-sphere SDF field with 3D world-space noise and Renewal;
    sphere_1d  the same field with 1D noise and Renewal+;
    torus      the nonstationary three-octave torus-union-plane field (1D, Renewal+);
    sphere_1d_nee, sphere_1d_mis  sphere_1d with the NEE or MIS 1D sampling scheme;
    torus_nee  the nonstationary single-octave torus-union-plane field with NEE;
    torus_mr_nee  the same length scale on the multi-resolution grid with NEE;
    torus_oct_nee  the three-octave field of `torus` with NEE (the octave sum's law)."""
    if kind == "torus_oct_nee":
        return torus_plane_medium(nonstationary=True, octaves=3, sigma_a=0.0, sigma_s=1.0,
                                  sampling_scheme=abi.SCHEME_NEE)
    if kind in ("sphere_1d_nee", "sphere_1d_mis"):
        return sphere_medium(one_d=True, context=abi.CTX_RENEWAL_PLUS, sigma_a=0.0, sigma_s=1.0,
                             sampling_scheme=abi.SCHEME_NEE if kind.endswith("nee") else abi.SCHEME_MIS)
    if kind in ("torus_nee", "torus_mr_nee", "torus_mr"):
        return torus_plane_medium(nonstationary=True, octaves=1, sigma_a=0.0, sigma_s=1.0,
                                  multires=int(kind.startswith("torus_mr")),
                                  sampling_scheme=abi.SCHEME_UNI if kind == "torus_mr" else abi.SCHEME_NEE)
    if kind == "sphere_3d":
        return sphere_medium(one_d=False, context=abi.CTX_RENEWAL, sigma_a=0.0, sigma_s=1.0)
    if kind == "sphere_1d":
        return sphere_medium(one_d=True, context=abi.CTX_RENEWAL_PLUS, sigma_a=0.0, sigma_s=1.0)
    if kind == "torus":
        return torus_plane_medium(nonstationary=True, octaves=3, sigma_a=0.0, sigma_s=1.0)
    raise KeyError(kind)


def render_scene(width=256, height=256, spp=16, max_bounces=4, box_half=1.5, **kw):
    """The image workload: pinhole camera at z = 4 looking at the origin (45 degree
    vertical field of view), a 1 x 1 quad light at y = 3 facing down with radiance
    20, Lambert albedo 0.8, the medium in the cube [-h, h]^3."""
    return abi.make_scene(width=width, height=height, spp=spp, max_bounces=max_bounces, box_half=box_half,
                          light_emission=(20.0, 20.0, 20.0), albedo=(0.8, 0.8, 0.8), **kw)


def config4_batch(n=64, seed=11, sizes=(64, 128, 256, 512, 1024), size_p=(0.35, 0.3, 0.2, 0.1, 0.05),
                  spps=(1, 2, 4, 8, 16, 32, 64), max_bounces=4, spp_scale=1.0):
    """The uneven image batch: n media drawn from `seed` -- sphere, torus, plane or
    torus-union-plane mean SDFs, length scales 0.02-0.3, one to three octaves (1D
    noise), Renewal or Renewal+, std 0.02-0.06 -- each with its own image (size from
    `sizes` with probabilities `size_p`, spp from `spps` times spp_scale), Lambert
    albedo 0.8, 4 bounces.  Returns (media, scenes); scene k renders medium k."""
    rng = np.random.default_rng(seed)
    media, scenes = [], []
    for i in range(n):
        kind = int(rng.integers(0, 4))
        octaves = int(rng.integers(1, 4))
        ctx = abi.CTX_RENEWAL_PLUS if rng.random() < 0.5 else abi.CTX_RENEWAL
        ell = float(rng.uniform(0.02, 0.3))
        sigma = float(rng.uniform(0.02, 0.06))
        params = dict(sigma=sigma, length_scale=ell, kernel_scale=3.0, impulse_density=8.0,
                      seed=int(rng.integers(1, 1000)), one_d_sampling=1, correlation_context=ctx,
                      step_size=float(max(0.004, ell / 10)), min_step=8, sigma_s=1.0, sigma_a=0.0)
        if kind == 0:
            params.update(mean_kind=abi.MEAN_SPHERE, mean_params=(0, 0, 0, 1))
        elif kind == 1:
            params.update(mean_kind=abi.MEAN_TORUS, mean_params=(0, 0, 0, 1.0, 0.35))
        elif kind == 2:
            params.update(mean_kind=abi.MEAN_PLANE, mean_params=(0, 1, 0, -0.5))
        else:
            params.update(mean_kind=abi.MEAN_TORUS_PLANE, mean_params=(0, 0, 0, 1.0, 0.35, -0.5))
        if octaves > 1:
            params.update(n_octaves=octaves, octave_sigma=[sigma / 2 ** k for k in range(octaves)],
                          octave_scale=[0.5 ** k for k in range(octaves)],
                          octave_seed=[0x1F123BB5 * k for k in range(octaves)])
        media.append(abi.make_medium(**params))
        size = int(rng.choice(sizes, p=size_p))
        spp = max(1, int(round(int(rng.choice(spps)) * spp_scale)))
        scenes.append(render_scene(width=size, height=size, spp=spp, max_bounces=max_bounces, medium=i,
                                   box_half=1.5 if kind == 0 else 2.0, sampler_seed=7 + i))
    return media, scenes


def batch_flights(media, per_medium, seed=31, index_offset=0):
    """Primary flights through every medium of an image batch (origins on a radius-4
    sphere toward the region around the origin, cube 2), interleaved in one batch
    with its medium stream: training data for the learned arm of the batch."""
    parts = []
    for k, d in enumerate(media):
        b = torus_flights(per_medium, d, seed=seed + k, half=2.0, index_offset=index_offset + k * per_medium)
        parts.append(b)
    n = per_medium * len(media)
    out = abi.FlightBatch(n)
    for name in ("origin_near", "dir_far", "seeds", "prev"):
        getattr(out, name)[:] = np.concatenate([getattr(p, name) for p in parts])
    out.medium = np.repeat(np.arange(len(media), dtype=np.uint32), per_medium)
    return out
