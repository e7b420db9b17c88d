"""Uneven batches over many media in one launch (the per-flight medium stream):
media drawn from seed 11 -- sphere, torus, plane and torus-union-plane means,
length scales 0.02-0.3, one to three octaves, stationary or nonstationary,
Renewal or Renewal+, 1D or 3D noise -- with their flights interleaved in one
batch.  The batch must agree with the oracle (the flight bars of
test_gpu_parity) and with one batch per medium."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle


def draw_media(n, seed=11, allow_3d=True, only_3d=False, spaces=False):
    """spaces: the 3D media cycle through isotropic ray space, a brute-force
    nonstationary length scale and the multi-resolution grid (in isotropic space
    every other time)."""
    rng = np.random.default_rng(seed)
    media = []
    for i in range(n):
        kind = rng.integers(0, 4)
        one_d = not only_3d and ((not allow_3d) or rng.random() < 0.75)
        octaves = int(rng.integers(1, 4)) if one_d else 1
        ns = (one_d and rng.random() < 0.3) or (spaces and not one_d and i % 3 != 0)
        ctx = abi.CTX_RENEWAL_PLUS if rng.random() < 0.5 else abi.CTX_RENEWAL
        ell = float(rng.uniform(0.02, 0.3))
        params = dict(sigma=float(rng.uniform(0.02, 0.06)), length_scale=ell if not ns else 1.0, kernel_scale=3.0,
                      impulse_density=8.0, seed=int(rng.integers(1, 1000)), one_d_sampling=int(one_d),
                      correlation_context=ctx, step_size=float(max(0.004, ell / 10)), min_step=8,
                      sigma_s=0.8, sigma_a=0.2)
        if kind == 0:
            params.update(mean_kind=abi.MEAN_SPHERE, mean_params=(0, 0, 0, 1))
        elif kind == 1:
            params.update(mean_kind=abi.MEAN_TORUS, mean_params=(0, 0, 0, 1.0, 0.35))
        elif kind == 2:
            params.update(mean_kind=abi.MEAN_PLANE, mean_params=(0, 1, 0, -0.25))
        else:
            params.update(mean_kind=abi.MEAN_TORUS_PLANE, mean_params=(0, 0, 0, 1.0, 0.35, -0.5))
        if ns:
            params.update(ls_kind=abi.LS_SINCOS, ls_params=(0.6 * ell, 0.4 * ell, 3.0, 2.0), ls_max=ell)
        if spaces and not one_d:
            params.update(isotropic_3d_sampling=int(i % 3 == 0 or i % 6 == 5), multires=int(i % 3 == 2))
            if i % 3 == 2:
                params.update(length_scale=1.0)
        if octaves > 1:
            params.update(n_octaves=octaves, octave_sigma=[params["sigma"] / 2 ** k for k in range(octaves)],
                          octave_scale=[0.5 ** k for k in range(octaves)],
                          octave_seed=[0x1F123BB5 * k for k in range(octaves)])
        media.append(abi.make_medium(**params))
    return media


def mixed_batch(media, per_medium, seed=5):
    parts, index = [], []
    for i, d in enumerate(media):
        b = workloads.sphere_flights(per_medium, d, seed=seed + i, index_offset=i * per_medium)
        parts.append(b)
        index.append(np.full(per_medium, i, np.uint32))
    n = per_medium * len(media)
    batch = abi.FlightBatch(n)
    order = np.random.default_rng(seed).permutation(n)
    for name in ("origin_near", "dir_far", "seeds", "prev"):
        getattr(batch, name)[:] = np.concatenate([getattr(p, name) for p in parts])[order]
    batch.medium = np.concatenate(index)[order]
    return batch, parts, order


def test_oracle_mixed_batch_equals_per_medium():
    media = draw_media(6)
    batch, parts, order = mixed_batch(media, 64)
    rec = oracle.trace_flights(media, batch)
    per = np.concatenate([oracle.trace_flights(d, p) for d, p in zip(media, parts)])[order]
    assert np.array_equal(rec.view(np.uint32), per.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["1d", "mixed", "3d", "3d_spaces"])
def test_gpu_mixed_media_one_launch(mode):
    """1D media only (the octave and nonstationary fast passes with their skipping),
    1D and 3D media together (the generic fast pass), 3D media only (the 3D fast
    pass with its range-bound skipping, per-lane media) and 3D media in isotropic
    space, nonstationary and on the multi-resolution grid (the generic evaluator)."""
    from gpis_extend_gb300 import runtime
    from test_gpu_parity import flights_vs_oracle
    media = draw_media(16, allow_3d=mode != "1d", only_3d=mode.startswith("3d"), spaces=mode == "3d_spaces")
    batch, parts, order = mixed_batch(media, 256 if mode == "1d" else 96)
    with runtime.Context(media) as ctx:
        rec = ctx.trace_host(batch)
    flights_vs_oracle(media[0], batch, rec, check_grad=True, media=media)
    g = abi.unpack_results(rec)
    sep = []
    for d, p in zip(media, parts):
        with runtime.Context(d) as c1:
            sep.append(c1.trace_host(p))
    s = abi.unpack_results(np.concatenate(sep)[order])
    assert np.array_equal(g["status"], s["status"])
    assert np.mean(g["hit"] == s["hit"]) >= 0.999
    both = g["hit"] & s["hit"]
    assert np.mean(np.abs(g["t"][both] - s["t"][both]) <= 1.5e-4) >= 0.999
