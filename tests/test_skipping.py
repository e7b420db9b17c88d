"""Step skipping beyond the stationary single-octave 1D case: 3D media (EvalSkip3D:
the field's range over the next steps, bounded from the impulses of the query's 27
cells, the conditioning splat and the mean's slope) and multi-octave or
nonstationary 1D media with a grid mean (the slope bound at the local scale's
range).  A sound bound changes no result: every case here skips steps (the device
counter) and still meets the flight bars of test_gpu_parity against the oracle, on
the primary pass and on the conditioned secondaries (Renewal's value splat,
Renewal+'s gradient terms), with an anisotropic length scale and with grid means."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, runtime, workloads
from oracle import oracle
from test_gpu_parity import flights_vs_oracle

pytestmark = pytest.mark.gpu


def sphere_grid(res=24, half=1.5):
    """The unit-sphere SDF baked into a res^3 grid over the cube [-half, half]^3."""
    ax = np.linspace(-half, half, res, dtype=np.float64)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    vox = (np.sqrt(x * x + y * y + z * z) - 1.0).astype(np.float32)
    h = (2.0 * half) / (res - 1)
    w2i = (1.0 / h, 0, 0, half / h, 0, 1.0 / h, 0, half / h, 0, 0, 1.0 / h, half / h)
    return abi.make_mean_grid(vox, world_to_index=w2i)


def sphere_grid_medium(**kw):
    return abi.attach_grid(workloads.sphere_medium(one_d=False, **kw), sphere_grid())


def sphere_grid_1d(nonstationary, octaves):
    """A 1D multi-octave or nonstationary field (the torus-plane family's length
    scales and octaves) over the baked sphere grid."""
    return abi.attach_grid(workloads.torus_plane_medium(nonstationary=nonstationary, octaves=octaves), sphere_grid())


CASES = {
    "renewal_plus": lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL_PLUS),
    "anisotropic": lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL, aniso=(1.0, 0.6, 1.4)),
    "grid_mean": lambda: sphere_grid_medium(context=abi.CTX_RENEWAL),
    "large_sigma": lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL, sigma=0.3,
                                                    length_scale=0.2),
    "octaves_grid_mean": lambda: sphere_grid_1d(nonstationary=False, octaves=3),
    "nonstationary_grid_mean": lambda: sphere_grid_1d(nonstationary=True, octaves=1),
}


@pytest.mark.parametrize("kind", sorted(CASES))
def test_gpu_skipping_keeps_flights(kind):
    desc = CASES[kind]()
    prim = workloads.sphere_flights(8192, desc)
    with runtime.Context(desc) as ctx:
        ctx.counters(reset=True)
        rec = ctx.trace_host(prim)
        cnt = ctx.counters(reset=True)
        assert cnt["skipped_steps"] > 0.2 * cnt["steps"], cnt
        flights_vs_oracle(desc, prim, rec)
        rec_cpu = oracle.trace_flights(desc, prim)
        sec, _ = workloads.secondary_flights(prim, rec_cpu, desc)
        rec2 = ctx.trace_host(sec)
        flights_vs_oracle(desc, sec, rec2)
