"""Schedule knobs (gpis_tune_set) and the autotuner: no knob changes a result.
The fast pass's persistent grid, the march's rounds, the render's pass size and
the host pipeline's chunk are varied and every flight record / image must stay
bit-identical."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, proposal, workloads


@pytest.mark.gpu
def test_gpu_knobs_keep_results():
    import torch
    from gpis_extend_gb300 import autotune, runtime
    desc = workloads.sphere_medium()
    prim = workloads.sphere_flights(1 << 16, desc)
    with runtime.Context(desc) as ctx:
        ref = ctx.trace_host(prim)
        for c in (1, 2, 3):
            assert ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM, c) == c
            assert np.array_equal(ctx.trace_host(prim).view(np.uint32), ref.view(np.uint32)), c
        for chunk in (4096, 1 << 14):
            ctx.tune(abi.TUNE_HOST_CHUNK, chunk)
            assert np.array_equal(ctx.trace_host(prim).view(np.uint32), ref.view(np.uint32)), chunk
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM, 1000)
        with pytest.raises(abi.GpisError):
            ctx.tune(7, 1)
        dev = runtime.DeviceFlights(prim)
        res = autotune.tune_march(ctx, [dev], candidates=(0, 1, 2), reps=1)
        assert res["best"] in (0, 1, 2) and ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM) == res["best"]
        torch.cuda.synchronize()
        assert np.array_equal(dev.rec.cpu().numpy().view(np.uint32), ref.view(np.uint32))


MEDIA_ROUNDS = {
    "sphere_1d": (lambda: workloads.sphere_medium(), workloads.sphere_flights, 1.5),
    "sphere_3d": (lambda: workloads.sphere_medium(one_d=False, context=abi.CTX_RENEWAL), workloads.sphere_flights,
                  1.5),
    "torus_octaves": (proposal.config2_medium, workloads.torus_flights, 2.0),
}


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(MEDIA_ROUNDS))
def test_gpu_march_rounds_keep_results(kind):
    """One, two or three rounds of fast and resume passes: the flights a resume pass
    decides and hands back to the fast pass (the conditioned secondaries above all)
    end with the same records as when the last resume pass marches them itself."""
    from gpis_extend_gb300 import runtime
    make, flights, half = MEDIA_ROUNDS[kind]
    desc = make()
    prim = flights(1 << 14, desc)
    with runtime.Context(desc) as ctx:
        ctx.tune(abi.TUNE_MARCH_ROUNDS, 1)
        rec = ctx.trace_host(prim)
        sec, _ = workloads.secondary_flights(prim, rec, desc, half=half)
        ref = [rec, ctx.trace_host(sec)]
        for r in (2, 3, 0):
            assert ctx.tune(abi.TUNE_MARCH_ROUNDS, r) == r
            for b, want in zip((prim, sec), ref):
                assert np.array_equal(ctx.trace_host(b).view(np.uint32), want.view(np.uint32)), (kind, r)
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_MARCH_ROUNDS, 4)


@pytest.mark.gpu
def test_gpu_render_pass_size_keeps_images():
    from gpis_extend_gb300 import runtime
    media, scenes = workloads.config4_batch(n=6, seed=3, sizes=(16, 32), size_p=(0.5, 0.5), spps=(1, 2, 3))
    with runtime.Context(media) as ctx:
        ref, st = ctx.render_batch(scenes)
        ctx.tune(abi.TUNE_RENDER_PASS_PATHS, 4096)
        got, st2 = ctx.render_batch(scenes)
    assert st2["passes"] > st["passes"]
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
