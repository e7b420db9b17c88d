"""Schedule knobs (gpis_tune_set) and the autotuner: no knob changes a result.
The fast pass's persistent grid and impulse window, the render's pass size and
the host pipeline's chunk are varied and every flight record / image must stay
bit-identical."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads


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
        # the stationary fast pass's impulse window in registers, then shared memory again
        for w in (1, 0):
            ctx.tune(abi.TUNE_FAST_WINDOW, w)
            assert np.array_equal(ctx.trace_host(prim).view(np.uint32), ref.view(np.uint32)), w
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_FAST_WINDOW, 2)
        for chunk in (4096, 1 << 14):
            ctx.tune(abi.TUNE_HOST_CHUNK, chunk)
            assert np.array_equal(ctx.trace_host(prim).view(np.uint32), ref.view(np.uint32)), chunk
        # in place on page-locked streams, and staged again
        pin = runtime.PinnedFlights(prim)
        for direct in (1, 0):
            ctx.tune(abi.TUNE_HOST_DIRECT, direct)
            pin.rec.zero_()
            ctx.trace_pinned(pin)
            assert np.array_equal(pin.results().view(np.uint32), ref.view(np.uint32)), direct
        # pageable streams take the staged path whatever the knob
        ctx.tune(abi.TUNE_HOST_DIRECT, 1)
        assert np.array_equal(ctx.trace_host(prim).view(np.uint32), ref.view(np.uint32))
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_HOST_DIRECT, 2)
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM, 1000)
        with pytest.raises(abi.GpisError):
            ctx.tune(7, 1)
        dev = runtime.DeviceFlights(prim)
        res = autotune.tune_march(ctx, [dev], candidates=(0, 1, 2), reps=1)
        assert res["best"] in (0, 1, 2) and ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM) == res["best"]
        torch.cuda.synchronize()
        assert np.array_equal(dev.rec.cpu().numpy().view(np.uint32), ref.view(np.uint32))


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
