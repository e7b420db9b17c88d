"""The schedule autotuner: times candidate values of the context's schedule knobs
(gpis_tune_set) on the caller's own workload and keeps the fastest.

Knobs: the fast pass's persistent grid (CTAs per SM), the render's pass size
(paths per wavefront pass), the host pipeline's chunk and whether it runs on
page-locked host streams in place, the skip cap before a proposed crossing
interval, and where the stationary 1D fast pass keeps its impulse window.  None of them changes
a result: every flight is independent of the grid and of its batch, so the
tuner compares times only.
"""
import time

import numpy as np

from . import abi


def _median_ms(fn, reps):
    import torch
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def tune_march(ctx, devs, candidates=(0, 1, 2, 3, 4), reps=3):
    """CTAs per SM of the fast pass's persistent grid, timed on device-resident batches
    (DeviceFlights).  0 is every resident CTA; values above the occupancy limit act as
    0.  Returns {candidate: ms} and leaves the fastest set."""
    times = {}

    def run():
        for d in devs:
            ctx.submit(d)

    for c in candidates:
        ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM, c)
        run()
        times[c] = _median_ms(run, reps)
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_MARCH_CTAS_PER_SM, best)
    return {"knob": "march_ctas_per_sm", "best": best, "ms": times}


def tune_render(ctx, scenes, candidates=(1 << 20, 1 << 21, 1 << 22, 1 << 23), spp_cap=2, reps=1):
    """Paths per render pass, timed on the scenes with their spp capped (device time of
    gpis_render_batch).  Returns {candidate: ms} and leaves the fastest set."""
    import copy
    small = []
    for sc in scenes:
        s = copy.copy(sc)
        s.spp = min(sc.spp, spp_cap)
        small.append(s)
    times = {}
    for c in candidates:
        ctx.tune(abi.TUNE_RENDER_PASS_PATHS, c)
        ms = []
        for _ in range(reps):
            _, st = ctx.render_batch(small)
            ms.append(st["ms"])
        times[c] = float(np.median(ms))
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_RENDER_PASS_PATHS, best)
    return {"knob": "render_pass_paths", "best": best, "ms": times}


def tune_host_chunk(ctx, pinned, candidates=(1 << 18, 1 << 19, 1 << 20, 1 << 21), reps=3, rounds=2):
    """Flights per chunk of gpis_flights_trace_host, timed on pinned batches (wall
    time of the blocking call).  The candidates are timed in `rounds` interleaved
    rounds and each keeps its best round's median, so that a transient slowdown of
    the host link during one candidate does not decide.  Returns {candidate: ms}
    and leaves the fastest set."""
    times = {}
    for _ in range(rounds):
        for c in candidates:
            ctx.tune(abi.TUNE_HOST_CHUNK, c)
            for p in pinned:
                ctx.trace_pinned(p)
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                for p in pinned:
                    ctx.trace_pinned(p)
                ts.append((time.perf_counter() - t0) * 1e3)
            times[c] = min(times.get(c, float("inf")), float(np.median(ts)))
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_HOST_CHUNK, best)
    return {"knob": "host_chunk", "best": best, "ms": times}


def tune_host_direct(ctx, pinned, reps=3):
    """Staged copies (0) or the kernels on the page-locked streams in place (1), timed on
    pinned batches (wall time of the blocking call).  Returns {candidate: ms} and
    leaves the fastest set."""
    times = {}
    for c in (0, 1):
        ctx.tune(abi.TUNE_HOST_DIRECT, c)
        for p in pinned:
            ctx.trace_pinned(p)
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            for p in pinned:
                ctx.trace_pinned(p)
            ts.append((time.perf_counter() - t0) * 1e3)
        times[c] = float(np.median(ts))
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_HOST_DIRECT, best)
    return {"knob": "host_direct", "best": best, "ms": times}


def tune_proposed_cap(ctx, devs, intervals, candidates=(16, 32, 64), reps=3):
    """The most steps one evaluation may skip before a flight's proposed interval,
    timed on the proposed march of device-resident batches with their intervals
    (every skipped step is certified, so the records do not depend on it).  Returns
    {candidate: ms} and leaves the fastest set."""
    from . import runtime
    times = {}

    def run():
        for d, iv in zip(devs, intervals):
            runtime.submit_proposed(ctx, d, iv)

    for c in candidates:
        ctx.tune(abi.TUNE_PROPOSED_SKIP_CAP, c)
        run()
        times[c] = _median_ms(run, reps)
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_PROPOSED_SKIP_CAP, best)
    return {"knob": "proposed_skip_cap", "best": best, "ms": times}


def tune_fast_window(ctx, devs, reps=3):
    """Where the stationary 1D fast pass keeps each lane's three-cell impulse window:
    0 shared memory, 1 registers; timed on device-resident batches.  Returns
    {candidate: ms} and leaves the fastest set."""
    times = {}

    def run():
        for d in devs:
            ctx.submit(d)

    for c in (0, 1):
        ctx.tune(abi.TUNE_FAST_WINDOW, c)
        run()
        times[c] = _median_ms(run, reps)
    best = min(times, key=times.get)
    ctx.tune(abi.TUNE_FAST_WINDOW, best)
    return {"knob": "fast_window", "best": best, "ms": times}
