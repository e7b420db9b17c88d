"""The march parameter after k steps (flights.cu: t_direct_ok, t_after) against k
sequential float-float additions (device_common.cuh: ff_add) and against exact
arithmetic, restated in NumPy float32 arithmetic (every operation one IEEE
rounding, as on the GPU).

The fast pass skips certified steps in one jump to t0 + k step instead of k
additions; the two must give the same float-float pair whenever t_direct_ok
holds, and that pair must be the exact sum (which the reference's double
accumulation, t += step, also holds while the sum spans at most 53 bits)."""
import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def ff_add_step(h, l, b):
    s, e = two_sum(h, b)
    l2 = (l + e).astype(f32)
    h2 = (s + l2).astype(f32)
    lo = (l2 - (h2 - s).astype(f32)).astype(f32)
    return h2, lo


def t_after(t0, step, k):
    kf = k.astype(f32)
    p = (kf * step).astype(f32)
    # fma(k, step, -p): the product's rounding error, exact in float64 and in float32
    pe = (kf.astype(np.float64) * step.astype(np.float64) - p.astype(np.float64)).astype(f32)
    s, e = two_sum(t0, p)
    l = (e + pe).astype(f32)
    h = (s + l).astype(f32)
    lo = (l - (h - s).astype(f32)).astype(f32)
    return h, lo


def ilogb(x):
    return np.frexp(np.abs(x).astype(np.float64))[1] - 1


def t_direct_ok(t0, step, far):
    top = ilogb(np.maximum(np.abs(far), np.abs(t0)) + 4.0 * step)
    es = ilogb(step)
    q = np.where(t0 == 0, es, np.minimum(ilogb(t0), es)) - 23
    return (step > 0) & np.isfinite(t0) & np.isfinite(far) & (top - q <= 44)


def test_jump_equals_sequential_steps_and_the_exact_sum():
    rng = np.random.default_rng(11)
    n = 20000
    near = rng.uniform(0, 8, n).astype(f32)
    far = (near + rng.uniform(0.05, 8, n)).astype(f32)
    # the march's step: min((far - near) / min_step, step_size), and arbitrary small steps
    step = np.minimum(((far - near) / f32(8)).astype(f32), f32(0.01))
    small = rng.random(n) < 0.3
    step[small] = rng.uniform(2e-5, 0.02, small.sum()).astype(f32)
    jit = rng.uniform(0, 1, n).astype(f32)
    t0 = (near + (step * jit).astype(f32)).astype(f32)
    t0[:50] = 0.0
    ok = t_direct_ok(t0, step, far)
    assert ok.mean() > 0.95
    h, l = t0.copy(), np.zeros(n, f32)
    checked = 0
    for k in range(1, 1201):
        h, l = ff_add_step(h, l, step)
        live = ok & (h < far)
        if k % 7 and k < 1190:
            continue
        dh, dl = t_after(t0, step, np.full(n, k, np.int64))
        assert np.array_equal(dh[live], h[live]) and np.array_equal(dl[live], l[live]), k
        exact = t0.astype(np.float64) + k * step.astype(np.float64)
        assert np.array_equal(h[live].astype(np.float64) + l[live].astype(np.float64), exact[live]), k
        checked += int(live.sum())
    assert checked > 1_000_000
