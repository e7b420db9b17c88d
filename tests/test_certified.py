"""Certified crossing decisions (the resume pass that decides a crossing on fast
values when error bounds make the decision certain) against the precise evaluator
alone (GPIS_TUNE_PRECISE_DECISIONS = 1) and against the oracle.

The refinement after a crossing (SparseConvolutionNoiseMedium.cpp:296-330) takes
the sign of the field at t = ta + fac * step and compares fac with 0.01 after
each x0.9 back-off.  The certified pass takes those decisions only when they
cannot differ from the reference's, so every status, hit and back-off must be the
precise path's, misses bit for bit, and a hit's t may move only by the bound on
the refinement point (step * dfac, far below 1e-5 on these fields)."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def _trace_both(desc, flights):
    from gpis_extend_gb300 import runtime
    with runtime.Context(desc) as ctx:
        assert ctx.tune(abi.TUNE_PRECISE_DECISIONS) == 0
        cert = ctx.trace_host(flights)
        ctx.tune(abi.TUNE_PRECISE_DECISIONS, 1)
        precise = ctx.trace_host(flights)
        with pytest.raises(abi.GpisError):
            ctx.tune(abi.TUNE_PRECISE_DECISIONS, 2)
    return cert, precise


def _agree(cert, precise):
    c, p = abi.unpack_results(cert), abi.unpack_results(precise)
    assert np.array_equal(c["status"], p["status"])
    assert np.array_equal(c["hit"], p["hit"])
    miss = ~c["hit"]
    assert np.array_equal(cert[miss].view(np.uint32), precise[miss].view(np.uint32))
    hit = c["hit"]
    dt = np.abs(c["t"][hit].astype(np.float64) - p["t"][hit])
    # back-off to t = 0 on one side only would be a decision that differed
    assert np.array_equal(c["t"][hit] == 0, p["t"][hit] == 0)
    return hit, dt


@pytest.mark.parametrize("context", [abi.CTX_RENEWAL_PLUS, abi.CTX_RENEWAL])
def test_gpu_certified_decisions_equal_precise(context):
    desc = workloads.sphere_medium(context=context)
    prim = workloads.sphere_flights(1 << 18, desc)
    cert, precise = _trace_both(desc, prim)
    hit, dt = _agree(cert, precise)
    print(f"primary: {hit.sum()} hits, max |dt| {dt.max():.3e}, identical t on {np.mean(dt == 0):.4f}")
    assert hit.sum() > 0.9 * len(hit)
    assert dt.max() <= 1e-5
    # the conditioned secondaries (Renewal / Renewal+ conditioning at each hit)
    sec, _ = workloads.secondary_flights(prim, precise, desc)
    cert2, precise2 = _trace_both(desc, sec)
    hit2, dt2 = _agree(cert2, precise2)
    print(f"secondary: {hit2.sum()} hits, max |dt| {dt2.max() if hit2.any() else 0:.3e}")
    assert hit2.sum() > 0
    assert dt2.max() <= 1e-5
    # and both against the oracle on a sample
    idx = np.arange(0, sec.n, 16)
    sub = sec.subset(idx)
    ref = oracle.trace_flights(desc, sub)
    st = oracle.compare_flights(cert2[idx], ref, desc.sigma, 1.5)
    assert st["hit_disagreements"] == 0 and st["t_outliers"] == 0, st
