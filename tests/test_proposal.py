"""The learned crossing proposal (csrc/proposal.cu) against its NumPy restatement
(oracle/proposal_ref.py): features, the BF16 forward, the backward (every
parameter's gradient), Adam, the fused inference kernel, training on plain
flights, and flights with proposals identical to plain flights.

Tolerances: the kernels and the restatement round the same GEMM operands to
BF16; the kernels accumulate in FP32 and the restatement in FP64, so an
activation can round to the neighbouring BF16 value now and then (2^-8
relative): outputs within 1e-2 absolute, gradients within 3e-2 relative L2 per
tensor."""
import numpy as np
import pytest

from gpis_extend_gb300 import abi, proposal, workloads
from oracle import proposal_ref as R


def random_features(n, rng):
    f = rng.normal(size=(n, 24)).astype(np.float32)
    f[:, 20] = (rng.random(n) < 0.5).astype(np.float32)
    return f


def random_targets(n, rng):
    return np.stack([rng.uniform(0.02, 0.98, n), (rng.random(n) < 0.7).astype(np.float64)], axis=1).astype(np.float32)


def _bf16_bits(x):
    """Round float32 to BF16 (nearest even); the bit patterns and their values."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return u, (u.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(32, 16), (64, 32), (128, 128), (96, 48)])
def test_gpu_tensor_core_gemm_check(gpu, n, k):
    """The tcgen05 path (operand layout, descriptors, tensor-memory read-back)
    against an FP64 product of the same BF16 operands; FP32 accumulation."""
    from gpis_extend_gb300 import runtime
    rng = np.random.default_rng(n * 1000 + k)
    ab, av = _bf16_bits(rng.normal(size=(128, k)))
    bb, bv = _bf16_bits(rng.normal(size=(n, k)))
    d = runtime.debug_tc_gemm(ab, bb)
    want = av.astype(np.float64) @ bv.astype(np.float64).T
    assert np.abs(d - want).max() < 1e-4 * np.sqrt(k) * 4


def test_reference_backward_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(R, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(0)
    p = R.unflatten(proposal.init_params(1).astype(np.float64))
    f = rng.normal(size=(16, 24))
    tg = random_targets(16, rng)
    o, c = R.forward(p, f)
    _, g = R.loss_and_grad_out(o, tg[:, 0].astype(np.float64), tg[:, 1] > 0)
    gflat = R.flatten(R.backward(p, c, g))
    flat = R.flatten(p)
    for i in rng.choice(len(flat), 30, replace=False):
        e = 1e-6
        fp, fm = flat.copy(), flat.copy()
        fp[i] += e
        fm[i] -= e
        lp = R.loss_and_grad_out(R.forward(R.unflatten(fp), f)[0], tg[:, 0], tg[:, 1] > 0)[0]
        lm = R.loss_and_grad_out(R.forward(R.unflatten(fm), f)[0], tg[:, 0], tg[:, 1] > 0)[0]
        fd = (lp - lm) / (2 * e)
        assert abs(fd - gflat[i]) <= 1e-4 * (abs(fd) + 1e-3), (i, fd, gflat[i])


def test_init_params_layout():
    p = proposal.init_params(3)
    assert p.size == R.n_params() == 18336
    d = R.unflatten(p)
    assert np.all(d["w_ih"][:, 2:] == 0) and np.all(d["w1"][:, 40:] == 0)
    assert np.all(d["w4"][25:] == 0) and np.all(d["b4"][25:] == 0)


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    from gpis_extend_gb300 import runtime
    return torch, runtime


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["sphere", "torus"])
def test_gpu_features_match_restatement(gpu, kind):
    torch, runtime = gpu
    if kind == "sphere":
        desc = workloads.sphere_medium()
        prim = workloads.sphere_flights(4096, desc)
        half = 1.5
    else:
        desc = proposal.config2_medium()
        prim = workloads.torus_flights(4096, desc)
        half = 2.0
    with runtime.Context(desc) as ctx:
        rec = ctx.trace_host(prim)
        sec, _ = workloads.secondary_flights(prim, rec, desc, half=half)
        for b in (prim, sec):
            dev = runtime.DeviceFlights(b)
            f = runtime.proposal_features(ctx, dev).cpu().numpy()
            ref = R.features(desc, b.origin_near, b.dir_far, b.seeds, b.prev)
            err = np.abs(f - ref)
            assert np.all(err <= 1e-4 * (1 + np.abs(ref))), (np.unravel_index(np.argmax(err), err.shape), err.max())


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_reference(gpu):
    torch, runtime = gpu
    rng = np.random.default_rng(4)
    n = 512
    f = random_features(n, rng)
    tg = random_targets(n, rng)
    params = proposal.init_params(5)
    with runtime.Proposal(params) as prop:
        fd = torch.from_numpy(f).cuda()
        td = torch.from_numpy(tg).cuda()
        out = prop.forward(fd).cpu().numpy()
        grad, loss = prop.gradient(fd, td)
    p = R.unflatten(params.astype(np.float64))
    o, cache = R.forward(p, f)
    assert np.max(np.abs(out[:, :25] - o[:, :25])) <= 1e-2
    assert np.median(np.abs(out[:, :25] - o[:, :25])) <= 1e-4
    lref, g = R.loss_and_grad_out(o, tg[:, 0].astype(np.float64), tg[:, 1] > 0)
    assert abs(loss - lref) <= 1e-3 * (1 + abs(lref))
    gref = R.backward(p, cache, g)
    gd = R.unflatten(grad.astype(np.float64))
    for name, _ in R.PARAMS:
        a, b = gd[name], gref[name]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        print(name, "relative L2", rel)
        assert rel <= 3e-2, (name, rel)


@pytest.mark.gpu
def test_gpu_training_gemms_tcgen05_match_mma_sync(gpu):
    """The training GEMMs on tcgen05 (tensor-memory accumulators) against the warp-level
    mma.sync kernels: the same BF16 operands accumulated in FP32 in another order, so
    the outputs agree to 1e-5 relative and every gradient tensor to 1e-4 relative L2."""
    torch, runtime = gpu
    rng = np.random.default_rng(14)
    n = 1008
    f = torch.from_numpy(random_features(n, rng)).cuda()
    tg = torch.from_numpy(random_targets(n, rng)).cuda()
    params = proposal.init_params(8)
    got = {}
    for k in ("tc2", "mma"):
        with runtime.Proposal(params) as prop:
            prop.set_kernel(k)
            out = prop.forward(f).cpu().numpy()
            grad, loss = prop.gradient(f, tg)
        got[k] = (out, grad, loss)
    (o1, g1, l1), (o2, g2, l2) = got["tc2"], got["mma"]
    assert np.max(np.abs(o1 - o2)) <= 1e-5 * (1 + np.max(np.abs(o2)))
    assert abs(l1 - l2) <= 1e-5 * (1 + abs(l2))
    a, b = R.unflatten(g1.astype(np.float64)), R.unflatten(g2.astype(np.float64))
    for name, _ in R.PARAMS:
        rel = np.linalg.norm(a[name] - b[name]) / max(np.linalg.norm(b[name]), 1e-12)
        assert rel <= 1e-4, (name, rel)


@pytest.mark.gpu
def test_gpu_adam_step_matches_reference(gpu):
    torch, runtime = gpu
    rng = np.random.default_rng(6)
    n = 256
    f = torch.from_numpy(random_features(n, rng)).cuda()
    t = torch.from_numpy(random_targets(n, rng)).cuda()
    params = proposal.init_params(7)
    with runtime.Proposal(params) as prop:
        g0, _ = prop.gradient(f, t)
        prop.train_step(f, t, 1e-2)
        p1 = prop.get_params()
        g1, _ = prop.gradient(f, t)
        prop.train_step(f, t, 1e-2)
        p2 = prop.get_params()
    flat, m, v = params.astype(np.float64), np.zeros(params.size), np.zeros(params.size)
    flat, m, v = R.adam(flat, g0.astype(np.float64), m, v, 1, 1e-2)
    assert np.max(np.abs(p1 - flat)) <= 1e-5
    flat, m, v = R.adam(p1.astype(np.float64), g1.astype(np.float64), m, v, 2, 1e-2)
    assert np.max(np.abs(p2 - flat)) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["tc2", "tc1", "mma"])
def test_gpu_fused_inference_matches_unfused(gpu, kernel):
    """Each fused inference kernel (tcgen05 with two or one 128-flight tiles per
    block, warp mma.sync) against the unfused BF16 forward."""
    torch, runtime = gpu
    desc = proposal.config2_medium()
    b = workloads.torus_flights(2048, desc)
    params = proposal.init_params(9)
    with runtime.Context(desc) as ctx, runtime.Proposal(params) as prop:
        prop.set_kernel(kernel)
        dev = runtime.DeviceFlights(b)
        f = runtime.proposal_features(ctx, dev)
        iv = prop.infer(dev, f).cpu().numpy()
        out = prop.forward(f).cpu().numpy()
    logits = out[:, :8]
    top2 = np.sort(logits, axis=1)[:, -2:]
    clear = (top2[:, 1] - top2[:, 0]) > 1e-2
    ua, ub, q = R.interval(out.astype(np.float64))
    near, far = b.origin_near[:, 3], b.dir_far[:, 3]
    tm = far - near
    # an untrained network's logits are close together: compare the rows whose
    # leading component is clear of the second by more than the two paths differ
    assert clear.sum() >= 200
    assert np.all(np.abs((iv[clear, 0] - near[clear]) / tm[clear] - ua[clear]) <= 2e-2)
    assert np.all(np.abs((iv[clear, 1] - near[clear]) / tm[clear] - ub[clear]) <= 2e-2)
    assert np.all(np.abs(iv[:, 2] - q) <= 1e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["tc2", "tc1"])
def test_gpu_tensor_core_wait_time_out_is_reported(gpu, kernel):
    """The tensor-memory kernel's bounded completion wait, made to run out: with a
    poll limit of 0 every MMA round gives up at once, the threads stop together,
    wait (with the default bound) for the MMAs already committed, free their
    tensor memory and raise the flag.  The next call reports GPIS_EIO without
    launching; with the limit restored the call after succeeds and gives the same
    intervals as before (the context is still usable)."""
    torch, runtime = gpu
    desc = proposal.config2_medium()
    b = workloads.torus_flights(1024, desc, seed=3)
    with runtime.Context(desc) as ctx, runtime.Proposal(proposal.init_params(2)) as prop:
        prop.set_kernel(kernel)
        dev = runtime.DeviceFlights(b)
        f = runtime.proposal_features(ctx, dev)
        good = prop.infer(dev, f).cpu().numpy()
        prop.set_wait_limit(0)
        prop.infer(dev, f)
        torch.cuda.synchronize()
        prop.set_wait_limit()
        with pytest.raises(abi.GpisError) as e:
            prop.infer(dev, f)
        assert e.value.code == abi.GPIS_EIO
        assert "timed out" in str(e.value)
        again = prop.infer(dev, f).cpu().numpy()
        torch.cuda.synchronize()
        if kernel == "tc2":
            # the training GEMMs' wait: the gradient call that timed out reports it
            rng = np.random.default_rng(1)
            ft = torch.from_numpy(random_features(256, rng)).cuda()
            tt = torch.from_numpy(random_targets(256, rng)).cuda()
            g0, _ = prop.gradient(ft, tt)
            prop.set_wait_limit(0)
            with pytest.raises(abi.GpisError) as e2:
                prop.gradient(ft, tt)
            assert e2.value.code == abi.GPIS_EIO
            prop.set_wait_limit()
            g1, _ = prop.gradient(ft, tt)
            assert np.allclose(g0, g1, rtol=1e-5, atol=1e-7)
    assert np.array_equal(again.view(np.uint32), good.view(np.uint32))


@pytest.mark.gpu
def test_gpu_tensor_core_inference_tiles(gpu):
    """The tcgen05 kernels with one and two tiles per block give the same bits; a
    ragged batch (not a multiple of 128) gives the rows of the full batch; the
    mma.sync kernel agrees to the BF16 rounding of the activations."""
    torch, runtime = gpu
    desc = proposal.config2_medium()
    b = workloads.torus_flights(4096, desc, seed=5)
    with runtime.Context(desc) as ctx, runtime.Proposal(proposal.init_params(4)) as prop:
        dev = runtime.DeviceFlights(b)
        f = runtime.proposal_features(ctx, dev)
        got = {}
        for k in ("tc2", "tc1", "mma"):
            prop.set_kernel(k)
            got[k] = prop.infer(dev, f).cpu().numpy()
        prop.set_kernel("tc2")
        part = runtime.DeviceFlights(b.subset(np.arange(1000)))
        fp = f[:1000].contiguous()
        ragged = prop.infer(part, fp).cpu().numpy()
    assert np.array_equal(got["tc2"].view(np.uint32), got["tc1"].view(np.uint32))
    assert np.array_equal(ragged.view(np.uint32), got["tc2"][:1000].view(np.uint32))
    assert np.all(np.isfinite(got["tc2"]))
    assert np.abs(got["tc2"][:, 2] - got["mma"][:, 2]).max() <= 1e-2
    near, far = b.origin_near[:, 3], b.dir_far[:, 3]
    m_tc = got["tc2"][:, 3]
    m_mma = got["mma"][:, 3]
    agree = np.abs(m_tc - m_mma) <= 2e-2
    assert agree.mean() > 0.9
    assert np.all((got["tc2"][:, 0] >= near - 1e-4) & (got["tc2"][:, 1] <= far + 1e-4))


@pytest.mark.gpu
def test_gpu_training_learns_and_proposals_keep_flights(gpu):
    """Training on plain config-2 flights lowers the loss and puts more crossings
    inside the proposed intervals; proposed flights equal plain flights bit for bit."""
    torch, runtime = gpu
    desc = proposal.config2_medium()
    batches = proposal.flight_set(desc, 1 << 15)
    with runtime.Context(desc) as ctx, runtime.Proposal(proposal.init_params(0)) as prop:
        f, t = proposal.dataset(ctx, batches)
        hist, secs = proposal.train(prop, f, t, steps=300, batch=4096, lr=3e-3, log_every=50)
        print("loss", hist, "seconds", secs)
        assert hist[-1][1] < hist[0][1] - 0.2
        test = workloads.torus_flights(1 << 14, desc, seed=23)
        dev = runtime.DeviceFlights(test)
        ctx.submit(dev)
        torch.cuda.synchronize()
        plain = dev.rec.cpu().numpy().copy()
        feats = runtime.proposal_features(ctx, dev)
        iv = prop.infer(dev, feats)
        dev.rec.zero_()
        runtime.submit_proposed(ctx, dev, iv)
        torch.cuda.synchronize()
        prop_rec = dev.rec.cpu().numpy()
        inside, hits = proposal.interval_hits(iv.cpu().numpy(), test, plain)
        print("crossings inside the proposed interval", inside, "of", hits)
        assert inside > 0.5
    assert np.array_equal(plain.view(np.uint32), prop_rec.view(np.uint32))


@pytest.mark.gpu
def test_gpu_proposed_sphere_flights_identical_with_any_proposal(gpu):
    """Soundness: whatever the intervals, every flight's record is unchanged (the
    stationary sphere field, where the proposal lifts the skip cap)."""
    torch, runtime = gpu
    desc = workloads.sphere_medium()
    prim = workloads.sphere_flights(1 << 15, desc)
    rng = np.random.default_rng(1)
    with runtime.Context(desc) as ctx:
        dev = runtime.DeviceFlights(prim)
        ctx.submit(dev)
        torch.cuda.synchronize()
        plain = dev.rec.cpu().numpy().copy()
        far = prim.dir_far[:, 3]
        for mode in ("far", "random", "zero"):
            iv = np.zeros((prim.n, 4), np.float32)
            if mode == "far":
                iv[:, 0] = far
            elif mode == "random":
                iv[:, 0] = rng.uniform(0, 1, prim.n) * far
            iv[:, 1] = far
            ivd = torch.from_numpy(iv).cuda()
            dev.rec.zero_()
            runtime.submit_proposed(ctx, dev, ivd)
            torch.cuda.synchronize()
            got = dev.rec.cpu().numpy()
            assert np.array_equal(plain.view(np.uint32), got.view(np.uint32)), mode
