"""The learned crossing proposal: parameter initialisation, training data from the
plain flight kernels, the training loop and the proposed flight path.

The network and its kernels live in csrc/proposal.cu (gpis_proposal_*); this
module drives them through runtime.Proposal.  Training data are flights the
plain GPU sampler itself traced: the features of each flight and its target
(u* = (t_hit - near) / (far - near), hit).
"""
import time

import numpy as np

from . import abi, workloads

HID, N_IN, MLP_IN, WIDTH, N_OUT = 32, 16, 48, 64, 32
# (name, shape (out, in), fan-in of the default uniform initialisation)
LAYOUT = [("w_ih", (3 * HID, N_IN), 2), ("b_ih", (3 * HID,), HID), ("w_hh", (3 * HID, HID), HID),
          ("b_hh", (3 * HID,), HID), ("w1", (WIDTH, MLP_IN), 40), ("b1", (WIDTH,), 40),
          ("w2", (WIDTH, WIDTH), WIDTH), ("b2", (WIDTH,), WIDTH), ("w3", (WIDTH, WIDTH), WIDTH),
          ("b3", (WIDTH,), WIDTH), ("w4", (N_OUT, WIDTH), WIDTH), ("b4", (N_OUT,), WIDTH)]


def init_params(seed=0):
    """U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for every weight and bias; the padded input
    columns (w_ih 2..15, w1 40..47) and output rows (25..31) are zero."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape, fan_in in LAYOUT:
        bound = 1.0 / np.sqrt(fan_in)
        w = rng.uniform(-bound, bound, shape)
        if name == "w_ih":
            w[:, 2:] = 0.0
        elif name == "w1":
            w[:, 40:] = 0.0
        elif name == "w4":
            w[25:, :] = 0.0
        elif name == "b4":
            w[25:] = 0.0
        parts.append(w.ravel())
    return np.concatenate(parts).astype(np.float32)


def config2_medium():
    """The three-octave nonstationary torus-union-plane field of the image workload."""
    return workloads.torus_plane_medium(nonstationary=True, octaves=3, sigma_a=0.0, sigma_s=1.0)


def flight_set(desc, n, seed=11, half=2.0):
    """Primary flights through the torus-plane field and the conditioned secondary
    flights from their hits (traced by the plain kernels): a list of FlightBatch."""
    from . import runtime
    prim = workloads.torus_flights(n, desc, seed=seed, half=half)
    with runtime.Context(desc) as ctx:
        rec = ctx.trace_host(prim)
    sec, _ = workloads.secondary_flights(prim, rec, desc, seed=seed, half=half)
    return [prim, sec]


def targets(batch, rec):
    """(u*, hit) per flight: u* = (t - near) / (far - near) at hits, 1 at misses."""
    res = abi.unpack_results(rec)
    near, far = batch.origin_near[:, 3].astype(np.float64), batch.dir_far[:, 3].astype(np.float64)
    hit = res["hit"] & (res["status"] == abi.FLIGHT_OK)
    u = np.where(hit, (res["t"] - near) / np.maximum(far - near, 1e-30), 1.0)
    return np.stack([np.clip(u, 0.0, 1.0), hit.astype(np.float64)], axis=1).astype(np.float32)


def dataset(ctx, batches):
    """Device tensors (features (n, 24), targets (n, 2)) of the batches, traced by the
    plain kernels of ctx; n is cut to a multiple of 16."""
    import torch
    from . import runtime
    feats, tg = [], []
    for b in batches:
        dev = runtime.DeviceFlights(b)
        ctx.submit(dev)
        f = runtime.proposal_features(ctx, dev)
        torch.cuda.synchronize()
        rec = dev.rec.cpu().numpy()
        feats.append(f)
        tg.append(torch.from_numpy(targets(b, rec)).cuda())
    f = torch.cat(feats)
    t = torch.cat(tg)
    n = (f.shape[0] // 16) * 16
    return f[:n].contiguous(), t[:n].contiguous()


def train(prop, feats, targets_, steps, batch=8192, lr=3e-3, seed=0, log_every=0):
    """Adam on random minibatches of the device dataset; returns (loss history, seconds)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = feats.shape[0]
    hist = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        idx = torch.randint(0, n, (batch,), device="cuda", generator=g)
        fb = feats.index_select(0, idx).contiguous()
        tb = targets_.index_select(0, idx).contiguous()
        want = log_every and (k % log_every == 0 or k == steps - 1)
        loss = prop.train_step(fb, tb, lr, want_loss=bool(want))
        if want:
            hist.append((k, loss))
    torch.cuda.synchronize()
    return hist, time.perf_counter() - t0


def interval_hits(intervals, batch, rec):
    """Fraction of hits whose t lies inside the proposed [t_a, t_b]; proposed misses."""
    res = abi.unpack_results(rec)
    hit = res["hit"] & (res["status"] == abi.FLIGHT_OK)
    iv = np.asarray(intervals)
    inside = hit & (res["t"] >= iv[:, 0]) & (res["t"] <= iv[:, 1])
    return float(inside.sum() / max(1, hit.sum())), int(hit.sum())
