"""Benchmark of the GPIS ray-flight path on GB300.

Workload (one "step"): the batched flight microbenchmark -- 2^22 primary flights
through the stationary SE field over the unit-sphere SDF (sigma 0.05, l 0.1,
localScale 3, 8 impulses per cell, cell hash seeded 1, 1D noise, Renewal+,
step 0.01, min_step 8), origins on a radius-3 sphere aimed at uniform points of
the unit ball (seed 7), clipped to the cube |x|,|y|,|z| <= 1.5; followed by the
conditioned secondary flights reflected at every primary hit.  Inputs are
seeded synthetic data generated once; every step re-traces all flights.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --workload image0|image2 [--size S] [--spp P] [--steps K]
    python bench.py --workload learned [--flights N] [--train-flights N] [--train-steps K]
    python bench.py --workload batch [--steps K] [--spp-scale F] [--no-learned]

The image workloads render with gpis_render (the wavefront path tracer around
the medium) and report the flights traced per second of render:
image0 = 256 x 256, 16 spp, 4 bounces, the sphere field with 3D noise and
Renewal, Lambert albedo 0.8, a 1 x 1 quad light at y = 3; image2 = 1024 x 1024,
256 spp, 8 bounces, the nonstationary three-octave torus-union-plane field with
1D noise and Renewal+, a copper conductor phase with 1D NEE (for the octave sum
the NEE law is that of the summed transverse gradient).

The learned arm: a proposal network (GRU 32 + 3 x 64 GELU MLP -> 8-component
logistic mixture over the crossing interval, BF16 tensor-core kernels) trained
on flights the plain kernels traced, then features + inference + the march with
proposals on the same flights.  The default line carries it as `learned` (a
network trained on 2^20 disjoint sphere flights); `--workload learned` runs it on
the three-octave torus-plane field with 2^22 + secondary training flights.

Prints one JSON line (rank 0).  `value` is device-resident throughput (flights/s,
inputs already in HBM, 512 MiB of flight streams > L2 so no flush is needed);
`e2e` is the same metric through gpis_flights_trace_host from pinned host
buffers (copies inside the timed region); `roofline` is the march kernel's
algorithmic FP32 rate against cuBLAS SGEMM measured in the same run;
`cpu_baseline` is the oracle (CPU restatement) on all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GPIS ray-flights/s on 1 GB300: plain vs learned proposal at equal image RMSE"
UNIT = "flights/s"
WORKLOAD = ("batched sphere-field flights: 2^22 primary (seed 7, radius-3 origins, cube 1.5) + "
            "conditioned secondary reflections, 1D SE Renewal+, sigma 0.05, l 0.1, N 8, step 0.01")


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi SM clock and throttle-reason samples during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        self.lines += [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def sgemm_peak_tflops(torch):
    """FP32 FFMA peak as cuBLAS SGEMM delivers it (TF32 off), best of 5, 8192^3."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        for _ in range(2):
            torch.mm(a, b)
        best = None
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.mm(a, b)
            e.record()
            torch.cuda.synchronize()
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
        del a, b
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def load_traffic():
    """Per-flight DRAM bytes of the march kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "march_dram.json")
    if not os.path.exists(p):
        return None
    try:
        return json.load(open(p))
    except (OSError, ValueError):
        return None


def cpu_baseline(desc, prim, sec, gpu_recs=None):
    """The oracle on all host cores over the whole workload (every primary and
    secondary flight of one step), timed; its records are the parity check of the
    GPU's records of the same flights (gpu_recs: primary, secondary).  Beside it,
    one thread on a sample of about a second."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    rp = oracle.trace_flights(desc, prim, n_threads=0)
    rs = oracle.trace_flights(desc, sec, n_threads=0)
    dt = time.perf_counter() - t0
    rate = (prim.n + sec.n) / dt
    m1 = int(min(prim.n, max(1024, rate / cores / 2)))
    s1 = min(m1, sec.n)
    t1 = time.perf_counter()
    oracle.trace_flights(desc, prim.subset(np.arange(m1)), n_threads=1)
    oracle.trace_flights(desc, sec.subset(np.arange(s1)), n_threads=1)
    dt1 = time.perf_counter() - t1
    base = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the whole workload: {prim.n} primary + {sec.n} secondary flights, oracle (C restatement, "
                      f"float mode) on {cores} threads, {dt:.1f} s",
            "one_thread": {"value": (m1 + s1) / dt1, "unit": UNIT,
                           "sample": f"first {m1} primary + first {s1} secondary flights, {dt1:.1f} s"}}
    parity = None
    if gpu_recs is not None:
        parity = {}
        for name, g, c in (("primary", gpu_recs[0], rp), ("secondary", gpu_recs[1], rs)):
            parity[name] = oracle.compare_flights(g, c, desc.sigma, 1.5)
        tot = {k: sum(parity[x][k] for x in ("primary", "secondary"))
               for k in ("flights", "hit_disagreements", "hits", "t_outliers", "t_outliers_backoff",
                         "t_outliers_other")}
        tot["hit_agreement"] = 1.0 - tot["hit_disagreements"] / max(1, tot["flights"])
        tot["hits_within_t_tol"] = 1.0 - tot["t_outliers"] / max(1, tot["hits"])
        tot["bars"] = ("hit/miss agreement >= 0.9999; |dt| <= 1e-4 x scene scale (1.5) on >= 0.9999 of hits, "
                       "every outlier a back-off case; miss values within 1e-5 of sigma; normals within 2e-3")
        tot["pass"] = bool(tot["hit_agreement"] >= 0.9999 and tot["hits_within_t_tol"] >= 0.9999
                           and tot["t_outliers_other"] == 0
                           and all(parity[x]["status_agreement"] == 1.0 and parity[x]["miss_t_equal"] == 1.0
                                   and parity[x]["miss_value_within_tol"] >= 0.9999
                                   and parity[x]["normals_within_tol"] >= 0.999 for x in ("primary", "secondary")))
        parity["all"] = tot
    return base, parity


def run_reference(args, world, rank):
    """The reference arm: the reference's CPU path for this workload, timed on the
    host cores.  The reference CPU library does not build here (Boost, TBB,
    OpenVDB, OpenEXR absent), so the arm runs the oracle port with all threads."""
    if rank != 0:
        return
    from gpis_extend_gb300 import abi, workloads
    from oracle import oracle
    desc = workloads.sphere_medium()
    n = args.flights
    prim = workloads.sphere_flights(n, desc)
    # secondary flights come from the oracle's own primary hits on the sampled range
    cores = os.cpu_count() or 1
    per_step = args.ref_sample
    prim_s = prim.subset(np.arange(per_step))
    rec = oracle.trace_flights(desc, prim_s)
    sec_s, _ = workloads.secondary_flights(prim_s, rec, desc)
    for _ in range(args.warmup):
        oracle.trace_flights(desc, prim_s)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.trace_flights(desc, prim_s)
        oracle.trace_flights(desc, sec_s)
    dt = time.perf_counter() - t0
    flights = args.steps * (prim_s.n + sec_s.n)
    value = flights / dt
    sample = (f"per step the first {prim_s.n} primary flights of the workload and their "
              f"{sec_s.n} conditioned secondaries, oracle port on {cores} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "arm": "reference CPU path (oracle port: the reference "
                   "CPU library needs Boost/TBB/OpenVDB/OpenEXR, absent on this image)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


IMAGE_WORKLOADS = {
    "image0": dict(medium="sphere_3d", size=256, spp=16, bounces=4,
                   text="image render: 256x256 pinhole at z=4, 16 spp, 4 bounces, sphere SDF field, 3D SE noise "
                        "sigma 0.05 l 0.1 N 8, Renewal, Lambert albedo 0.8, 1x1 quad light at y=3"),
    "image2": dict(medium="torus_oct_nee", size=1024, spp=256, bounces=8, phase="conductor", box=2.0,
                   text="image render: 1024x1024, 256 spp, 8 bounces, torus (R 1, r 0.35) union plane y=-0.5, "
                        "l(p)=0.11+0.09 sin3x cos2z, 3 octaves sigma 0.04/0.02/0.01, 1D noise, Renewal+, "
                        "copper conductor phase with 1D NEE (the octave sum's law), cube 2, 1x1 quad light at y=3"),
}


def train_proposal(ctx, desc, make_flights, n_train, steps, batch, half, seed=101):
    """The learned proposal trained on flights the plain kernels traced (primaries of
    make_flights and the conditioned secondaries at their hits)."""
    from gpis_extend_gb300 import proposal, runtime, workloads
    prim = make_flights(n_train, desc, seed=seed, half=half)
    rec = ctx.trace_host(prim)
    sec, _ = workloads.secondary_flights(prim, rec, desc, seed=seed, half=half)
    f, t = proposal.dataset(ctx, [prim, sec])
    prop = runtime.Proposal(proposal.init_params(0))
    hist, secs = proposal.train(prop, f, t, steps=steps, batch=batch, lr=3e-3, log_every=max(1, steps // 4))
    info = {"flights": int(f.shape[0]), "steps": steps, "batch": batch, "seconds": secs,
            "loss": [[k, round(v, 4)] for k, v in hist]}
    return prop, info


def learned_arm(ctx, prop, batches, devs, steps, stream, plain_ms):
    """Per step and batch: features, fused inference, the march with proposals.  Returns
    the arm's summary (flights/s, ratio to the plain arm, interval statistics, identity
    of every record with the plain records)."""
    import torch
    from gpis_extend_gb300 import abi, autotune, proposal, runtime
    plain = [d.rec.clone() for d in devs]
    feats = [torch.empty((d.n, 24), dtype=torch.float32, device="cuda") for d in devs]
    ivs = [torch.empty((d.n, 4), dtype=torch.float32, device="cuda") for d in devs]

    # the ceiling of this use of a proposal: the true crossing of every flight (from
    # the plain records) as its interval, so the march may skip up to `cap` certified
    # steps per evaluation everywhere before the crossing; the march alone is timed
    def true_intervals(d, rec):
        r = rec.view(-1, 8)
        hit = r[:, 5] == 0.0
        far = d.dir_far[:, 3]
        ta = torch.where(hit, r[:, 0], far)
        iv = torch.zeros((d.n, 4), dtype=torch.float32, device="cuda")
        iv[:, 0] = ta
        iv[:, 1] = ta
        iv[:, 2] = (~hit).float()
        return iv

    true_ivs = [true_intervals(d, p) for d, p in zip(devs, plain)]

    def march_ms(intervals, reps):
        for d, iv in zip(devs, intervals):
            runtime.submit_proposed(ctx, d, iv, stream)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            for d, iv in zip(devs, intervals):
                runtime.submit_proposed(ctx, d, iv, stream)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    plain_march = plain_ms / steps
    ceiling = {}
    for cap in (16, 64, 256):
        ctx.tune(abi.TUNE_PROPOSED_SKIP_CAP, cap)
        ms_c = march_ms(true_ivs, max(2, steps // 2))
        same = all(torch.equal(p.view(torch.int32), d.rec.view(torch.int32)) for p, d in zip(plain, devs))
        ceiling[str(cap)] = {"march_ms_per_step": ms_c, "ratio_vs_plain": plain_march / ms_c,
                             "identical_to_plain": bool(same)}
    for d, f, iv in zip(devs, feats, ivs):
        runtime.proposal_features(ctx, d, stream, out=f)
        prop.infer(d, f, stream, out=iv)
    torch.cuda.synchronize()
    sched = autotune.tune_proposed_cap(ctx, devs, ivs)

    def step():
        for d, f, iv in zip(devs, feats, ivs):
            runtime.proposal_features(ctx, d, stream, out=f)
            prop.infer(d, f, stream, out=iv)
            runtime.submit_proposed(ctx, d, iv, stream)

    step()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    # the parts of one step, timed alone
    part = {}
    for name, fn in (("features", lambda d, f, iv: runtime.proposal_features(ctx, d, stream, out=f)),
                     ("inference", lambda d, f, iv: prop.infer(d, f, stream, out=iv)),
                     ("march", lambda d, f, iv: runtime.submit_proposed(ctx, d, iv, stream))):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for d, f, iv in zip(devs, feats, ivs):
            fn(d, f, iv)
        b.record(stream)
        torch.cuda.synchronize()
        part[name] = a.elapsed_time(b)
    # the fused inference alone with each of its kernels (the arm uses the default, tc2)
    kernels = {}
    for k in ("tc2", "tc1", "mma"):
        kernels[k + "_blocks_per_sm"] = prop.occupancy(k)
        prop.set_kernel(k)
        for d, f, iv in zip(devs, feats, ivs):
            prop.infer(d, f, stream, out=iv)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for d, f, iv in zip(devs, feats, ivs):
            prop.infer(d, f, stream, out=iv)
        b.record(stream)
        torch.cuda.synchronize()
        kernels[k] = a.elapsed_time(b)
    prop.set_kernel("tc2")
    for d, f, iv in zip(devs, feats, ivs):
        prop.infer(d, f, stream, out=iv)
    torch.cuda.synchronize()
    identical = all(torch.equal(p.view(torch.int32), d.rec.view(torch.int32)) for p, d in zip(plain, devs))
    inside, hits = 0.0, 0
    for b_, d, iv in zip(batches, devs, ivs):
        fr, h = proposal.interval_hits(iv.cpu().numpy(), b_, d.rec.cpu().numpy())
        inside += fr * h
        hits += h
    n = sum(d.n for d in devs)
    value = n * steps / (ms * 1e-3)
    plain_value = n * steps / (plain_ms * 1e-3)
    return {"value": value, "unit": UNIT, "ms_per_step": ms / steps, "plain_value": plain_value,
            "ratio_vs_plain": value / plain_value, "ms_per_part": part, "inference_ms_by_kernel": kernels,
            "plain_march_ms_per_step": plain_march, "schedule": sched,
            "ceiling_true_interval": ceiling,
            "ceiling_note": "the march with every flight's true crossing as its interval (skip cap per "
                            "evaluation before it), features and inference excluded: the most this use "
                            "of any proposal can buy",
            "inside_interval": inside / max(1, hits), "miss_fallback_rate": 1.0 - inside / max(1, hits),
            "identical_to_plain": bool(identical),
            "equal_image_rmse": "every flight record equals the plain arm's bit for bit, so images and their "
                                "RMSE are equal at equal spp"}


def run_learned(args):
    """The learned-proposal workload on its own line."""
    line = learned_workload(args)
    print(json.dumps(line), flush=True)


def learned_workload(args):
    """The learned-proposal workload on the three-octave torus-plane field: about 10^7
    training flights from the plain kernels (primaries and their conditioned
    secondaries), then plain vs learned on a fresh set, with the ceiling of the
    proposal's use beside it.  Returns the line."""
    import torch
    from gpis_extend_gb300 import build, proposal, runtime, workloads
    build.build()
    desc = proposal.config2_medium()
    ctx = runtime.Context(desc)
    prop, info = train_proposal(ctx, desc, workloads.torus_flights, args.train_flights, args.train_steps, 8192, 2.0)
    n = args.flights
    prim = workloads.torus_flights(n, desc, seed=23)
    rec = ctx.trace_host(prim)
    sec, _ = workloads.secondary_flights(prim, rec, desc, seed=23, half=2.0)
    devs = [runtime.DeviceFlights(prim), runtime.DeviceFlights(sec)]
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        for d in devs:
            ctx.submit(d, stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        for d in devs:
            ctx.submit(d, stream)
    end.record(stream)
    torch.cuda.synchronize()
    plain_ms = start.elapsed_time(end)
    learned = learned_arm(ctx, prop, [prim, sec], devs, args.steps, stream, plain_ms)
    clocks.stop()
    flights = prim.n + sec.n
    line = {
        "metric": METRIC, "value": learned["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": learned["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 field, bf16 network", "data": "synthetic",
        "config": {"workload": "learned proposal on the three-octave torus-plane field: GRU 32 + 3x64 GELU MLP "
                               "-> 8-component logistic mixture, BF16 weights, FP32 accumulation; primary flights "
                               "(radius-4 origins, seed 23, cube 2) + conditioned secondaries",
                   "arm": "learned", "flights_per_step": flights, "train": info},
        "plain": {"value": flights * args.steps / (plain_ms * 1e-3), "ms_per_step": plain_ms / args.steps},
        "e2e": {"value": None, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "device-resident arms only; the host entry is measured by the default workload"},
        "learned": learned,
        "gpu_launches": args.steps * 2 * 6,
        "clocks": clocks.summary(),
    }
    prop.close()
    ctx.close()
    return line


def run_batch(args):
    """The uneven image batch in one wavefront (gpis_render_batch): 64 media and images
    from seed 11, the render pass size from the autotuner, the bounce loop as a graph."""
    import torch
    from gpis_extend_gb300 import autotune, build, runtime, workloads
    build.build()
    media, scenes = workloads.config4_batch(spp_scale=args.spp_scale)
    ctx = runtime.Context(media)
    sched = autotune.tune_render(ctx, scenes)
    ctx.render_batch([workloads.render_scene(width=32, height=32, spp=1, max_bounces=4, medium=k)
                      for k in range(len(media))])
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    dev_ms, flights, wall, launches = 0.0, 0, 0.0, 0
    st = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        imgs, st = ctx.render_batch(scenes)
        wall += time.perf_counter() - t0
        dev_ms += st["ms"]
        flights += st["distance_flights"] + st["shadow_flights"]
        launches += st["launches"]
    clocks.stop()
    pixels = sum(sc.width * sc.height for sc in scenes)
    learned = None
    if not args.no_learned:
        # the learned arm side by side: a proposal trained on 2^15 flights through each
        # medium of the batch, then the same render with features, inference and the
        # proposed march in every round
        try:
            from gpis_extend_gb300 import proposal
            tf = workloads.batch_flights(media, 1 << 15)
            f, t = proposal.dataset(ctx, [tf])
            prop = runtime.Proposal(proposal.init_params(0))
            hist, secs = proposal.train(prop, f, t, steps=400, batch=8192, lr=3e-3, log_every=100)
            l_ms, l_imgs, ok = 0.0, None, True
            for _ in range(args.steps):
                l_imgs, lst = ctx.render_batch(scenes, proposal=prop)
                l_ms += lst["ms"]
            ok = all(np.array_equal(a, b) for a, b in zip(imgs, l_imgs))
            learned = {"value": flights / (l_ms * 1e-3), "unit": UNIT, "ms_per_step": l_ms / args.steps,
                       "ratio_vs_plain": dev_ms / l_ms, "identical_to_plain": bool(ok),
                       "train": {"flights": int(f.shape[0]), "steps": 400, "seconds": secs,
                                 "loss": [[k, round(v, 4)] for k, v in hist]}}
            prop.close()
        except Exception as e:  # noqa: BLE001
            learned = {"error": f"{type(e).__name__}: {e}"}
    line = {
        "metric": METRIC, "value": flights / (dev_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": 1, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "uneven image batch in one wavefront: 64 media from seed 11 (sphere/torus/plane/"
                               "torus-union-plane means, l 0.02-0.3, 1-3 octaves, Renewal or Renewal+), images "
                               "64^2-1024^2, 1-64 spp, 4 bounces, Lambert 0.8; bounce loop as a CUDA graph",
                   "arm": "plain", "scenes": len(scenes), "pixels": pixels, "paths_per_step": st["paths"],
                   "flights_per_step": flights // args.steps, "passes": st["passes"], "graphed": st["graphed"],
                   "spp_scale": args.spp_scale, "schedule": sched,
                   "sizes": sorted(int(sc.width) for sc in scenes), "spp": [int(sc.spp) for sc in scenes]},
        "e2e": {"value": flights / wall, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": pixels * 12},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "learned": learned,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_image(args):
    """An image workload: flights/s during gpis_render, device time (CUDA events in the
    renderer) and host wall time around the call (e2e)."""
    import torch
    from gpis_extend_gb300 import build, roofline, runtime, workloads
    from oracle import oracle
    cfg = IMAGE_WORKLOADS[args.workload]
    size = args.size or cfg["size"]
    spp = args.spp or cfg["spp"]
    build.build()
    desc = workloads.render_medium(cfg["medium"])
    sc = workloads.render_scene(width=size, height=size, spp=spp, max_bounces=cfg["bounces"],
                                phase=cfg.get("phase", "lambert"), box_half=cfg.get("box", 1.5))
    ctx = runtime.Context(desc)
    for _ in range(args.warmup):
        ctx.render(workloads.render_scene(width=64, height=64, spp=1, max_bounces=cfg["bounces"]))
    ctx.counters(reset=True)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    dev_ms, flights, wall, launches = 0.0, 0, 0.0, 0
    img = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        img, st = ctx.render(sc)
        wall += time.perf_counter() - t0
        dev_ms += st["ms"]
        flights += st["distance_flights"] + st["shadow_flights"]
        launches += st["launches"]
    clocks.stop()
    graphed = st["graphed"]
    value = flights / (dev_ms * 1e-3)
    # the march kernels' share for the roofline: one more render with per-kernel events
    # (rounds launched directly while profiling)
    ctx.counters(reset=True)
    ctx.profile_read(reset=True)
    ctx.profile(True)
    ctx.render(sc)
    ctx.profile(False)
    kms, klaunch = ctx.profile_read(reset=True)
    cnt = ctx.counters(reset=True)
    one_d = bool(desc.one_d_sampling)
    n_imp = int(desc.impulse_density)
    oct_factor = int(desc.n_octaves) if one_d else 1
    fpe = (roofline.flops_per_eval_1d(n_imp) * oct_factor) if one_d else roofline.flops_per_eval_3d(n_imp)
    evals = cnt["steps"] - cnt["skipped_steps"] + cnt["refine_evals"] + cnt["flights"] + (cnt["flights"] - cnt["hits"])
    achieved = evals * fpe / (kms[1] * 1e-3) / 1e12 if kms[1] > 0 else None
    peak = sgemm_peak_tflops(torch)
    # CPU baseline: the restatement renders one row per core through the middle of the
    # same scene, with the spp cut so that a row takes about cpu_seconds (a 1-spp row on
    # one thread sizes it); flights per second do not depend on the spp
    import copy
    cores = os.cpu_count() or 1
    mid = size // 2
    probe = copy.copy(sc)
    probe.spp = 1
    t0 = time.perf_counter()
    oracle.render_rows(desc, probe, mid, 1)
    t1 = time.perf_counter() - t0
    csc = copy.copy(sc)
    csc.spp = int(max(1, min(spp, round(args.cpu_seconds / max(t1, 1e-3)))))
    rows = int(max(1, min(size, cores)))
    row0 = max(0, mid - rows // 2)
    t0 = time.perf_counter()
    _, cc = oracle.render_rows(desc, csc, row0, rows)
    cdt = time.perf_counter() - t0
    cpu_flights = cc["distance_flights"] + cc["shadow_flights"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["text"], "width": size, "height": size, "spp": spp,
                   "max_bounces": cfg["bounces"], "arm": "plain", "paths_per_step": size * size * spp,
                   "flights_per_step": flights // args.steps, "graphed": graphed},
        "e2e": {"value": flights / wall, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": size * size * 3 * 4},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if achieved and peak else None, "traffic": None,
                     "kernel": "k_march (fast + resume passes) inside gpis_render (one profiled render)",
                     "flops_per_eval": fpe, "evals": evals, "march_ms": kms[1],
                     "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, best of 5, measured in this run"},
        "image": {"mean": float(img.mean()), "max": float(img.max())},
        "counters": cnt,
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": cpu_flights / cdt, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"rows {row0}-{row0 + rows - 1} of the same scene (through its middle) at "
                                   f"{csc.spp} spp, pt_oracle.c on {cores} threads, {cpu_flights} flights in "
                                   f"{cdt:.1f} s"},
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--flights", type=int, default=1 << 22)
    ap.add_argument("--ref-sample", type=int, default=1 << 16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true")
    ap.add_argument("--workload", default="flights", choices=["flights", "image0", "image2", "learned", "batch"])
    ap.add_argument("--spp-scale", type=float, default=1.0)
    ap.add_argument("--train-flights", type=int, default=5_200_000)
    ap.add_argument("--train-steps", type=int, default=1200)
    ap.add_argument("--size", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    world, rank, local = dist_env()

    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "learned":
        run_learned(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload != "flights":
        run_image(args)
        return

    import torch
    from gpis_extend_gb300 import abi, build, roofline, runtime, workloads

    build.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from gpis_extend_gb300 import replicas
    red = replicas.Reducer(dist, device="cuda")
    barrier, max_over_ranks, sum_over_ranks = red.barrier, red.max, red.sum

    desc = workloads.sphere_medium()
    n = args.flights
    prim = workloads.sphere_flights(n, desc, index_offset=replicas.flight_range(n, rank))
    ctx = runtime.Context(desc)
    rec = ctx.trace_host(prim)
    sec, _ = workloads.secondary_flights(prim, rec, desc)
    dev_p = runtime.DeviceFlights(prim)
    dev_s = runtime.DeviceFlights(sec)
    flights_per_step = prim.n + sec.n
    stream = torch.cuda.current_stream()
    # the schedule: the fast pass's persistent grid from the autotuner, on these flights
    from gpis_extend_gb300 import autotune
    schedule = [autotune.tune_fast_window(ctx, [dev_p, dev_s]), autotune.tune_march(ctx, [dev_p, dev_s])]

    # ---- device-resident throughput --------------------------------------------
    for _ in range(args.warmup):
        ctx.submit(dev_p, stream)
        ctx.submit(dev_s, stream)
    torch.cuda.synchronize()
    ctx.counters(reset=True)
    ctx.profile_read(reset=True)
    ctx.profile(True)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        ctx.submit(dev_p, stream)
        ctx.submit(dev_s, stream)
    end.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(end)
    ctx.profile(False)
    kms, klaunch = ctx.profile_read(reset=True)
    cnt = ctx.counters(reset=True)
    ms_max = max_over_ranks(ms)
    total_flights = sum_over_ranks(float(flights_per_step * args.steps))
    value = total_flights / (ms_max * 1e-3)

    # ---- end to end through the host entry point -------------------------------
    pin_p = runtime.PinnedFlights(prim)
    pin_s = runtime.PinnedFlights(sec)
    schedule.append(autotune.tune_host_chunk(ctx, [pin_p, pin_s]))
    schedule.append(autotune.tune_host_direct(ctx, [pin_p, pin_s]))
    ctx.trace_pinned(pin_p)
    ctx.trace_pinned(pin_s)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.trace_pinned(pin_p)
        ctx.trace_pinned(pin_s)
    t_e2e = time.perf_counter() - t0
    barrier()
    clocks.stop()
    e2e_value = sum_over_ranks(float(flights_per_step * args.steps)) / max_over_ranks(t_e2e)
    h2d = roofline.BYTES_IN_PER_FLIGHT * flights_per_step
    d2h = roofline.BYTES_OUT_PER_FLIGHT * flights_per_step

    # ---- roofline of the march kernel ------------------------------------------
    march_launches = max(1, klaunch[1])
    march_ms = kms[1] / march_launches
    evals_march = (cnt["steps"] - cnt["skipped_steps"] + cnt["refine_evals"] + cnt["flights"]
                   + (cnt["flights"] - cnt["hits"]))
    flops = evals_march * roofline.flops_per_eval_1d(8) / march_launches
    achieved = flops / (march_ms * 1e-3) / 1e12
    peak = sgemm_peak_tflops(torch) if rank == 0 else None
    traffic = None
    tr = load_traffic()
    if tr and tr.get("bytes_per_flight"):
        traffic = tr["bytes_per_flight"] * flights_per_step / 2.0
    # beside the flops: all 32-bit operations of the reference formulation (flops plus
    # the hash, PCG and compare work) against the SMs' 32-bit lane throughput at the
    # clock sampled during the timed region
    ops_eval = roofline.flops_per_eval_1d(8) + roofline.int_ops_per_eval_1d(8)
    ops_achieved = evals_march * ops_eval / march_launches / (march_ms * 1e-3) / 1e12
    sm_mhz = clocks.summary().get("sm_mhz") or 0.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    ops_peak = sms * roofline.LANES_PER_SM * sm_mhz * 1e6 / 1e12 if sm_mhz else None
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if peak else None, "traffic": traffic,
            "traffic_source": ((tr or {}).get("source", "") + "; DRAM bytes per flight of that capture times "
                               "the flights of one launch, not measured in this run") if traffic else None,
            "kernel": "k_march<EvalCoop1D<8>> fast pass + certified and precise resume passes",
            "march_ms_per_launch": march_ms,
            "kernel_ms_per_step": [k / max(1, args.steps) for k in kms],
            "flops_per_eval": roofline.flops_per_eval_1d(8),
            "evals_per_launch": evals_march / march_launches,
            "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, best of 5, measured in this run",
            "ops32": {"per_eval": ops_eval, "achieved": ops_achieved, "peak": ops_peak, "unit": "Tops/s",
                      "frac": (ops_achieved / ops_peak) if ops_peak else None,
                      "peak_source": f"{sms} SMs x {roofline.LANES_PER_SM} 32-bit lanes x the sampled SM clock",
                      "note": "the reference formulation's operations: it regenerates the three cells at every "
                              "evaluation; the kernels regenerate "
                              f"{cnt['cell_refills'] / max(1.0, evals_march):.3f} cells per evaluation, so this "
                              "rate overstates the work executed; the utilisation is issue_active"},
            # the passes' issue-slot utilisation from the committed ncu capture, not
            # measured here
            "issue_active_ncu": dict((tr or {}).get("issue_active") or {}, source=(tr or {}).get("source"))}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "arm": "plain", "flights_per_step_per_gpu": flights_per_step,
                   "primary": prim.n, "secondary": sec.n, "l2": "inputs 512 MiB > L2 (no flush)",
                   "parallelism": f"replicas x{world} (disjoint flight ranges)", "schedule": schedule},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        # per batch: k_prepare (the fast pass's set-up and the conditioning), the fast
        # pass, the resume pass and k_finish; two batches per step
        "gpu_launches": args.steps * 2 * 4,
        "roofline": roof,
        "counters": cnt,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_learned:
        # the learned-proposal arm on the same flights (config-1 network trained on a
        # disjoint flight set); a failure is reported, not raised
        try:
            prop, info = train_proposal(ctx, desc, workloads.sphere_flights, 1 << 20, 400, 8192, 1.5)
            learned = learned_arm(ctx, prop, [prim, sec], [dev_p, dev_s], args.steps, stream, ms)
            learned["train"] = info
            prop.close()
        except Exception as e:  # noqa: BLE001
            learned = {"error": f"{type(e).__name__}: {e}"}
        line["learned"] = learned
    if rank == 0 and world == 1 and not args.no_learned:
        # the learned arm on its own configuration: the three-octave torus-plane
        # field, 2^22 primaries and their secondaries per step, a network trained on
        # about 10^7 flights of that field
        try:
            l3 = learned_workload(args)
            lr = l3["learned"]
            line["learned_config3"] = {
                "workload": l3["config"]["workload"], "flights_per_step": l3["config"]["flights_per_step"],
                "value": lr["value"], "plain_value": lr["plain_value"], "ratio_vs_plain": lr["ratio_vs_plain"],
                "ms_per_step": lr["ms_per_step"], "plain_ms_per_step": l3["plain"]["ms_per_step"],
                "ms_per_part": lr["ms_per_part"], "ceiling_true_interval": lr["ceiling_true_interval"],
                "schedule": lr["schedule"], "inside_interval": lr["inside_interval"],
                "miss_fallback_rate": lr["miss_fallback_rate"], "identical_to_plain": lr["identical_to_plain"],
                "train": l3["config"]["train"]}
        except Exception as e:  # noqa: BLE001
            line["learned_config3"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the oracle over every flight of the step, timed as the CPU baseline; its
        # records check the GPU's records of the last timed step flight by flight
        ctx.submit(dev_p, stream)
        ctx.submit(dev_s, stream)
        torch.cuda.synchronize()
        gpu_recs = (dev_p.results(), dev_s.results())
        line["cpu_baseline"], line["parity"] = cpu_baseline(desc, prim, sec, gpu_recs)
    if rank == 0 and world == 1 and not args.no_ref_gpu:
        # the GPU baseline to beat: the reference's own traceSegments kernel
        # (RaySegmentBatch.cu, compiled unmodified) and the flight kernels on the
        # same flights over the sphere SDF baked into a 256^3 grid (the only mean
        # that kernel supports); device time per pass with CUDA events
        try:
            from oracle import ref_gpu_baseline as rgb
            if rgb.available():
                r = rgb.compare(args.flights, reps=5, grid_res=256)
                line["ref_gpu_kernel"] = {
                    "value": r["reference_flights_per_s"], "unit": UNIT,
                    "flight_kernels_value": r["flight_kernels_flights_per_s"], "ratio": r["speedup_total"],
                    "hit_agreement": {k: v["hit_agreement"] for k, v in r["flights"].items()},
                    "t_agreement": {k: v["t_agreement"] for k, v in r["flights"].items()},
                    "workload": r["workload"], "passes": r["flights"]}
            else:
                line["ref_gpu_kernel"] = {"unavailable": "reference cubin not built (needs the reference tree)"}
        except Exception as e:  # noqa: BLE001
            line["ref_gpu_kernel"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
