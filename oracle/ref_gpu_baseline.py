"""The reference's own GPU kernel as a baseline (TEST INFRASTRUCTURE ONLY).

traceSegments of src/gpu/cuda/RaySegmentBatch.cu is compiled, unmodified and
device code only, to oracle/_ref/ray_segment_batch.cubin by `make -C oracle ref`
(which needs the reference tree); oracle/ref_gpu_runner.cpp launches it through
the CUDA driver API.  The kernel covers the 1D SE Renewal+ UNI subset with a
dense trilinear mean grid (RaySegmentBatch.cu:73-95), so both paths run on the
sphere SDF baked into a grid.

    python -m oracle.ref_gpu_baseline [--flights N] [--reps K] [--grid G]

prints one JSON line: flights/s of the reference kernel and of the flight
kernels on the same primary and secondary flights (device-resident, CUDA
events, mean over K launches after one warm-up pass), plus their agreement.
"""
import argparse
import ctypes
import json
import os
import subprocess

import numpy as np

from gpis_extend_gb300 import abi, workloads

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ray_segment_batch.cubin")
RUNNER = os.path.join(HERE, "_build", "libref_gpu_runner.so")

REF_INPUT = np.dtype([("origin", "<f4", 3), ("direction", "<f4", 3), ("near", "<f4"), ("far", "<f4"),
                      ("jitter", "<f4"), ("noise_seed", "<u4"), ("normal_seed", "<u4"),
                      ("first_scatter", "<u4"), ("prev_value", "<f4"), ("prev_gradient", "<f4", 3)])
REF_OUTPUT = np.dtype([("t", "<f4"), ("value", "<f4"), ("gradient", "<f4", 3), ("hit", "<u4"),
                       ("steps", "<u4"), ("status", "<u4")])
assert REF_INPUT.itemsize == 64 and REF_OUTPUT.itemsize == 32

_lib = None


def available():
    return os.path.exists(CUBIN)


def load():
    """Build the runner (g++, driver API) and load the reference cubin on device 0."""
    global _lib
    if _lib is not None:
        return _lib
    if not available():
        raise FileNotFoundError(f"{CUBIN} is absent (make -C oracle ref builds it from the reference tree)")
    subprocess.check_call(["make", "-s", "-C", HERE, "runner"])
    L = ctypes.CDLL(RUNNER)
    L.refgpu_init.restype = ctypes.c_int
    L.refgpu_init.argtypes = [ctypes.c_char_p]
    L.refgpu_run.restype = ctypes.c_int
    vp = ctypes.c_void_p
    L.refgpu_run.argtypes = [vp, vp, ctypes.c_uint64, vp, vp, vp, vp, vp, vp, ctypes.c_float, ctypes.c_float,
                             vp, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double)]
    rc = L.refgpu_init(CUBIN.encode())
    if rc:
        raise RuntimeError(f"loading the reference kernel failed: {rc}")
    _lib = L
    return L


def sphere_grid(res=256, half=1.5):
    """The unit-sphere SDF on a res^3 grid over [-half, half]^3 (voxel centres at the
    grid nodes), with the world-to-index map and clamps of a TabulatedMean."""
    x = np.linspace(-half, half, res)
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")
    vox = (np.sqrt(xx * xx + yy * yy + zz * zz) - 1.0).astype(np.float32)
    s = (res - 1) / (2.0 * half)
    w2i = (s, 0, 0, half * s, 0, s, 0, half * s, 0, 0, s, half * s)
    return abi.make_mean_grid(vox, world_to_index=w2i)


def grid_medium(grid, **kw):
    d = workloads.sphere_medium(**kw)
    return abi.attach_grid(d, grid)


def to_aos(batch):
    a = np.zeros(batch.n, REF_INPUT)
    a["origin"] = batch.origin_near[:, :3]
    a["direction"] = batch.dir_far[:, :3]
    a["near"] = batch.origin_near[:, 3]
    a["far"] = batch.dir_far[:, 3]
    a["jitter"] = batch.jitter
    a["noise_seed"] = batch.seeds[:, 0]
    a["normal_seed"] = batch.seeds[:, 1]
    a["first_scatter"] = (batch.seeds[:, 2] & abi.FLAG_FIRST_SCATTER) != 0
    a["prev_value"] = batch.prev[:, 0]
    a["prev_gradient"] = batch.prev[:, 1:]
    return a


def run(batch, grid, desc, reps=1):
    """Trace batch with the reference kernel; returns (outputs, ms per launch, ms host-to-host)."""
    L = load()
    inp = to_aos(batch)
    out = np.zeros(batch.n, REF_OUTPUT)
    vox = grid._keep
    dims = np.array(grid.dims[:], np.int32)
    org = np.array(grid.origin[:], np.int32)
    w2i = np.array(grid.world_to_index[:], np.float32)
    cmin = np.array(grid.clamp_min[:], np.float32)
    cmax = np.array(grid.clamp_max[:], np.float32)
    pf = np.array([desc.length_scale, desc.sigma, desc.kernel_scale, desc.impulse_density, desc.step_size],
                  np.float32)
    pu = np.array([desc.min_step, desc.max_steps or 16384], np.uint32)
    msk = ctypes.c_double(0.0)
    mse = ctypes.c_double(0.0)
    rc = L.refgpu_run(inp.ctypes.data, out.ctypes.data, batch.n, vox.ctypes.data, dims.ctypes.data,
                      org.ctypes.data, w2i.ctypes.data, cmin.ctypes.data, cmax.ctypes.data,
                      float(grid.offset), float(grid.scale), pf.ctypes.data, pu.ctypes.data, int(reps),
                      ctypes.byref(msk), ctypes.byref(mse))
    if rc:
        raise RuntimeError(f"reference kernel failed: {rc}")
    return out, msk.value, mse.value


def agreement(ref_out, rec):
    """Hit agreement and the fraction of common hits with |dt| <= 1.5e-4."""
    r = abi.unpack_results(rec)
    ok = (ref_out["status"] == 0) & (r["status"] == abi.FLIGHT_OK)
    hit_ref = ref_out["hit"] == 1
    agree = hit_ref[ok] == r["hit"][ok]
    both = ok & hit_ref & r["hit"]
    dt = np.abs(ref_out["t"][both] - r["t"][both])
    return float(agree.mean()), float(np.mean(dt <= 1.5e-4)) if both.any() else 1.0, int(ok.sum())


def compare(n_flights=1 << 22, reps=5, grid_res=256):
    """Both kernels on the same baked-grid flights (primary, then the conditioned
    secondaries at the flight kernels' hits): per pass the device time per launch
    (CUDA events, mean over reps after a warm-up), flights/s and agreement."""
    import torch
    from gpis_extend_gb300 import runtime

    grid = sphere_grid(grid_res)
    desc = grid_medium(grid)
    prim = workloads.sphere_flights(n_flights, desc)
    res = {"workload": f"sphere SDF baked to a {grid_res}^3 grid, sigma 0.05, l 0.1, N 8, 1D Renewal+ UNI, "
                       f"{n_flights} primary flights + their conditioned secondaries",
           "flights": {}}
    with runtime.Context(desc) as ctx:
        rec = ctx.trace_host(prim)
        sec, _ = workloads.secondary_flights(prim, rec, desc)
        stream = torch.cuda.current_stream()
        for name, batch in (("primary", prim), ("secondary", sec)):
            ref_out, ref_ms, ref_e2e = run(batch, grid, desc, reps=reps)
            dev = runtime.DeviceFlights(batch)
            ctx.submit(dev, stream)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                ctx.submit(dev, stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ours_ms = e0.elapsed_time(e1) / reps
            ours_rec = ctx.trace_host(batch)
            hit_agree, t_agree, n_ok = agreement(ref_out, ours_rec)
            res["flights"][name] = {
                "n": batch.n, "reference_kernel_ms": ref_ms, "reference_host_to_host_ms": ref_e2e,
                "flight_kernels_ms": ours_ms,
                "reference_flights_per_s": batch.n / (ref_ms * 1e-3),
                "flight_kernels_flights_per_s": batch.n / (ours_ms * 1e-3),
                "speedup": ref_ms / ours_ms, "hit_agreement": hit_agree, "t_agreement": t_agree,
                "compared": n_ok}
    tot_ref = sum(v["reference_kernel_ms"] for v in res["flights"].values())
    tot_ours = sum(v["flight_kernels_ms"] for v in res["flights"].values())
    n_all = sum(v["n"] for v in res["flights"].values())
    res["reference_flights_per_s"] = n_all / (tot_ref * 1e-3)
    res["flight_kernels_flights_per_s"] = n_all / (tot_ours * 1e-3)
    res["speedup_total"] = tot_ref / tot_ours
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--flights", type=int, default=1 << 22)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--grid", type=int, default=256)
    args = ap.parse_args()
    print(json.dumps(compare(args.flights, args.reps, args.grid)))


if __name__ == "__main__":
    main()
