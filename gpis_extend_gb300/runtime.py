"""Context objects over the C ABI (gpis_ctx_*), with torch tensors as device memory.

``Context.trace_host`` is the blocking host-array entry (gpis_flights_trace_host);
``Context.submit`` enqueues a batch whose streams already live in HBM
(gpis_flights_submit).  Both raise :class:`abi.GpisError` on any failure; there is
no CPU fallback.
"""
import ctypes

import numpy as np

from . import abi


def _torch():
    import torch
    return torch


class DeviceFlights:
    """Flight streams and result records resident on the GPU (torch tensors)."""

    def __init__(self, batch, device="cuda"):
        torch = _torch()
        self.n = batch.n
        self.origin_near = torch.from_numpy(batch.origin_near).to(device)
        self.dir_far = torch.from_numpy(batch.dir_far).to(device)
        self.seeds = torch.from_numpy(batch.seeds.view(np.int32)).to(device)
        self.prev = torch.from_numpy(batch.prev).to(device)
        self.medium = None
        if batch.medium is not None:
            self.medium = torch.from_numpy(batch.medium.view(np.int32)).to(device)
        self.rec = torch.zeros((self.n, 8), dtype=torch.float32, device=device)

    def soa(self):
        s = abi.FlightSoA()
        s.origin_near = self.origin_near.data_ptr()
        s.dir_far = self.dir_far.data_ptr()
        s.seeds = self.seeds.data_ptr()
        s.prev = self.prev.data_ptr()
        s.medium = self.medium.data_ptr() if self.medium is not None else None
        return s

    def result_soa(self):
        r = abi.ResultSoA()
        r.rec = self.rec.data_ptr()
        return r

    def results(self):
        return self.rec.cpu().numpy()


class PinnedFlights:
    """Flight streams and result records in pinned host memory (torch tensors)."""

    def __init__(self, batch):
        torch = _torch()
        self.n = batch.n

        def pin(a):
            t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                            pin_memory=True)
            t.numpy()[...] = a.view(np.float32 if a.dtype == np.float32 else np.int32)
            return t

        self.origin_near = pin(batch.origin_near)
        self.dir_far = pin(batch.dir_far)
        self.seeds = pin(batch.seeds)
        self.prev = pin(batch.prev)
        self.medium = pin(batch.medium) if batch.medium is not None else None
        self.rec = torch.zeros((self.n, 8), dtype=torch.float32, pin_memory=True)

    soa = DeviceFlights.soa
    result_soa = DeviceFlights.result_soa

    def results(self):
        return self.rec.numpy()


class Context:
    """A gpis_ctx over one or more media on the current CUDA device."""

    def __init__(self, media):
        if isinstance(media, abi.MediumDesc):
            media = [media]
        self.lib = abi.load_library()
        self._media = list(media)
        arr = (abi.MediumDesc * len(media))(*media)
        h = ctypes.c_void_p()
        abi.check(self.lib.gpis_ctx_create(arr, len(media), ctypes.byref(h)), "gpis_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.gpis_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def trace_host(self, batch, rec=None):
        if rec is None:
            rec = abi.new_results(batch.n)
        soa = batch.soa()
        res = abi.result_soa(rec)
        abi.check(self.lib.gpis_flights_trace_host(self.h, ctypes.byref(soa), ctypes.byref(res), batch.n),
                  "gpis_flights_trace_host")
        return rec

    def nee(self, batch, points, t_segment, normals):
        """1D specular NEE (gpis_nee_host) on the realizations of the flights in batch:
        returns (n, 4) float32 {pdf, gradient}."""
        n = batch.n
        pt = np.zeros((n, 4), np.float32)
        pt[:, :3] = points
        pt[:, 3] = t_segment
        nr = np.zeros((n, 4), np.float32)
        nr[:, :3] = normals
        out = np.zeros((n, 4), np.float32)
        q = abi.NeeSoA(batch.soa(), pt.ctypes.data, nr.ctypes.data)
        abi.check(self.lib.gpis_nee_host(self.h, ctypes.byref(q), out.ctypes.data, n), "gpis_nee_host")
        return out

    def render(self, scene):
        """gpis_render: returns (image (h, w, 3) float32, stats dict)."""
        img = np.zeros((scene.height, scene.width, 3), np.float32)
        st = abi.RenderStats()
        abi.check(self.lib.gpis_render(self.h, ctypes.byref(scene), img.ctypes.data, ctypes.byref(st)),
                  "gpis_render")
        return img, {k: getattr(st, k) for k, _ in abi.RenderStats._fields_}

    def tune(self, key, value=None):
        """Set (value given) and return a schedule knob (abi.TUNE_*)."""
        if value is not None:
            abi.check(self.lib.gpis_tune_set(self.h, key, int(value)), "gpis_tune_set")
        v = ctypes.c_uint64()
        abi.check(self.lib.gpis_tune_get(self.h, key, ctypes.byref(v)), "gpis_tune_get")
        return v.value

    def render_batch(self, scenes, proposal=None):
        """gpis_render_batch (gpis_render_batch_proposed with a Proposal): returns (list of
        images (h, w, 3) float32, stats dict)."""
        imgs = [np.zeros((sc.height, sc.width, 3), np.float32) for sc in scenes]
        arr = (abi.SceneDesc * len(scenes))(*scenes)
        ptrs = (ctypes.c_void_p * len(scenes))(*[im.ctypes.data for im in imgs])
        st = abi.RenderStats()
        if proposal is None:
            abi.check(self.lib.gpis_render_batch(self.h, arr, len(scenes), ptrs, ctypes.byref(st)),
                      "gpis_render_batch")
        else:
            abi.check(self.lib.gpis_render_batch_proposed(self.h, proposal.h, arr, len(scenes), ptrs,
                                                          ctypes.byref(st)), "gpis_render_batch_proposed")
        return imgs, {k: getattr(st, k) for k, _ in abi.RenderStats._fields_}

    def trace_pinned(self, pinned):
        """gpis_flights_trace_host on PinnedFlights (host -> device -> host, synchronous)."""
        soa = pinned.soa()
        res = pinned.result_soa()
        abi.check(self.lib.gpis_flights_trace_host(self.h, ctypes.byref(soa), ctypes.byref(res), pinned.n),
                  "gpis_flights_trace_host")

    def submit(self, dev, stream=None):
        """Enqueue a DeviceFlights batch on a CUDA stream (torch stream or None)."""
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream()
        soa = dev.soa()
        res = dev.result_soa()
        abi.check(self.lib.gpis_flights_submit(self.h, ctypes.byref(soa), ctypes.byref(res), dev.n,
                                               ctypes.c_void_p(s.cuda_stream)), "gpis_flights_submit")

    def profile(self, on=True):
        abi.check(self.lib.gpis_profile_enable(self.h, int(on)), "gpis_profile_enable")

    def profile_read(self, reset=False):
        """Accumulated (ms, launches) of the prepare, march and finish kernels."""
        ms = (ctypes.c_double * 3)()
        ln = (ctypes.c_uint64 * 3)()
        abi.check(self.lib.gpis_profile_read(self.h, ms, ln, int(reset)), "gpis_profile_read")
        return list(ms), list(ln)

    def sample_distance(self, medium, rays, states, jitter):
        """Batched Medium::sampleDistance (gpis_medium_sample_distance); states update in place."""
        samples = np.zeros(len(rays), abi.SAMPLE_DTYPE)
        jit = np.ascontiguousarray(jitter, np.float32)
        abi.check(self.lib.gpis_medium_sample_distance(self.h, medium, rays.ctypes.data, states.ctypes.data,
                                                       jit.ctypes.data, samples.ctypes.data, len(rays)),
                  "gpis_medium_sample_distance")
        return samples

    def transmittance(self, medium, rays, states, jitter):
        """Batched Medium::transmittance (gpis_medium_transmittance)."""
        tr = np.zeros(len(rays), np.float32)
        jit = np.ascontiguousarray(jitter, np.float32)
        abi.check(self.lib.gpis_medium_transmittance(self.h, medium, rays.ctypes.data, states.ctypes.data,
                                                     jit.ctypes.data, tr.ctypes.data, len(rays)),
                  "gpis_medium_transmittance")
        return tr

    def counters(self, reset=False):
        c = abi.Counters()
        abi.check(self.lib.gpis_status(self.h, ctypes.byref(c), int(reset)), "gpis_status")
        return {k: int(getattr(c, k)) for k, _ in abi.Counters._fields_}

    def debug_field(self, origins, points, dirs, seeds, prev):
        """Field/noise at points on the device; returns (n, 8) float32."""
        torch = _torch()
        n = len(points)

        def dev4(a, dt=np.float32):
            x = np.zeros((n, 4), dt)
            a = np.asarray(a)
            x[:, :a.shape[1]] = a
            if dt == np.uint32:
                x = x.view(np.int32)
            return torch.from_numpy(x).cuda()

        o, p, d = dev4(origins), dev4(points), dev4(dirs)
        s, pv = dev4(seeds, np.uint32), dev4(prev)
        out = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
        abi.check(self.lib.gpis_debug_field(self.h, o.data_ptr(), p.data_ptr(), d.data_ptr(), s.data_ptr(),
                                            pv.data_ptr(), n, out.data_ptr()), "gpis_debug_field")
        return out.cpu().numpy()


def debug_exp(x):
    """gpis_debug_exp: the precise evaluator's exponential at the float32 arguments x."""
    torch = _torch()
    xs = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    ys = torch.empty_like(xs)
    abi.check(abi.load_library().gpis_debug_exp(xs.data_ptr(), ys.data_ptr(), xs.numel()), "gpis_debug_exp")
    return ys.cpu().numpy()


def debug_cells_1d(cells, seeds, impulses):
    torch = _torch()
    lib = abi.load_library()
    n = len(cells)
    c = torch.from_numpy(np.asarray(cells, np.uint32).view(np.int32)).cuda()
    s = torch.from_numpy(np.asarray(seeds, np.uint32).view(np.int32)).cuda()
    pos = torch.zeros(n * impulses, dtype=torch.float32, device="cuda")
    w = torch.zeros(n * impulses, dtype=torch.float32, device="cuda")
    abi.check(lib.gpis_debug_cells_1d(c.data_ptr(), s.data_ptr(), n, impulses, pos.data_ptr(), w.data_ptr()),
              "gpis_debug_cells_1d")
    return pos.cpu().numpy().reshape(n, impulses), w.cpu().numpy().reshape(n, impulses)


def debug_cells_3d(cells, seeds, impulses, order=0):
    torch = _torch()
    lib = abi.load_library()
    n = len(cells)
    c = torch.from_numpy(np.ascontiguousarray(cells, np.int32)).cuda()
    s = torch.from_numpy(np.asarray(seeds, np.uint32).view(np.int32)).cuda()
    pos = torch.zeros(n * impulses * 3, dtype=torch.float32, device="cuda")
    w = torch.zeros(n * impulses, dtype=torch.float32, device="cuda")
    abi.check(lib.gpis_debug_cells_3d(c.data_ptr(), s.data_ptr(), n, impulses, order, pos.data_ptr(),
                                      w.data_ptr()), "gpis_debug_cells_3d")
    return pos.cpu().numpy().reshape(n, impulses, 3), w.cpu().numpy().reshape(n, impulses)


def debug_tc_gemm(a_bf16, b_bf16):
    """D = A B^T on the tcgen05 path: A (128, K) and B (N, K) as uint16 BF16 bit
    patterns; returns D (128, N) float32."""
    lib = abi.load_library()
    a = np.ascontiguousarray(a_bf16, np.uint16)
    b = np.ascontiguousarray(b_bf16, np.uint16)
    assert a.shape[0] == 128 and a.shape[1] == b.shape[1]
    n, k = b.shape
    d = np.zeros((128, n), np.float32)
    abi.check(lib.gpis_debug_tc_gemm(a.ctypes.data, b.ctypes.data, n, k, d.ctypes.data), "gpis_debug_tc_gemm")
    return d


def se_splat_1d(q, c, scale):
    torch = _torch()
    lib = abi.load_library()
    qd = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(c, np.float32)).cuda()
    v = torch.zeros_like(qd)
    dv = torch.zeros_like(qd)
    abi.check(lib.gpis_se_splat_1d(qd.data_ptr(), cd.data_ptr(), v.data_ptr(), dv.data_ptr(), len(q),
                                   float(scale), None), "gpis_se_splat_1d")
    torch.cuda.synchronize()
    return v.cpu().numpy(), dv.cpu().numpy()


class Proposal:
    """The learned crossing proposal (gpis_proposal_*) on the current CUDA device.

    Device batches are torch tensors: features (n, 24) float32, targets (n, 2)
    float32 (u*, hit), intervals (n, 4) float32 (t_a, t_b, miss probability, m)."""

    def __init__(self, params=None):
        self.lib = abi.load_library()
        self.n_params = int(self.lib.gpis_proposal_n_params())
        h = ctypes.c_void_p()
        ptr = None
        if params is not None:
            params = np.ascontiguousarray(params, np.float32)
            assert params.size == self.n_params
            ptr = params.ctypes.data
        abi.check(self.lib.gpis_proposal_create(ptr, ctypes.byref(h)), "gpis_proposal_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.gpis_proposal_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        abi.check(self.lib.gpis_proposal_set_params(self.h, params.ctypes.data), "gpis_proposal_set_params")

    def get_params(self):
        out = np.zeros(self.n_params, np.float32)
        abi.check(self.lib.gpis_proposal_get_params(self.h, out.ctypes.data), "gpis_proposal_get_params")
        return out

    def train_step(self, feats, targets, lr, want_loss=True):
        loss = ctypes.c_float()
        abi.check(self.lib.gpis_proposal_train_step(self.h, feats.data_ptr(), targets.data_ptr(), feats.shape[0],
                                                    float(lr), ctypes.byref(loss) if want_loss else None),
                  "gpis_proposal_train_step")
        return loss.value if want_loss else None

    def gradient(self, feats, targets):
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        abi.check(self.lib.gpis_proposal_gradient(self.h, feats.data_ptr(), targets.data_ptr(), feats.shape[0],
                                                  g.ctypes.data, ctypes.byref(loss)), "gpis_proposal_gradient")
        return g, loss.value

    def forward(self, feats):
        torch = _torch()
        out = torch.zeros((feats.shape[0], 32), dtype=torch.float32, device=feats.device)
        abi.check(self.lib.gpis_proposal_forward(self.h, feats.data_ptr(), feats.shape[0], out.data_ptr()),
                  "gpis_proposal_forward")
        return out

    def set_kernel(self, kernel):
        """The fused inference kernel: "tc2" (tcgen05, two 128-flight tiles per block),
        "tc1" (one tile per block) or "mma" (warp-level mma.sync)."""
        abi.check(self.lib.gpis_proposal_set_kernel(self.h, abi.PROPOSAL_KERNELS[kernel]), "gpis_proposal_set_kernel")

    def set_wait_limit(self, polls=None):
        """Polls of the tensor-memory kernel's completion wait per MMA round (None:
        the default); 0 makes the wait time out, reported by the next infer."""
        polls = abi.PROPOSAL_WAIT_DEFAULT if polls is None else int(polls)
        abi.check(self.lib.gpis_proposal_set_wait_limit(self.h, polls), "gpis_proposal_set_wait_limit")

    def occupancy(self, kernel):
        """Resident blocks per SM of a fused inference kernel."""
        n = int(self.lib.gpis_proposal_occupancy(self.h, abi.PROPOSAL_KERNELS[kernel]))
        abi.check(min(n, 0), "gpis_proposal_occupancy")
        return n

    def infer(self, dev, feats, stream=None, out=None):
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream()
        if out is None:
            out = torch.zeros((dev.n, 4), dtype=torch.float32, device=feats.device)
        soa = dev.soa()
        abi.check(self.lib.gpis_proposal_infer(self.h, ctypes.byref(soa), feats.data_ptr(), out.data_ptr(), dev.n,
                                               ctypes.c_void_p(s.cuda_stream)), "gpis_proposal_infer")
        return out


def proposal_features(ctx, dev, stream=None, out=None):
    """gpis_proposal_features of a DeviceFlights batch: (n, 24) float32 on the device."""
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    if out is None:
        out = torch.zeros((dev.n, 24), dtype=torch.float32, device="cuda")
    soa = dev.soa()
    abi.check(ctx.lib.gpis_proposal_features(ctx.h, ctypes.byref(soa), out.data_ptr(), dev.n,
                                             ctypes.c_void_p(s.cuda_stream)), "gpis_proposal_features")
    return out


def submit_proposed(ctx, dev, intervals, stream=None):
    """gpis_flights_submit_proposed: the flights of dev with proposals (results in dev.rec)."""
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    soa = dev.soa()
    res = dev.result_soa()
    abi.check(ctx.lib.gpis_flights_submit_proposed(ctx.h, ctypes.byref(soa), intervals.data_ptr(), ctypes.byref(res),
                                                   dev.n, ctypes.c_void_p(s.cuda_stream)),
              "gpis_flights_submit_proposed")
