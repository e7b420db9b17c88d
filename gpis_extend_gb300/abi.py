"""ctypes mirror of include/gpis.h and the loader of libgpis_gb300.so.

The structures here are the data formats of the C ABI; the library functions
are bound in :func:`load_library`.  The library is built in-tree by
``gpis_extend_gb300.build`` and is required: every entry point that computes
raises :class:`GpisError` when the library or a CUDA device is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpis_gb300.so")

# status codes
GPIS_OK = 0
GPIS_EIO = 5
GPIS_ENOMEM = 12
GPIS_ENODEV = 19
GPIS_EINVAL = 22
GPIS_ERANGE = 34
GPIS_ENOTSUP = 95

FLIGHT_OK = 0
FLIGHT_INVALID_INPUT = 1
FLIGHT_STEP_LIMIT = 2
FLIGHT_PROPOSAL_MISS = 3

CTX_GLOBAL, CTX_RENEWAL_PLUS, CTX_RENEWAL, CTX_NONE = 0, 1, 2, 3
SCHEME_UNI, SCHEME_NEE, SCHEME_MIS = 0, 1, 2
MEAN_SPHERE, MEAN_HOMOGENEOUS, MEAN_GRID, MEAN_PLANE, MEAN_TORUS, MEAN_TORUS_PLANE = range(6)
LS_CONSTANT, LS_SINCOS = 0, 1
STATIC_MAX_FLIGHTS = 65536
FLAG_FIRST_SCATTER = 1
FLAG_SHADOW = 2

CONTEXT_NAMES = {"global": CTX_GLOBAL, "renewal+": CTX_RENEWAL_PLUS,
                 "renewal": CTX_RENEWAL, "none": CTX_NONE}
SCHEME_NAMES = {"uni": SCHEME_UNI, "nee": SCHEME_NEE, "mis": SCHEME_MIS}


class GpisError(RuntimeError):
    """A C-ABI call returned a non-zero status or the library is unavailable."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


class MeanGrid(ctypes.Structure):
    _fields_ = [
        ("voxels", ctypes.c_void_p),
        ("origin", ctypes.c_int32 * 3),
        ("dims", ctypes.c_int32 * 3),
        ("world_to_index", ctypes.c_float * 12),
        ("clamp_min", ctypes.c_float * 3),
        ("clamp_max", ctypes.c_float * 3),
        ("offset", ctypes.c_float),
        ("scale", ctypes.c_float),
    ]


class MediumDesc(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_float),
        ("length_scale", ctypes.c_float),
        ("aniso", ctypes.c_float * 3),
        ("kernel_scale", ctypes.c_float),
        ("ls_kind", ctypes.c_uint32),
        ("ls_params", ctypes.c_float * 4),
        ("ls_max", ctypes.c_float),
        ("multires", ctypes.c_uint32),
        ("n_octaves", ctypes.c_uint32),
        ("octave_sigma", ctypes.c_float * 4),
        ("octave_scale", ctypes.c_float * 4),
        ("octave_seed", ctypes.c_uint32 * 4),
        ("mean_kind", ctypes.c_uint32),
        ("mean_params", ctypes.c_float * 8),
        ("grid", ctypes.POINTER(MeanGrid)),
        ("step_size", ctypes.c_float),
        ("min_step", ctypes.c_uint32),
        ("seed", ctypes.c_uint32),
        ("impulse_density", ctypes.c_float),
        ("single_realization", ctypes.c_uint32),
        ("isotropic_3d_sampling", ctypes.c_uint32),
        ("one_d_sampling", ctypes.c_uint32),
        ("sampling_scheme", ctypes.c_uint32),
        ("correlation_xy", ctypes.c_uint32),
        ("correlation_context", ctypes.c_uint32),
        ("sigma_a", ctypes.c_float),
        ("sigma_s", ctypes.c_float),
        ("density", ctypes.c_float),
        ("max_steps", ctypes.c_uint32),
        ("impulse_xyz_order", ctypes.c_uint32),
        ("max_bounces", ctypes.c_int32),
        ("reserved_", ctypes.c_uint32),
    ]


class Ray(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("dir", ctypes.c_float * 3), ("near_t", ctypes.c_float),
                ("far_t", ctypes.c_float)]


class MediumState(ctypes.Structure):
    _fields_ = [("pixel_sample_segment", ctypes.c_uint32 * 4), ("scene_seed", ctypes.c_uint32),
                ("first_scatter", ctypes.c_uint32), ("bounce", ctypes.c_int32), ("last_gp_id", ctypes.c_int32),
                ("last_val", ctypes.c_float), ("last_aniso", ctypes.c_float * 3), ("info_t", ctypes.c_double),
                ("sampling_scheme", ctypes.c_uint32), ("reserved_", ctypes.c_uint32)]


class MediumSample(ctypes.Structure):
    _fields_ = [("t", ctypes.c_float), ("p", ctypes.c_float * 3), ("weight", ctypes.c_float * 3),
                ("pdf", ctypes.c_float), ("aniso", ctypes.c_float * 3), ("continued_t", ctypes.c_float),
                ("continued_weight", ctypes.c_float * 3), ("exited", ctypes.c_int32), ("gp_id", ctypes.c_int32),
                ("status", ctypes.c_int32), ("sampling_scheme", ctypes.c_uint32), ("reserved_", ctypes.c_uint32)]


# numpy views of the structures (same layout, for batches)
RAY_DTYPE = np.dtype([("pos", np.float32, 3), ("dir", np.float32, 3), ("near_t", np.float32), ("far_t", np.float32)])
STATE_DTYPE = np.dtype([("pss", np.uint32, 4), ("scene_seed", np.uint32), ("first_scatter", np.uint32),
                        ("bounce", np.int32), ("last_gp_id", np.int32), ("last_val", np.float32),
                        ("last_aniso", np.float32, 3), ("info_t", np.float64), ("sampling_scheme", np.uint32),
                        ("reserved_", np.uint32)])
SAMPLE_DTYPE = np.dtype([("t", np.float32), ("p", np.float32, 3), ("weight", np.float32, 3), ("pdf", np.float32),
                         ("aniso", np.float32, 3), ("continued_t", np.float32), ("continued_weight", np.float32, 3),
                         ("exited", np.int32), ("gp_id", np.int32), ("status", np.int32),
                         ("sampling_scheme", np.uint32), ("reserved_", np.uint32)])


class FlightSoA(ctypes.Structure):
    _fields_ = [
        ("origin_near", ctypes.c_void_p),
        ("dir_far", ctypes.c_void_p),
        ("seeds", ctypes.c_void_p),
        ("prev", ctypes.c_void_p),
        ("medium", ctypes.c_void_p),
    ]


class ResultSoA(ctypes.Structure):
    _fields_ = [("rec", ctypes.c_void_p)]


PHASE_LAMBERT, PHASE_MIRROR, PHASE_CONDUCTOR = 0, 1, 2
TUNE_MARCH_CTAS_PER_SM, TUNE_RENDER_PASS_PATHS, TUNE_HOST_CHUNK, TUNE_HOST_DIRECT = 0, 1, 2, 3
TUNE_PROPOSED_SKIP_CAP = 4
TUNE_FAST_WINDOW = 5
TUNE_PRECISE_DECISIONS = 6
PHASE_NAMES = {"lambert": PHASE_LAMBERT, "mirror": PHASE_MIRROR, "conductor": PHASE_CONDUCTOR}
PROPOSAL_KERNELS = {"tc2": 0, "tc1": 1, "mma": 2}
PROPOSAL_WAIT_DEFAULT = 1 << 22
# ConductorBsdf's default material, copper (ConductorBsdf.cpp:24-27)
CU_ETA = (0.200438, 0.924033, 1.10221)
CU_K = (3.91295, 2.45285, 2.14219)


class SceneDesc(ctypes.Structure):
    """gpis_scene_desc: camera, medium cube, quad light and phase of a render."""
    _fields_ = [
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
        ("max_bounces", ctypes.c_uint32),
        ("cam_pos", ctypes.c_float * 3), ("cam_target", ctypes.c_float * 3), ("cam_up", ctypes.c_float * 3),
        ("tan_half_fov", ctypes.c_float), ("box_half", ctypes.c_float),
        ("light_center", ctypes.c_float * 3), ("light_u", ctypes.c_float * 3), ("light_v", ctypes.c_float * 3),
        ("light_emission", ctypes.c_float * 3),
        ("phase", ctypes.c_uint32), ("albedo", ctypes.c_float * 3),
        ("scene_seed", ctypes.c_uint32), ("sampler_seed", ctypes.c_uint32), ("medium", ctypes.c_uint32),
        ("eta", ctypes.c_float * 3), ("k", ctypes.c_float * 3), ("reserved_", ctypes.c_uint32),
    ]


class RenderStats(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint64), ("distance_flights", ctypes.c_uint64),
                ("shadow_flights", ctypes.c_uint64), ("medium_events", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("ms", ctypes.c_double), ("launches", ctypes.c_uint64),
                ("nee_queries", ctypes.c_uint64), ("graphed", ctypes.c_uint32), ("passes", ctypes.c_uint32)]


def make_scene(width=64, height=64, spp=4, max_bounces=4, fov_deg=45.0, cam_pos=(0, 0, 4), cam_target=(0, 0, 0),
               cam_up=(0, 1, 0), box_half=1.5, light_center=(0, 3, 0), light_u=(1, 0, 0), light_v=(0, 0, 1),
               light_emission=(10, 10, 10), albedo=(0.8, 0.8, 0.8), scene_seed=1, sampler_seed=7, medium=0,
               phase=PHASE_LAMBERT, eta=CU_ETA, k=CU_K):
    """A SceneDesc; the default light is a 1x1 quad at y = 3 facing down.  phase is a
    PHASE_* value or its name; eta and k are the conductor's complex index (copper)."""
    import math
    sc = SceneDesc()
    sc.width, sc.height, sc.spp, sc.max_bounces = width, height, spp, max_bounces
    sc.cam_pos[:] = cam_pos
    sc.cam_target[:] = cam_target
    sc.cam_up[:] = cam_up
    sc.tan_half_fov = math.tan(math.radians(fov_deg) / 2)
    sc.box_half = box_half
    sc.light_center[:] = light_center
    sc.light_u[:] = light_u
    sc.light_v[:] = light_v
    sc.light_emission[:] = light_emission
    sc.phase = PHASE_NAMES[phase] if isinstance(phase, str) else int(phase)
    sc.albedo[:] = albedo
    sc.eta[:] = eta
    sc.k[:] = k
    sc.scene_seed, sc.sampler_seed, sc.medium = scene_seed, sampler_seed, medium
    return sc


class NeeSoA(ctypes.Structure):
    """gpis_nee_soa: the realization's flight streams plus point_t and normal (float4 each)."""
    _fields_ = [
        ("flight", FlightSoA),
        ("point_t", ctypes.c_void_p),
        ("normal", ctypes.c_void_p),
    ]


class Counters(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in
                ("flights", "steps", "refine_evals", "hits", "step_limit", "invalid",
                 "cell_refills", "skipped_steps")]


def medium_defaults():
    """Python copy of gpis_medium_desc_init (reference defaults)."""
    d = MediumDesc()
    d.sigma = 1.0
    d.length_scale = 1.0
    d.aniso[:] = (1.0, 1.0, 1.0)
    d.kernel_scale = 3.0
    d.ls_kind = LS_CONSTANT
    d.ls_params[:] = (1.0, 0.0, 0.0, 0.0)
    d.ls_max = 1.0
    d.multires = 0
    d.n_octaves = 1
    d.octave_sigma[:] = (1.0, 0.0, 0.0, 0.0)
    d.octave_scale[:] = (1.0, 1.0, 1.0, 1.0)
    d.octave_seed[:] = (0, 0, 0, 0)
    d.mean_kind = MEAN_SPHERE
    d.mean_params[:] = (0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0)
    d.grid = None
    d.step_size = 0.01
    d.min_step = 8
    d.seed = 0
    d.impulse_density = 3.0
    d.single_realization = 0
    d.isotropic_3d_sampling = 0
    d.one_d_sampling = 0
    d.sampling_scheme = SCHEME_UNI
    d.correlation_xy = 0
    d.correlation_context = CTX_RENEWAL_PLUS
    d.sigma_a = 0.0
    d.sigma_s = 0.0
    d.density = 1.0
    d.max_steps = 0
    d.impulse_xyz_order = 0
    d.max_bounces = 1024
    return d


def make_medium(**kw):
    """A MediumDesc from the defaults plus keyword overrides (arrays accepted)."""
    d = medium_defaults()
    for k, v in kw.items():
        if not hasattr(d, k):
            raise KeyError(k)
        cur = getattr(d, k)
        if isinstance(cur, ctypes.Array):
            vals = list(v)
            cur[:len(vals)] = vals
        else:
            setattr(d, k, v)
    return d


def make_mean_grid(voxels, origin=(0, 0, 0), world_to_index=None, clamp_min=None,
                   clamp_max=None, offset=0.0, scale=1.0):
    """A MeanGrid over a (z, y, x) float32 array; the array is kept alive on the struct."""
    vox = np.ascontiguousarray(voxels, dtype=np.float32)
    nz, ny, nx = vox.shape
    g = MeanGrid()
    g.voxels = vox.ctypes.data
    g.origin[:] = origin
    g.dims[:] = (nx, ny, nz)
    g.world_to_index[:] = world_to_index if world_to_index is not None else \
        (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0)
    g.clamp_min[:] = clamp_min if clamp_min is not None else (0, 0, 0)
    g.clamp_max[:] = clamp_max if clamp_max is not None else (nx - 1, ny - 1, nz - 1)
    g.offset = offset
    g.scale = scale
    g._keep = vox
    return g


def attach_grid(desc, grid):
    desc.mean_kind = MEAN_GRID
    desc.grid = ctypes.pointer(grid)
    desc._keep_grid = grid
    return desc


class FlightBatch:
    """Host-side flight streams (numpy, 16-byte records) and the result records."""

    def __init__(self, n):
        self.n = int(n)
        self.origin_near = np.zeros((self.n, 4), np.float32)
        self.dir_far = np.zeros((self.n, 4), np.float32)
        self.seeds = np.zeros((self.n, 4), np.uint32)
        self.prev = np.zeros((self.n, 4), np.float32)
        self.medium = None

    def set_jitter(self, jitter):
        self.seeds[:, 3] = np.ascontiguousarray(jitter, np.float32).view(np.uint32)

    @property
    def jitter(self):
        return self.seeds[:, 3].view(np.float32)

    def soa(self):
        s = FlightSoA()
        s.origin_near = self.origin_near.ctypes.data
        s.dir_far = self.dir_far.ctypes.data
        s.seeds = self.seeds.ctypes.data
        s.prev = self.prev.ctypes.data
        s.medium = self.medium.ctypes.data if self.medium is not None else None
        return s

    def subset(self, idx):
        b = FlightBatch(len(idx))
        b.origin_near[:] = self.origin_near[idx]
        b.dir_far[:] = self.dir_far[idx]
        b.seeds[:] = self.seeds[idx]
        b.prev[:] = self.prev[idx]
        if self.medium is not None:
            b.medium = np.ascontiguousarray(self.medium[idx])
        return b


def new_results(n):
    return np.zeros((int(n), 8), np.float32)


def result_soa(rec):
    r = ResultSoA()
    r.rec = rec.ctypes.data
    return r


def unpack_results(rec):
    """Named views of an (n, 8) result array."""
    u = rec.view(np.uint32)
    return {
        "t": rec[:, 0], "value": rec[:, 1], "grad": rec[:, 2:5], "transmittance": rec[:, 5],
        "hit": rec[:, 5] == 0.0, "steps": u[:, 6], "status": u[:, 7] & 0xFF,
        "gp_id": (u[:, 7] >> 8) & 0xFF,
    }


_LIB = None


def load_library(path=None):
    """Load libgpis_gb300.so and bind its entry points (raises GpisError if absent)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise GpisError(f"libgpis_gb300.so not built ({p}); run gpis_extend_gb300.build.build()")
    lib = ctypes.CDLL(p)
    c_int, c_u32, vp = ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p
    P = ctypes.POINTER
    sig = {
        "gpis_medium_desc_init": (None, [P(MediumDesc)]),
        "gpis_medium_desc_from_json": (c_int, [ctypes.c_char_p, P(MediumDesc)]),
        "gpis_ctx_create": (c_int, [P(MediumDesc), c_int, P(vp)]),
        "gpis_ctx_destroy": (None, [vp]),
        "gpis_flights_submit": (c_int, [vp, P(FlightSoA), P(ResultSoA), c_u32, vp]),
        "gpis_flights_trace_host": (c_int, [vp, P(FlightSoA), P(ResultSoA), c_u32]),
        "gpis_nee_submit": (c_int, [vp, P(NeeSoA), vp, c_u32, vp]),
        "gpis_nee_host": (c_int, [vp, P(NeeSoA), vp, c_u32]),
        "gpis_render": (c_int, [vp, P(SceneDesc), vp, P(RenderStats)]),
        "gpis_render_batch": (c_int, [vp, vp, c_u32, vp, P(RenderStats)]),
        "gpis_render_batch_proposed": (c_int, [vp, vp, vp, c_u32, vp, P(RenderStats)]),
        "gpis_tune_set": (c_int, [vp, c_u32, ctypes.c_uint64]),
        "gpis_tune_get": (c_int, [vp, c_u32, P(ctypes.c_uint64)]),
        "gpis_status": (c_int, [vp, P(Counters), c_int]),
        "gpis_profile_enable": (c_int, [vp, c_int]),
        "gpis_profile_read": (c_int, [vp, P(ctypes.c_double), P(ctypes.c_uint64), c_int]),
        "gpis_flight_seeds": (None, [P(MediumDesc), P(c_u32), c_u32, P(c_u32), P(c_u32)]),
        "gpis_debug_cells_1d": (c_int, [vp, vp, c_u32, c_u32, vp, vp]),
        "gpis_debug_cells_3d": (c_int, [vp, vp, c_u32, c_u32, c_u32, vp, vp]),
        "gpis_debug_field": (c_int, [vp, vp, vp, vp, vp, vp, c_u32, vp]),
        "gpis_debug_tc_gemm": (c_int, [vp, vp, c_u32, c_u32, vp]),
        "gpis_debug_exp": (c_int, [vp, vp, c_u32]),
        "gpis_proposal_set_kernel": (c_int, [vp, c_int]),
        "gpis_proposal_occupancy": (c_int, [vp, c_int]),
        "gpis_proposal_set_wait_limit": (c_int, [vp, c_u32]),
        "gpis_se_splat_1d": (c_int, [vp, vp, vp, vp, ctypes.c_size_t, ctypes.c_float, vp]),
        "gpis_flights_submit_static": (c_int, [P(MediumDesc), P(FlightSoA), P(ResultSoA), c_u32, vp]),
        "gpis_medium_sample_distance": (c_int, [vp, c_u32, vp, vp, vp, vp, c_u32]),
        "gpis_medium_transmittance": (c_int, [vp, c_u32, vp, vp, vp, vp, c_u32]),
        "gpis_proposal_n_params": (c_u32, []),
        "gpis_proposal_create": (c_int, [vp, P(vp)]),
        "gpis_proposal_destroy": (None, [vp]),
        "gpis_proposal_set_params": (c_int, [vp, vp]),
        "gpis_proposal_get_params": (c_int, [vp, vp]),
        "gpis_proposal_features": (c_int, [vp, P(FlightSoA), vp, c_u32, vp]),
        "gpis_proposal_train_step": (c_int, [vp, vp, vp, c_u32, ctypes.c_float, P(ctypes.c_float)]),
        "gpis_proposal_gradient": (c_int, [vp, vp, vp, c_u32, vp, P(ctypes.c_float)]),
        "gpis_proposal_forward": (c_int, [vp, vp, c_u32, vp]),
        "gpis_proposal_infer": (c_int, [vp, P(FlightSoA), vp, vp, c_u32, vp]),
        "gpis_flights_submit_proposed": (c_int, [vp, P(FlightSoA), vp, P(ResultSoA), c_u32, vp]),
        "gpis_last_error": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc, what="gpis call"):
    if rc != GPIS_OK:
        lib = load_library()
        msg = lib.gpis_last_error().decode(errors="replace")
        raise GpisError(f"{what} failed with status {rc}: {msg}", rc)
