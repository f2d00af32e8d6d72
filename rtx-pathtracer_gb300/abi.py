"""numpy / ctypes mirrors of the C structures declared in include/pathguide.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

MAX_COMPONENTS = 16
INVALID_REGION = 0xFFFFFFFF

PG_OK, PG_ERR_ARG, PG_ERR_CUDA, PG_ERR_TIMEOUT, PG_ERR_NUMERIC, PG_ERR_NOMEM, PG_ERR_IO, \
    PG_ERR_PARSE, PG_ERR_STATE = range(9)
PG_FIT_INIT, PG_FIT_CONTINUE, PG_FIT_UPDATE = 0, 1, 2
PG_STATE_FITTED, PG_STATE_NONFINITE, PG_STATE_FIT_FAILED = 1, 2, 4

STATE_DTYPE = np.dtype([
    ("weight", "<f4", (16,)), ("mu_x", "<f4", (16,)), ("mu_y", "<f4", (16,)),
    ("mu_z", "<f4", (16,)), ("kappa", "<f4", (16,)), ("r", "<f4", (16,)),
    ("norm", "<f4", (16,)), ("e_min2k", "<f4", (16,)), ("distance", "<f4", (16,)),
    ("dist_sum_w", "<f4", (16,)), ("parallax_mean", "<f4", (3,)),
    ("last_parallax_mean", "<f4", (3,)), ("k", "<u4"), ("sample_weight", "<f4"),
    ("num_samples", "<f4"), ("num_em_iterations", "<u4"), ("total_num_samples", "<u8"),
    ("ll_last", "<f4"), ("iters_last", "<u4"), ("flags", "<u4"), ("reserved", "<u4"),
])
assert STATE_DTYPE.itemsize == 704

VMF_THETA_DTYPE = np.dtype([
    ("mu", "<f4", (3,)), ("k", "<f4"), ("norm", "<f4"), ("e_min2k", "<f4"),
    ("distance", "<f4"), ("target", "<f4", (3,)),
])
VMM_THETA_DTYPE = np.dtype([
    ("thetas", VMF_THETA_DTYPE, (16,)), ("pi", "<f4", (16,)), ("mean_position", "<f4", (3,)),
    ("used_distributions", "<i4"),
])
assert VMM_THETA_DTYPE.itemsize == 720


class FitConfig(C.Structure):
    _fields_ = [
        ("min_itr", C.c_uint32), ("max_itr", C.c_uint32), ("rel_ll_threshold", C.c_float),
        ("num_initial_components", C.c_uint32), ("init_kappa", C.c_float),
        ("max_kappa", C.c_float), ("v_prior", C.c_float), ("r_prior", C.c_float),
        ("r_prior_weight", C.c_float), ("use_parallax", C.c_uint32),
    ]


class FitTuning(C.Structure):
    _fields_ = [("threads_per_cta", C.c_uint32), ("smem_samples", C.c_uint32),
                ("ctas_per_sm", C.c_uint32), ("cluster_size", C.c_uint32),
                ("components_per_thread", C.c_uint32), ("unroll", C.c_uint32),
                ("large_threshold", C.c_uint32), ("stream_stages", C.c_uint32)]


def default_fit_config(**kw) -> FitConfig:
    """The reference's fit properties: VMMFactoryProperties defaults
    (external/lightpmm/include/pmm/VMMFactory.h:45-61) with the overrides of
    PathGuiding::configureVMMFactory (src/PathGuiding.cpp:33-40)."""
    cfg = FitConfig(min_itr=1, max_itr=100, rel_ll_threshold=0.005, num_initial_components=8,
                    init_kappa=5.0, max_kappa=50000.0, v_prior=0.01, r_prior=0.0,
                    r_prior_weight=1.0, use_parallax=1)
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def forced_iterations(n: int, **kw) -> FitConfig:
    """Exactly n EM iterations, log-likelihood tracked every iteration
    (minItr 0, threshold -inf) - the fixed-work setting used for timing."""
    return default_fit_config(min_itr=0, max_itr=n, rel_ll_threshold=float("-inf"), **kw)


def ptr(a: np.ndarray) -> C.c_void_p:
    """Address of an array's data; the pointer holds a reference to the
    array, so a temporary (a converted copy) outlives the call it is passed to."""
    return a.ctypes.data_as(C.c_void_p)

# ---- tracer -------------------------------------------------------------
PG_MAT_DIFFUSE, PG_MAT_SPECULAR, PG_MAT_DIELECTRIC, PG_MAT_LIGHT, PG_MAT_GGX = 0, 1, 2, 3, 6
PG_MAT_PHONG, PG_MAT_CONDUCTOR, PG_MAT_BECKMANN = 4, 5, 7
NO_HIT = 0xFFFFFFFF
SPHERE_BIT = 0x80000000

MATERIAL_DTYPE = np.dtype([("type", "<i4"), ("albedo", "<f4", (3,)), ("emission", "<f4", (3,)),
                           ("roughness", "<f4"), ("ior", "<f4"), ("specular", "<f4", (3,)), ("exponent", "<f4"),
                           ("eta", "<f4"), ("k", "<f4"), ("texture", "<i4")])
SPHERE_DTYPE = np.dtype([("center", "<f4", (3,)), ("radius", "<f4"), ("material", "<u4"), ("reserved", "<u4", (3,))])
RAY_DTYPE = np.dtype([("org", "<f4", (3,)), ("tmin", "<f4"), ("dir", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])
NODE_DTYPE = np.dtype([("lo", "<f4", (3, 4)), ("hi", "<f4", (3, 4)), ("child", "<i4", (4,)), ("count", "<i4", (4,))])
assert MATERIAL_DTYPE.itemsize == 64 and SPHERE_DTYPE.itemsize == 32 and RAY_DTYPE.itemsize == 32
assert HIT_DTYPE.itemsize == 16 and NODE_DTYPE.itemsize == 128

# shading-function probes (pg_probe_shading)
PG_PROBE_FRESNEL, PG_PROBE_FRESNEL_CONDUCTOR, PG_PROBE_BSDF_EVAL, PG_PROBE_BSDF_SAMPLE, PG_PROBE_VMM_PDF, \
    PG_PROBE_VMM_SAMPLE, PG_PROBE_CONTINUE, PG_PROBE_TO_WORLD, PG_PROBE_WEIGHT_WINDOW, PG_PROBE_APPROX_DIFFUSE = range(10)
PROBE_FRONT, PROBE_PARALLAX, PROBE_GUIDED, PROBE_REGION, PROBE_GUIDE_ALL = 1, 2, 4, 8, 16
PROBE_DTYPE = np.dtype([("op", "<i4"), ("material", "<u4"), ("vmm", "<u4"), ("flags", "<u4"),
                        ("n", "<f4", (3,)), ("wi", "<f4", (3,)), ("wo", "<f4", (3,)), ("x", "<f4", (3,)),
                        ("u", "<f4", (5,)), ("a", "<f4"), ("b", "<f4"), ("c", "<f4")])
assert PROBE_DTYPE.itemsize == 96
RECORD_EVENT_DTYPE = np.dtype([("kind", "<i4"), ("pdf", "<f4"), ("tc", "<f4", (3,)), ("region", "<u4"),
                               ("light", "<f4", (3,))])
assert RECORD_EVENT_DTYPE.itemsize == 36


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("vfov_deg", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class CornellParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("ico_level", C.c_int32),
                ("light_radiance", C.c_float), ("ior", C.c_float)]


class PlatesParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("occluder_grid", C.c_uint32), ("seed", C.c_uint32)]


EXTRA_DTYPE = np.dtype([("chi2_div", "<f4", (16,)), ("chi2_n", "<f4", (16,)), ("cov", "<f4", (16, 3)),
                        ("cov_w", "<f4", (16,)), ("samples_since_merge", "<f4"), ("stat_passes", "<u4"),
                        ("em_iterations", "<u4"), ("reserved", "<u4")])
assert EXTRA_DTYPE.itemsize == 400


class SplitMergeConfig(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("min_samples_for_merging", C.c_uint32),
                ("min_samples_for_splitting", C.c_uint32), ("min_samples_for_post_split_fitting", C.c_uint32),
                ("split_min_divergence", C.c_float), ("merge_max_divergence", C.c_float),
                ("cluster_threshold", C.c_uint32), ("cluster_size", C.c_uint32)]


class RegionSplitConfig(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("samples_for_region_split", C.c_float)]


def default_region_split_config(**kw) -> RegionSplitConfig:
    """The reference's threshold (src/PathGuiding.h:122), enabled."""
    c = RegionSplitConfig(1, 10000.0)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def default_split_merge_config(**kw) -> SplitMergeConfig:
    """The reference's knobs (src/PathGuiding.h:124-129), enabled."""
    c = SplitMergeConfig(1, 8192, 4096, 4096, 0.5, 0.025, 0, 0)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class MlpConfig(C.Structure):
    _fields_ = [("batch", C.c_uint32), ("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("eps", C.c_float), ("seed", C.c_uint32), ("scene_aabb", C.c_float * 6)]


MLP_PARAMS = 20752
MLP_COMPONENTS = 16


class SceneInfo(C.Structure):
    _fields_ = [("n_triangles", C.c_uint32), ("n_spheres", C.c_uint32), ("n_materials", C.c_uint32),
                ("n_nodes", C.c_uint32), ("n_lights", C.c_uint32), ("aabb", C.c_float * 6), ("camera", Camera)]


class RenderParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint32), ("use_nee", C.c_uint32),
                ("use_mis", C.c_uint32), ("use_guiding", C.c_uint32), ("guiding_prob", C.c_float),
                ("record_samples", C.c_uint32), ("flags", C.c_uint32), ("reserved", C.c_uint32 * 3)]


PG_RENDER_COUNT_WORK = 1
PG_RENDER_TIME_STAGES = 2
PG_RENDER_GUIDE_ALMOST_DISCRETE = 4
PG_RENDER_IRRADIANCE_CACHE = 8
PG_RENDER_IC_FROZEN = 16
PG_RENDER_ADRRS = 32
STAGES = ("camera", "extend", "shade", "shadow", "advance", "commit")


class RenderStats(C.Structure):
    _fields_ = [("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("samples_recorded", C.c_uint64),
                ("paths", C.c_uint64), ("extension_node_visits", C.c_uint64),
                ("extension_triangle_tests", C.c_uint64), ("shadow_node_visits", C.c_uint64),
                ("shadow_triangle_tests", C.c_uint64), ("stage_ms", C.c_float * 6),
                ("stage_launches", C.c_uint32 * 6)]


class AdrrsConfig(C.Structure):
    _fields_ = [("estimate", C.c_void_p), ("s", C.c_float), ("split", C.c_uint32), ("reserved", C.c_uint32 * 4)]


class IrradianceCacheConfig(C.Structure):
    _fields_ = [("capacity", C.c_uint32), ("a", C.c_float), ("min_radius", C.c_float), ("create_prob", C.c_float),
                ("update_prob", C.c_float), ("use_gradients", C.c_uint32), ("gradients_max_length", C.c_float),
                ("visibility_check", C.c_uint32), ("use_on_glossy", C.c_uint32), ("num_nee", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


# pg_ic_entry (72 bytes) and pg_ic_request (40 bytes)
IC_ENTRY_DTYPE = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("normal", "<f4", 3), ("harmonic_r", "<f4"),
                           ("color", "<f4", 3), ("num_updates", "<u4"), ("rot_grad", "<f4", 3),
                           ("trans_grad", "<f4", 3)])
assert IC_ENTRY_DTYPE.itemsize == 72
IC_REQUEST_DTYPE = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("pixel", "<u4"), ("bounce", "<u4"),
                             ("pass", "<u4"), ("reserved", "<u4")])
assert IC_REQUEST_DTYPE.itemsize == 40
IC_UPDATE_BOUNCE = 255


def render_params(spp=1, max_depth=8, seed=1, use_nee=1, use_mis=1, use_guiding=0, guiding_prob=0.5,
                  record_samples=0, flags=0) -> RenderParams:
    return RenderParams(spp, max_depth, seed, use_nee, use_mis, use_guiding, guiding_prob, record_samples, flags)

# surrogate training-step implementations (pg_mlp_set_path)
PG_MLP_PATH_TCGEN05 = 0
PG_MLP_PATH_WARP_MMA = 1
