"""numpy / ctypes mirrors of the C structures declared in include/pathguide.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

MAX_COMPONENTS = 16
INVALID_REGION = 0xFFFFFFFF

PG_OK, PG_ERR_ARG, PG_ERR_CUDA, PG_ERR_TIMEOUT, PG_ERR_NUMERIC, PG_ERR_NOMEM, PG_ERR_IO, \
    PG_ERR_PARSE, PG_ERR_STATE = range(9)
PG_FIT_INIT, PG_FIT_CONTINUE, PG_FIT_UPDATE = 0, 1, 2

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
                ("large_threshold", C.c_uint32)]


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
    return C.c_void_p(a.ctypes.data)
