"""GB300 path-guiding library: Python mirror of the C ABI (include/pathguide.h).

The compute lives in libpathguide.so (hand-written sm_103a CUDA kernels behind
a C ABI).  This module only declares the ABI for ctypes and wraps device
pointers; there is no Python or CPU fallback - if the shared library is
missing, importing the bindings raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libpathguide.so"

_P = C.c_void_p
_U32 = C.c_uint32
_U64 = C.c_uint64
_I = C.c_int


class PathGuideError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{status_string(status)}: {message}")
        self.status = status


# name -> (restype, argtypes); one entry per function declared in include/*.h
SIGNATURES = {
    "pg_default_fit_config": (None, [C.POINTER(abi.FitConfig)]),
    "pg_ctx_create": (_I, [C.POINTER(abi.FitConfig), _U32, _U64, C.POINTER(_P)]),
    "pg_ctx_destroy": (_I, [_P]),
    "pg_last_error": (C.c_char_p, [_P]),
    "pg_status_string": (C.c_char_p, [_I]),
    "pg_get_fit_config": (_I, [_P, C.POINTER(abi.FitConfig)]),
    "pg_set_fit_config": (_I, [_P, C.POINTER(abi.FitConfig)]),
    "pg_init_regions": (_I, [_P, _U32, _P]),
    "pg_get_region_states": (_I, [_P, _P, _U32, _U32, _P]),
    "pg_set_region_states": (_I, [_P, _P, _U32, _U32, _P]),
    "pg_region_states_device": (_I, [_P, C.POINTER(_P)]),
    "pg_fit_regions": (_I, [_P, _P, _P, _U32, _I, _P]),
    "pg_eval_loglik": (_I, [_P, _P, _P, _U32, _P, _P]),
    "pg_set_fit_tuning": (_I, [_P, C.POINTER(abi.FitTuning)]),
    "pg_get_fit_tuning": (_I, [_P, C.POINTER(abi.FitTuning)]),
    "pg_sync_status": (_I, [_P, _P]),
    "pg_last_launch_count": (_I, [_P, C.POINTER(_U32)]),
    "pg_autotune_fit": (_I, [_P, _P, _P, _U32, _I, C.POINTER(abi.FitTuning), _U32, C.POINTER(abi.FitTuning),
                             C.POINTER(C.c_float), _P]),
    "pg_fit_graph_create": (_I, [_P, _P, _P, _U32, _I, _P, C.POINTER(_P)]),
    "pg_fit_graph_launch": (_I, [_P, _P]),
    "pg_fit_graph_destroy": (_I, [_P]),
    "pg_fit_regions_noalloc": (_I, [C.POINTER(abi.FitConfig), _P, _P, _P, _U32, _I, _P]),
    "pg_fit_regions_host": (_I, [_P, _P, _P, _U32, _I, _P]),
    "pg_default_split_merge_config": (None, [C.POINTER(abi.SplitMergeConfig)]),
    "pg_set_split_merge": (_I, [_P, C.POINTER(abi.SplitMergeConfig)]),
    "pg_split_merge": (_I, [_P, _P, _P, _P, _U32, _P]),
    "pg_get_region_extra": (_I, [_P, _P, _U32]),
    "pg_set_region_extra": (_I, [_P, _P, _U32]),
    "pg_default_region_split_config": (None, [C.POINTER(abi.RegionSplitConfig)]),
    "pg_set_region_split": (_I, [_P, C.POINTER(abi.RegionSplitConfig)]),
    "pg_split_regions": (_I, [_P, C.POINTER(_U32), _P]),
    "pg_get_region_tree": (_I, [_P, _P, _U32, C.POINTER(_U32)]),
    "pg_mlp_default_config": (None, [C.POINTER(abi.MlpConfig)]),
    "pg_mlp_create": (_I, [C.POINTER(abi.MlpConfig), C.POINTER(_P)]),
    "pg_mlp_destroy": (_I, [_P]),
    "pg_mlp_get_params": (_I, [_P, _P]),
    "pg_mlp_set_params": (_I, [_P, _P]),
    "pg_mlp_loss_grad": (_I, [_P, _P, _U32, _P, C.POINTER(C.c_float), _P]),
    "pg_mlp_train": (_I, [_P, _P, _U64, C.POINTER(C.c_float), _P]),
    "pg_mlp_infer": (_I, [_P, _P, _U32, _P, _P]),
    "pg_mlp_set_path": (_I, [_P, C.c_int]),
    "pg_mlp_write_guide": (_I, [_P, _P, _P]),
    "pg_mlp_judge_guide": (_I, [_P, _P, _P, _U64, _U32, C.POINTER(_U32), _P]),
    "pg_guide_nll": (_I, [_P, _P, _U64, C.POINTER(C.c_double), _P]),
    "pg_set_regions": (_I, [_P, _U32, _P, _P]),
    "pg_region_count": (_I, [_P, C.POINTER(_U32)]),
    "pg_get_region_aabbs": (_I, [_P, _P, _U32]),
    "pg_region_aabbs_device": (_I, [_P, C.POINTER(_P)]),
    "pg_sort_samples": (_I, [_P, _P, _U64, _U32, _P, _P, _P]),
    "pg_prefit_parallax": (_I, [_P, _P, _P, _U32, _U64, _P, _P, _P]),
    "pg_update_distances": (_I, [_P, _P, _P, _P, _U32, _P]),
    "pg_pack_vmm_theta": (_I, [_P, _U32, _P, _P]),
    "pg_update": (_I, [_P, _P, _U64, _P, _P]),
    "pg_scene_load": (_I, [C.c_char_p, _U32, _U32, C.POINTER(_P)]),
    "pg_scene_create_cornell": (_I, [C.POINTER(abi.CornellParams), C.POINTER(_P)]),
    "pg_scene_create_plates": (_I, [C.POINTER(abi.PlatesParams), C.POINTER(_P)]),
    "pg_scene_destroy": (_I, [_P]),
    "pg_scene_set_envmap": (_I, [_P, _P, _U32, _U32]),
    "pg_scene_get_envmap": (_I, [_P, _P, C.POINTER(_U32), C.POINTER(_U32)]),
    "pg_exr_read": (_I, [C.c_char_p, _P, _U64, C.POINTER(_U32), C.POINTER(_U32)]),
    "pg_exr_write": (_I, [C.c_char_p, _P, _U32, _U32]),
    "pg_scene_get_info": (_I, [_P, C.POINTER(abi.SceneInfo)]),
    "pg_scene_export": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "pg_scene_export_mesh": (_I, [_P, _P, _P, C.POINTER(_U32)]),
    "pg_scene_texture_sizes": (_I, [_P, C.POINTER(_U32), C.POINTER(_U64)]),
    "pg_scene_export_textures": (_I, [_P, _P, _P, _P]),
    "pg_png_read": (_I, [C.c_char_p, _P, _U64, C.POINTER(_U32), C.POINTER(_U32)]),
    "pg_scene_set_camera": (_I, [_P, C.POINTER(abi.Camera)]),
    "pg_trace_closest": (_I, [_P, _P, _U32, _P, _P]),
    "pg_trace_any": (_I, [_P, _P, _U32, _P, _P]),
    "pg_trace_closest_counted": (_I, [_P, _P, _U32, _P, _P, _P, _P]),
    "pg_probe_shading": (_I, [_P, _U32, _P, _U32, _P, _U32, _P, _P]),
    "pg_probe_records": (_I, [_P, _P, _U32, _P, _P, _P, _P]),
    "pg_render": (_I, [_P, C.POINTER(abi.RenderParams), _P, _P, _P, C.POINTER(abi.RenderStats), _P]),
    "pg_default_irradiance_cache_config": (None, [C.POINTER(abi.IrradianceCacheConfig)]),
    "pg_scene_set_irradiance_cache": (_I, [_P, C.POINTER(abi.IrradianceCacheConfig)]),
    "pg_scene_get_irradiance_cache": (_I, [_P, _P, _U32, C.POINTER(_U32)]),
    "pg_scene_set_irradiance_cache_entries": (_I, [_P, _P, _U32]),
    "pg_ic_query": (_I, [_P, _P, _P, _U32, _P, _P, _P]),
    "pg_scene_set_adrrs": (_I, [_P, C.POINTER(abi.AdrrsConfig)]),
    "pg_ic_compute": (_I, [_P, C.POINTER(abi.RenderParams), _P, _P, _U32, _P, _P]),
}

_LIB = None


def library() -> C.CDLL:
    """Loads libpathguide.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            if hasattr(lib, name):
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
        _LIB = lib
    return _LIB


def status_string(status: int) -> str:
    try:
        return library().pg_status_string(status).decode()
    except Exception:  # library not loadable: still report the number
        return f"status {status}"


def _stream_handle(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


def _dptr(x) -> int:
    """Device address of a torch tensor (or an int address)."""
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


class FitContext:
    """A pg_ctx: per-region mixture states and the batched EM fit on one GPU."""

    def __init__(self, cfg: abi.FitConfig | None = None, max_regions: int = 4096, max_samples: int = 0):
        self.lib = library()
        self.cfg = cfg if cfg is not None else abi.default_fit_config()
        h = C.c_void_p()
        st = self.lib.pg_ctx_create(C.byref(self.cfg), max_regions, max_samples, C.byref(h))
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(None).decode())
        self.h = h
        self.max_regions = max_regions

    def _check(self, st: int):
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_config(self, cfg: abi.FitConfig):
        self._check(self.lib.pg_set_fit_config(self.h, C.byref(cfg)))
        self.cfg = cfg

    def set_tuning(self, threads_per_cta=0, smem_samples=0, ctas_per_sm=0, cluster_size=0,
                   components_per_thread=0, unroll=0, large_threshold=0, stream_stages=0):
        t = abi.FitTuning(threads_per_cta, smem_samples, ctas_per_sm, cluster_size, components_per_thread, unroll,
                          large_threshold, stream_stages)
        self._check(self.lib.pg_set_fit_tuning(self.h, C.byref(t)))

    def init_regions(self, n_regions: int, stream=None):
        self._check(self.lib.pg_init_regions(self.h, n_regions, _stream_handle(stream)))

    def fit(self, dirw, offsets, n_regions: int, mode: int = abi.PG_FIT_INIT, stream=None):
        """Fits regions [0, n_regions).  dirw: device float4 per sample; offsets: device uint32 (n+1)."""
        self._check(self.lib.pg_fit_regions(self.h, _dptr(dirw), _dptr(offsets), n_regions, mode,
                                            _stream_handle(stream)))

    def fit_host(self, dirw, offsets, n_regions: int, mode: int = abi.PG_FIT_INIT, stream=None):
        """pg_fit_regions_host: the fit from HOST samples (a pinned torch tensor
        or a numpy array), copied on the context's copy stream.  The arrays
        must stay alive until the stream has run the fit."""
        def hptr(x):
            if isinstance(x, np.ndarray):
                return x.ctypes.data
            return _dptr(x)
        self._check(self.lib.pg_fit_regions_host(self.h, hptr(dirw), hptr(offsets), n_regions, mode,
                                                 _stream_handle(stream)))

    def eval_loglik(self, dirw, offsets, n_regions: int, ll_out, stream=None):
        self._check(self.lib.pg_eval_loglik(self.h, _dptr(dirw), _dptr(offsets), n_regions, _dptr(ll_out),
                                            _stream_handle(stream)))

    def sync(self, stream=None):
        self._check(self.lib.pg_sync_status(self.h, _stream_handle(stream)))

    def states(self, n: int, first: int = 0, stream=None) -> np.ndarray:
        out = np.zeros(n, dtype=abi.STATE_DTYPE)
        self._check(self.lib.pg_get_region_states(self.h, out.ctypes.data, first, n, _stream_handle(stream)))
        return out

    def set_states(self, states: np.ndarray, first: int = 0, stream=None):
        s = np.ascontiguousarray(states, dtype=abi.STATE_DTYPE)
        self._check(self.lib.pg_set_region_states(self.h, s.ctypes.data, first, s.shape[0],
                                                  _stream_handle(stream)))

    def states_device_ptr(self) -> int:
        p = C.c_void_p()
        self._check(self.lib.pg_region_states_device(self.h, C.byref(p)))
        return int(p.value or 0)

    # ---- regions, bucketing, parallax, distances, VMM_Theta ----
    def set_regions(self, split_count: int, scene_aabb, stream=None):
        a = np.ascontiguousarray(scene_aabb, dtype=np.float32)
        self._check(self.lib.pg_set_regions(self.h, split_count, a.ctypes.data, _stream_handle(stream)))

    def region_count(self) -> int:
        n = C.c_uint32()
        self._check(self.lib.pg_region_count(self.h, C.byref(n)))
        return int(n.value)

    def region_aabbs(self) -> np.ndarray:
        n = self.region_count()
        out = np.zeros((n, 6), dtype=np.float32)
        self._check(self.lib.pg_get_region_aabbs(self.h, out.ctypes.data, n))
        return out

    def sort_samples(self, records, n_records: int, n_regions: int, sorted_out, offsets_out, stream=None):
        self._check(self.lib.pg_sort_samples(self.h, _dptr(records), n_records, n_regions,
                                             _dptr(sorted_out) if sorted_out is not None else None,
                                             _dptr(offsets_out), _stream_handle(stream)))

    def prefit_parallax(self, sorted_records, offsets, n_regions: int, n_valid: int, dirw_out, dist_out, stream=None):
        self._check(self.lib.pg_prefit_parallax(self.h, _dptr(sorted_records), _dptr(offsets), n_regions, n_valid,
                                                _dptr(dirw_out), _dptr(dist_out), _stream_handle(stream)))

    def update_distances(self, dirw, dist, offsets, n_regions: int, stream=None):
        self._check(self.lib.pg_update_distances(self.h, _dptr(dirw), _dptr(dist), _dptr(offsets), n_regions,
                                                 _stream_handle(stream)))

    def pack_vmm_theta(self, n_regions: int, out, stream=None):
        self._check(self.lib.pg_pack_vmm_theta(self.h, n_regions, _dptr(out), _stream_handle(stream)))

    def update(self, records, n_records: int, vmm_out=None, stream=None):
        """PathGuiding::update: one device-resident guiding pass over the tracer's records."""
        self._check(self.lib.pg_update(self.h, _dptr(records), n_records,
                                       _dptr(vmm_out) if vmm_out is not None else None, _stream_handle(stream)))

    def guide_nll(self, records_dev, n: int, stream=None) -> float:
        """Weighted NLL of records under the context's current guide (the KL judge)."""
        v = C.c_double()
        self._check(self.lib.pg_guide_nll(self.h, _dptr(records_dev), n, C.byref(v), _stream_handle(stream)))
        return float(v.value)

    def autotune(self, dirw, offsets, n_regions: int, mode: int = abi.PG_FIT_INIT, candidates=None, stream=None):
        """pg_autotune_fit: times the candidate launch shapes (the built-in grid
        when None) on these samples, keeps the fastest; states are preserved."""
        best = abi.FitTuning()
        ms = C.c_float()
        if candidates:
            arr = (abi.FitTuning * len(candidates))(*candidates)
            cand, n = arr, len(candidates)
        else:
            cand, n = None, 0
        self._check(self.lib.pg_autotune_fit(self.h, _dptr(dirw), _dptr(offsets), n_regions, mode, cand, n,
                                             C.byref(best), C.byref(ms), _stream_handle(stream)))
        return best, float(ms.value)

    def capture_fit(self, dirw, offsets, n_regions: int, mode: int, stream) -> "FitGraph":
        """pg_fit_graph_create: the fit captured as a CUDA graph on `stream`."""
        g = C.c_void_p()
        self._check(self.lib.pg_fit_graph_create(self.h, _dptr(dirw), _dptr(offsets), n_regions, mode,
                                                 _stream_handle(stream), C.byref(g)))
        return FitGraph(self.lib, g)

    def last_launch_count(self) -> int:
        n = C.c_uint32()
        self._check(self.lib.pg_last_launch_count(self.h, C.byref(n)))
        return int(n.value)

    # ---- split and merge (PathGuiding::postFit with splitAndMerge) ----
    def set_split_merge(self, cfg: abi.SplitMergeConfig | None = None):
        """Turns the post-fit split/merge on with `cfg` (the reference's
        defaults when None); a config with enabled=0 turns it off."""
        c = cfg if cfg is not None else abi.default_split_merge_config()
        self._check(self.lib.pg_set_split_merge(self.h, C.byref(c)))

    def split_merge(self, dirw, pdf, offsets, n_regions: int, stream=None):
        """One post-fit split/merge pass of regions [0, n_regions) on the
        samples of the last fit and their sampling pdfs."""
        self._check(self.lib.pg_split_merge(self.h, _dptr(dirw), _dptr(pdf), _dptr(offsets), n_regions,
                                            _stream_handle(stream)))

    def extras(self, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=abi.EXTRA_DTYPE)
        self._check(self.lib.pg_get_region_extra(self.h, out.ctypes.data, n))
        return out

    # ---- region splitting (PathGuiding::update's split check) ----
    def set_region_split(self, cfg: abi.RegionSplitConfig | None = None):
        """Turns region splitting on with `cfg` (the reference's threshold when
        None); pg_update then splits regions after each fit."""
        c = cfg if cfg is not None else abi.default_region_split_config()
        self._check(self.lib.pg_set_region_split(self.h, C.byref(c)))

    def split_regions(self, stream=None) -> int:
        """One split check over the current regions; returns the region count."""
        n = C.c_uint32()
        self._check(self.lib.pg_split_regions(self.h, C.byref(n), _stream_handle(stream)))
        return int(n.value)

    def region_tree(self) -> np.ndarray:
        """The region tree (node v >= 0: children v, v + 1; v < 0: leaf of region -v - 1)."""
        n = C.c_uint32()
        self._check(self.lib.pg_get_region_tree(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        self._check(self.lib.pg_get_region_tree(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def set_extras(self, extras: np.ndarray):
        e = np.ascontiguousarray(extras)
        if e.dtype != abi.EXTRA_DTYPE:
            if e.dtype.itemsize != abi.EXTRA_DTYPE.itemsize:
                raise ValueError("extras must be pg_region_extra records (400 bytes each)")
            e = e.view(abi.EXTRA_DTYPE)
        self._check(self.lib.pg_set_region_extra(self.h, e.ctypes.data, e.shape[0]))


class FitGraph:
    """A captured fit (pg_fit_graph_*): launch() replays it on a stream."""

    def __init__(self, lib, handle):
        self.lib, self.h = lib, handle

    def launch(self, stream=None):
        st = self.lib.pg_fit_graph_launch(self.h, _stream_handle(stream))
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_fit_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """The learned guiding surrogate (pg_mlp_*): position -> 16-component vMF
    mixture, trained on guiding records with BF16 tensor-core kernels."""

    def __init__(self, scene_aabb, batch: int = 65536, lr: float = 1e-3, seed: int = 1):
        self.lib = library()
        cfg = abi.MlpConfig()
        self.lib.pg_mlp_default_config(C.byref(cfg))
        cfg.batch, cfg.lr, cfg.seed = batch, lr, seed
        for i, v in enumerate(scene_aabb):
            cfg.scene_aabb[i] = float(v)
        self.cfg = cfg
        h = C.c_void_p()
        st = self.lib.pg_mlp_create(C.byref(cfg), C.byref(h))
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(None).decode())
        self.h = h

    def _check(self, st):
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(abi.MLP_PARAMS, dtype=np.float32)
        self._check(self.lib.pg_mlp_get_params(self.h, out.ctypes.data))
        return out

    def set_path(self, path: int):
        """Training-step implementation: abi.PG_MLP_PATH_TCGEN05 (default) or
        abi.PG_MLP_PATH_WARP_MMA."""
        self._check(self.lib.pg_mlp_set_path(self.h, int(path)))

    def set_params(self, theta):
        a = np.ascontiguousarray(theta, dtype=np.float32)
        assert a.size == abi.MLP_PARAMS
        self._check(self.lib.pg_mlp_set_params(self.h, a.ctypes.data))

    def loss_grad(self, records_dev, n: int, grad_dev=None, stream=None) -> float:
        loss = C.c_float()
        self._check(self.lib.pg_mlp_loss_grad(self.h, _dptr(records_dev), n,
                                              _dptr(grad_dev) if grad_dev is not None else None, C.byref(loss),
                                              _stream_handle(stream)))
        return float(loss.value)

    def train(self, records_dev, n: int, stream=None, want_loss: bool = True):
        loss = C.c_float()
        self._check(self.lib.pg_mlp_train(self.h, _dptr(records_dev), n, C.byref(loss) if want_loss else None,
                                          _stream_handle(stream)))
        return float(loss.value) if want_loss else None

    def infer(self, positions_dev, n: int, mixtures_dev, stream=None):
        self._check(self.lib.pg_mlp_infer(self.h, _dptr(positions_dev), n, _dptr(mixtures_dev),
                                          _stream_handle(stream)))

    def write_guide(self, ctx: FitContext, stream=None):
        self._check(self.lib.pg_mlp_write_guide(self.h, ctx.h, _stream_handle(stream)))

    def judge_guide(self, ctx: FitContext, records_dev, n: int, min_records: int = 32, stream=None) -> int:
        """Per region, keeps the context's fitted mixture or takes the
        network's, whichever has the lower weighted NLL on the records."""
        k = C.c_uint32()
        self._check(self.lib.pg_mlp_judge_guide(self.h, ctx.h, _dptr(records_dev), n, min_records, C.byref(k),
                                                _stream_handle(stream)))
        return int(k.value)


NOALLOC_MAX_REGIONS = 65536


def fit_regions_noalloc(cfg: abi.FitConfig, states_dev, dirw, offsets, n_regions: int,
                        mode: int = abi.PG_FIT_INIT, stream=None) -> int:
    """pg_fit_regions_noalloc: the batched fit without a context and without any
    device allocation, for callers that may not allocate (renderers with their
    own memory arena, plugin hosts given only their own buffers).  states_dev is
    the caller's device array of n_regions pg_region_state records, updated in
    place; device-side failures are flagged in the states (PG_STATE_*).
    Returns the status."""
    return library().pg_fit_regions_noalloc(C.byref(cfg), _dptr(states_dev), _dptr(dirw), _dptr(offsets),
                                            n_regions, mode, _stream_handle(stream))


def probe_shading(mats: np.ndarray, vmms: np.ndarray, probes: np.ndarray) -> np.ndarray:
    """pg_probe_shading on the current CUDA device: the renderer's shading
    functions on explicit inputs (probes: abi.PROBE_DTYPE records; mats:
    abi.MATERIAL_DTYPE; vmms: abi.VMM_THETA_DTYPE).  Returns (n, 8) float32."""
    import torch
    dev = lambda a: torch.from_numpy(np.frombuffer(np.ascontiguousarray(a).tobytes(), dtype=np.uint8).copy()).cuda()
    n = len(probes)
    dm, dv, dp = dev(mats), dev(vmms), dev(probes)
    out = torch.zeros((max(n, 1), 8), dtype=torch.float32, device="cuda")
    st = library().pg_probe_shading(_dptr(dm), len(mats), _dptr(dv), len(vmms), _dptr(dp), n, _dptr(out), None)
    if st != abi.PG_OK:
        raise PathGuideError(st, "pg_probe_shading")
    torch.cuda.synchronize()
    return out[:n].cpu().numpy()


def probe_records(events: np.ndarray, path_offsets: np.ndarray):
    """pg_probe_records on the current CUDA device: the renderer's sample
    recording replayed over paths of abi.RECORD_EVENT_DTYPE events.  Returns
    (weights (P, 16), flags (P, 16), counts (P,))."""
    import torch
    ev = np.ascontiguousarray(events, dtype=abi.RECORD_EVENT_DTYPE)
    offs = np.ascontiguousarray(path_offsets, dtype=np.uint32)
    P = len(offs) - 1
    d_ev = torch.from_numpy(np.frombuffer(ev.tobytes(), dtype=np.uint8).copy()).cuda()
    d_off = torch.from_numpy(offs.view(np.int32).copy()).cuda()
    w = torch.zeros((max(P, 1), 16), dtype=torch.float32, device="cuda")
    f = torch.zeros((max(P, 1), 16), dtype=torch.int32, device="cuda")
    c = torch.zeros(max(P, 1), dtype=torch.int32, device="cuda")
    st = library().pg_probe_records(_dptr(d_ev), _dptr(d_off), P, _dptr(w), _dptr(f), _dptr(c), None)
    if st != abi.PG_OK:
        raise PathGuideError(st, "pg_probe_records")
    torch.cuda.synchronize()
    return w[:P].cpu().numpy(), f[:P].cpu().numpy().view(np.uint32), c[:P].cpu().numpy().view(np.uint32)


def read_png(path) -> np.ndarray:
    """A PNG image as (height, width, 4) uint8 RGBA (pg_png_read)."""
    lib = library()
    w, h = C.c_uint32(), C.c_uint32()
    st = lib.pg_png_read(str(path).encode(), None, 0, C.byref(w), C.byref(h))
    if st != abi.PG_OK:
        raise PathGuideError(st, lib.pg_last_error(None).decode())
    out = np.zeros((h.value, w.value, 4), dtype=np.uint8)
    st = lib.pg_png_read(str(path).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h))
    if st != abi.PG_OK:
        raise PathGuideError(st, lib.pg_last_error(None).decode())
    return out


def read_exr(path) -> np.ndarray:
    """An OpenEXR image as (height, width, 3) float32 (pg_exr_read)."""
    lib = library()
    w, h = C.c_uint32(), C.c_uint32()
    st = lib.pg_exr_read(str(path).encode(), None, 0, C.byref(w), C.byref(h))
    if st != abi.PG_OK:
        raise PathGuideError(st, lib.pg_last_error(None).decode())
    out = np.zeros((h.value, w.value, 3), dtype=np.float32)
    st = lib.pg_exr_read(str(path).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h))
    if st != abi.PG_OK:
        raise PathGuideError(st, lib.pg_last_error(None).decode())
    return out


def write_exr(path, rgb) -> None:
    """Writes (height, width, 3) floats as an uncompressed FLOAT OpenEXR file (pg_exr_write)."""
    lib = library()
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    st = lib.pg_exr_write(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0])
    if st != abi.PG_OK:
        raise PathGuideError(st, lib.pg_last_error(None).decode())


class Scene:
    """A pg_scene: geometry, materials, lights and camera with its BVH (SceneLoader)."""

    def __init__(self, handle):
        self.lib = library()
        self.h = handle

    @classmethod
    def _make(cls, fn, *args):
        lib = library()
        h = C.c_void_p()
        st = getattr(lib, fn)(*args, C.byref(h))
        if st != abi.PG_OK:
            raise PathGuideError(st, lib.pg_last_error(None).decode())
        return cls(h)

    @classmethod
    def cornell(cls, width=1280, height=720, ico_level=5, light_radiance=15.0, ior=1.5):
        p = abi.CornellParams(width, height, ico_level, light_radiance, ior)
        return cls._make("pg_scene_create_cornell", C.byref(p))

    @classmethod
    def plates(cls, width=1920, height=1080, occluder_grid=707, seed=4):
        p = abi.PlatesParams(width, height, occluder_grid, seed)
        return cls._make("pg_scene_create_plates", C.byref(p))

    @classmethod
    def load(cls, path, width, height):
        return cls._make("pg_scene_load", str(path).encode(), width, height)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.PG_OK:
            raise PathGuideError(st, self.lib.pg_last_error(None).decode())

    def info(self) -> abi.SceneInfo:
        i = abi.SceneInfo()
        self._check(self.lib.pg_scene_get_info(self.h, C.byref(i)))
        return i

    def set_camera(self, cam: abi.Camera):
        self._check(self.lib.pg_scene_set_camera(self.h, C.byref(cam)))

    def export(self) -> dict:
        """Host copies of the built scene (BVH, triangles, materials, spheres, mesh)."""
        i = self.info()
        nodes = np.zeros(i.n_nodes, dtype=abi.NODE_DTYPE)
        tv = np.zeros((i.n_triangles, 12), dtype=np.float32)
        order = np.zeros(i.n_triangles, dtype=np.uint32)
        tmat = np.zeros(i.n_triangles, dtype=np.uint32)
        mats = np.zeros(i.n_materials, dtype=abi.MATERIAL_DTYPE)
        sph = np.zeros(i.n_spheres, dtype=abi.SPHERE_DTYPE)
        self._check(self.lib.pg_scene_export(self.h, nodes.ctypes.data, tv.ctypes.data, order.ctypes.data,
                                             tmat.ctypes.data, mats.ctypes.data, sph.ctypes.data))
        nv = C.c_uint32()
        self._check(self.lib.pg_scene_export_mesh(self.h, None, None, C.byref(nv)))
        pos = np.zeros((nv.value, 3), dtype=np.float32)
        idx = np.zeros((i.n_triangles, 3), dtype=np.uint32)
        self._check(self.lib.pg_scene_export_mesh(self.h, pos.ctypes.data, idx.ctypes.data, C.byref(nv)))
        out = {"nodes": nodes, "tri_verts": tv, "tri_order": order, "tri_mat": tmat, "mats": mats,
               "spheres": sph, "pos": pos, "idx": idx, "info": i}
        nt, ntx = C.c_uint32(), C.c_uint64()
        self._check(self.lib.pg_scene_texture_sizes(self.h, C.byref(nt), C.byref(ntx)))
        out["tri_uv"] = np.zeros((i.n_triangles, 6), dtype=np.float32)
        out["tex_info"] = np.zeros((nt.value, 4), dtype=np.uint32)
        out["tex_data"] = np.zeros((ntx.value, 4), dtype=np.uint8)
        self._check(self.lib.pg_scene_export_textures(self.h, out["tri_uv"].ctypes.data, out["tex_info"].ctypes.data,
                                                      out["tex_data"].ctypes.data))
        env = self.envmap()
        if env is not None:
            out["env"] = env
        return out

    def set_envmap(self, rgb):
        """The environment map: a lat-long RGB image (height, width, 3), row 0
        looking up; None removes it (pg_scene_set_envmap)."""
        if rgb is None:
            self._check(self.lib.pg_scene_set_envmap(self.h, None, 0, 0))
            return
        a = np.ascontiguousarray(rgb, dtype=np.float32)
        if a.ndim != 3 or a.shape[2] != 3:
            raise ValueError("environment map must be (height, width, 3)")
        self._check(self.lib.pg_scene_set_envmap(self.h, a.ctypes.data, a.shape[1], a.shape[0]))

    def envmap(self):
        w, h = C.c_uint32(), C.c_uint32()
        self._check(self.lib.pg_scene_get_envmap(self.h, None, C.byref(w), C.byref(h)))
        if w.value == 0:
            return None
        out = np.zeros((h.value, w.value, 3), dtype=np.float32)
        self._check(self.lib.pg_scene_get_envmap(self.h, out.ctypes.data, C.byref(w), C.byref(h)))
        return out

    def trace_closest(self, rays_dev, n, hits_dev, stream=None):
        self._check(self.lib.pg_trace_closest(self.h, _dptr(rays_dev), n, _dptr(hits_dev), _stream_handle(stream)))

    def trace_closest_counted(self, rays_dev, n, hits_dev, nodes_dev, tris_dev, stream=None):
        self._check(self.lib.pg_trace_closest_counted(self.h, _dptr(rays_dev), n, _dptr(hits_dev), _dptr(nodes_dev),
                                                      _dptr(tris_dev), _stream_handle(stream)))

    def trace_any(self, rays_dev, n, occ_dev, stream=None):
        self._check(self.lib.pg_trace_any(self.h, _dptr(rays_dev), n, _dptr(occ_dev), _stream_handle(stream)))

    def render(self, params: abi.RenderParams, image_dev, guide: "FitContext | None" = None, records_dev=None,
               stream=None, stats: bool = True) -> "abi.RenderStats | None":
        """Adds params.spp samples per pixel of radiance into image_dev (float32, H*W*3).
        With stats, waits for the render and returns its counters; without,
        returns at once (stream-ordered)."""
        st = abi.RenderStats() if stats else None
        self._check(self.lib.pg_render(self.h, C.byref(params), guide.h if guide is not None else None,
                                       _dptr(image_dev), _dptr(records_dev) if records_dev is not None else None,
                                       C.byref(st) if st is not None else None, _stream_handle(stream)))
        return st

    # --- irradiance cache
    def set_irradiance_cache(self, cfg: "abi.IrradianceCacheConfig | None" = None, **fields):
        """Sets (and empties) the scene's irradiance cache: the defaults of
        pg_default_irradiance_cache_config, or cfg, with `fields` overriding."""
        if cfg is None:
            cfg = abi.IrradianceCacheConfig()
            self.lib.pg_default_irradiance_cache_config(C.byref(cfg))
        for k, v in fields.items():
            setattr(cfg, k, v)
        self._check(self.lib.pg_scene_set_irradiance_cache(self.h, C.byref(cfg)))
        return cfg

    def set_adrrs(self, estimate_dev, s: float = 5.0, split: bool = True):
        """The pixel estimate (device float32, H*W*3 mean radiance, kept alive
        by the caller) and window of PG_RENDER_ADRRS renders."""
        self._adrrs_estimate = estimate_dev
        cfg = abi.AdrrsConfig(_dptr(estimate_dev), s, int(split))
        self._check(self.lib.pg_scene_set_adrrs(self.h, C.byref(cfg)))

    def irradiance_cache(self) -> np.ndarray:
        """The cache's entries (IC_ENTRY_DTYPE)."""
        n = C.c_uint32()
        self._check(self.lib.pg_scene_get_irradiance_cache(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=abi.IC_ENTRY_DTYPE)
        if n.value:
            self._check(self.lib.pg_scene_get_irradiance_cache(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def set_irradiance_cache_entries(self, entries: np.ndarray):
        e = np.ascontiguousarray(entries, dtype=abi.IC_ENTRY_DTYPE)
        self._check(self.lib.pg_scene_set_irradiance_cache_entries(self.h, e.ctypes.data if len(e) else None,
                                                                   len(e)))

    def ic_query(self, positions, normals):
        """Cache queries at (n, 3) points with normals: (rgb (n, 3), found (n,))."""
        import torch
        pos = torch.as_tensor(np.ascontiguousarray(positions, dtype=np.float32)).cuda()
        nrm = torch.as_tensor(np.ascontiguousarray(normals, dtype=np.float32)).cuda()
        n = pos.shape[0]
        rgb = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
        found = torch.zeros(n, dtype=torch.int32, device="cuda")
        self._check(self.lib.pg_ic_query(self.h, _dptr(pos), _dptr(nrm), n, _dptr(rgb), _dptr(found),
                                         _stream_handle(None)))
        torch.cuda.synchronize()
        return rgb.cpu().numpy(), found.cpu().numpy().astype(np.uint32)

    def ic_compute(self, params: abi.RenderParams, requests: np.ndarray,
                   guide: "FitContext | None" = None) -> np.ndarray:
        """The entries calculateCacheData makes at the requests (IC_REQUEST_DTYPE)."""
        import torch
        req = np.ascontiguousarray(requests, dtype=abi.IC_REQUEST_DTYPE)
        n = len(req)
        d_req = torch.from_numpy(req.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(n * abi.IC_ENTRY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        self._check(self.lib.pg_ic_compute(self.h, C.byref(params), guide.h if guide is not None else None,
                                           _dptr(d_req), n, _dptr(d_out), _stream_handle(None)))
        return d_out.cpu().numpy().view(abi.IC_ENTRY_DTYPE)

    def get_scene_size(self):
        """SceneLoader::getSceneSize (src/SceneLoader.h:118): the scene box (min xyz, max xyz)."""
        return list(self.info().aabb)
