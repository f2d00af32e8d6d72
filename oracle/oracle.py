"""ctypes bindings of the oracle libraries (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs import this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


def _load_abi():
    """The package's own abi module, so ctypes structures are shared with it."""
    import sys
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import __graft_entry__ as entry
    return entry.load_package().abi


abi = _load_abi()
_P = C.c_void_p
_U32 = C.c_uint32
_I = C.c_int


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Oracle:
    """The plain-C restatement (liboracle.so)."""

    def __init__(self, path: Path | None = None):
        path = path or HERE / "liboracle.so"
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.pgo_fit_lpmm32.argtypes = [C.POINTER(abi.FitConfig), _I, _U32, _P, _P, _P, _P, _I]
        L.pgo_fit_f64.argtypes = [C.POINTER(abi.FitConfig), _I, _U32, _P, _P, _P, _P, _I]
        L.pgo_init_states.argtypes = [C.POINTER(abi.FitConfig), _U32, _P, _I]
        L.pgo_initial_mus.argtypes = [_U32, _P]
        L.pgo_eval_ll_f64.argtypes = [_U32, _P, _P, _P, _P]
        L.pgo_fastexp.argtypes = [C.c_float]
        L.pgo_fastexp.restype = C.c_float
        L.pgo_prefit_parallax.argtypes = [_U32, _P, _P, _P, _P, _P]
        L.pgo_update_distances.argtypes = [_U32, _P, _P, _P, _P]
        L.pgo_reposition.argtypes = [_P, _P]
        L.pgo_pack_vmm_theta.argtypes = [_U32, _P, _I, _P]
        L.pgo_region_aabbs.argtypes = [_U32, _P, _P]
        L.pgo_sort_samples.argtypes = [_P, C.c_uint64, _U32, _P, _P]
        L.pgo_sort_samples.restype = C.c_uint64
        L.pgo_split_regions.argtypes = [_U32, _U32, C.c_float, _P, _P, _P, _P, _P, _P]
        L.pgo_split_regions.restype = _U32
        L.pgo_region_of.argtypes = [_P, _P, _P]
        L.pgo_region_of.restype = _U32
        L.pgo_postfit_lpmm32.argtypes = [C.POINTER(abi.FitConfig), C.POINTER(abi.SplitMergeConfig), _U32, _P, _P,
                                         _P, _P, _P, _I]

    def init_states(self, cfg, n, exact=True):
        s = np.zeros(n, dtype=abi.STATE_DTYPE)
        self.lib.pgo_init_states(C.byref(cfg), n, abi.ptr(s), int(exact))
        return s

    def fit(self, cfg, dirw, offsets, states=None, mode=abi.PG_FIT_INIT, f64=True, threads=None):
        dirw = _f32(dirw)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        R = offsets.shape[0] - 1
        st = np.zeros(R, dtype=abi.STATE_DTYPE) if states is None else states.copy()
        threads = threads or (os.cpu_count() or 1)
        if f64:
            ll = np.zeros(R, dtype=np.float64)
            self.lib.pgo_fit_f64(C.byref(cfg), mode, R, abi.ptr(dirw), abi.ptr(offsets), abi.ptr(st),
                                 abi.ptr(ll), threads)
        else:
            ll = np.zeros(R, dtype=np.float32)
            self.lib.pgo_fit_lpmm32(C.byref(cfg), mode, R, abi.ptr(dirw), abi.ptr(offsets),
                                    abi.ptr(st), abi.ptr(ll), threads)
        return st, ll

    def eval_ll(self, dirw, offsets, states):
        dirw = _f32(dirw)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        R = offsets.shape[0] - 1
        ll = np.zeros(R, dtype=np.float64)
        self.lib.pgo_eval_ll_f64(R, abi.ptr(dirw), abi.ptr(offsets), abi.ptr(states), abi.ptr(ll))
        return ll

    def initial_mus(self, K):
        out = np.zeros(48, dtype=np.float32)
        self.lib.pgo_initial_mus(K, abi.ptr(out))
        return out.reshape(3, 16)

    def fastexp(self, x):
        return np.array([self.lib.pgo_fastexp(float(v)) for v in np.ravel(x)], dtype=np.float32)

    def prefit_parallax(self, sorted_records, offsets, means):
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        R = offsets.shape[0] - 1
        N = sorted_records.shape[0]
        dirw = np.zeros((N, 4), dtype=np.float32)
        dist = np.zeros(N, dtype=np.float32)
        means = _f32(means)
        self.lib.pgo_prefit_parallax(R, abi.ptr(sorted_records), abi.ptr(offsets), abi.ptr(means),
                                     abi.ptr(dirw), abi.ptr(dist))
        return dirw, dist

    def postfit(self, cfg, sm, dirw, pdf, offsets, states, extras, threads=None):
        """PathGuiding::postFit's split and merge on lightpmm's FP32 arithmetic
        (no distance update); returns new states and statistics."""
        st = np.ascontiguousarray(states.copy())
        ex = np.ascontiguousarray(extras.copy())
        if ex.dtype != abi.EXTRA_DTYPE:
            ex = ex.view(abi.EXTRA_DTYPE)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        dirw, pdf = _f32(dirw), _f32(pdf)  # kept alive across the call
        threads = threads or (os.cpu_count() or 1)
        self.lib.pgo_postfit_lpmm32(C.byref(cfg), C.byref(sm), offsets.shape[0] - 1, abi.ptr(dirw),
                                    abi.ptr(pdf), abi.ptr(offsets), abi.ptr(st), abi.ptr(ex), threads)
        return st, ex

    def split_regions(self, cap, thr, states, extras, aabbs, nodes, leaf_of, n_nodes):
        """PathGuiding::update's region split check over all current regions;
        arrays are grown to `cap` regions and returned with the new counts."""
        n = states.shape[0]
        st = np.zeros(cap, dtype=states.dtype)
        st[:n] = states
        ex = None
        if extras is not None:
            ex = np.zeros(cap, dtype=abi.EXTRA_DTYPE)
            ex[:n] = extras.view(abi.EXTRA_DTYPE) if extras.dtype != abi.EXTRA_DTYPE else extras
        bx = np.zeros((cap, 6), dtype=np.float32)
        bx[:n] = aabbs
        nd = np.zeros(2 * cap, dtype=np.int32)
        nd[:n_nodes] = nodes[:n_nodes]
        lf = np.zeros(cap, dtype=np.uint32)
        lf[:n] = leaf_of[:n]
        nn = C.c_uint32(n_nodes)
        count = self.lib.pgo_split_regions(n, cap, float(thr), abi.ptr(st), abi.ptr(ex) if ex is not None else None,
                                           abi.ptr(bx), abi.ptr(nd), abi.ptr(lf), C.byref(nn))
        return (st[:count], ex[:count] if ex is not None else None, bx[:count], nd[:nn.value], lf[:count],
                int(nn.value))

    def complete_tree(self, split_count):
        """The region tree of pg_set_regions (breadth first) and each region's leaf."""
        n = 1 << split_count
        nodes = np.zeros(2 * n - 1, dtype=np.int32)
        nodes[:n - 1] = 2 * np.arange(n - 1) + 1
        nodes[n - 1:] = -np.arange(n, dtype=np.int32) - 1
        return nodes, (n - 1 + np.arange(n)).astype(np.uint32)

    def region_of(self, root, nodes, points):
        root = _f32(root)
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        pts = _f32(points).reshape(-1, 3)
        out = np.zeros(pts.shape[0], dtype=np.uint32)
        for i in range(pts.shape[0]):
            p = np.ascontiguousarray(pts[i])
            out[i] = self.lib.pgo_region_of(abi.ptr(root), abi.ptr(nodes), abi.ptr(p))
        return out

    def update_distances(self, dirw, dist, offsets, states):
        st = states.copy()
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        self.lib.pgo_update_distances(offsets.shape[0] - 1, abi.ptr(_f32(dirw)), abi.ptr(_f32(dist)),
                                      abi.ptr(offsets), abi.ptr(st))
        return st

    def reposition(self, state, new_to_old):
        s = np.array(state, dtype=abi.STATE_DTYPE).reshape(1).copy()
        v = _f32(new_to_old)
        self.lib.pgo_reposition(abi.ptr(s), abi.ptr(v))
        return s[0]

    def pack_vmm_theta(self, states, use_parallax=True):
        out = np.zeros(states.shape[0], dtype=abi.VMM_THETA_DTYPE)
        self.lib.pgo_pack_vmm_theta(states.shape[0], abi.ptr(states), int(use_parallax), abi.ptr(out))
        return out

    def region_aabbs(self, split_count, scene_aabb):
        out = np.zeros((1 << split_count, 6), dtype=np.float32)
        a = _f32(scene_aabb)
        self.lib.pgo_region_aabbs(split_count, abi.ptr(a), abi.ptr(out))
        return out

    def sort_samples(self, records, n_regions):
        sorted_out = np.zeros_like(records)
        offsets = np.zeros(n_regions + 1, dtype=np.uint32)
        n = self.lib.pgo_sort_samples(abi.ptr(records), records.shape[0], n_regions,
                                      abi.ptr(sorted_out), abi.ptr(offsets))
        return sorted_out[:n], offsets


class ReferenceFit:
    """The reference's own lightpmm fit (oracle/_ref/liblightpmm_ref.so, built by
    oracle/build_oracle.py: on x86-64 from the tree with the vendored
    vectorclass, elsewhere from the staged headers with the portable
    vectorclass stand-in)."""

    PATH = HERE / "_ref" / "liblightpmm_ref.so"

    @classmethod
    def available(cls, path: Path | None = None) -> bool:
        return (path or cls.PATH).exists()

    def __init__(self, path: Path | None = None):
        self.lib = C.CDLL(str(path or self.PATH))
        L = self.lib
        L.lpmm_ref_init.argtypes = [C.POINTER(abi.FitConfig), _U32, _P]
        L.lpmm_ref_fit.argtypes = [C.POINTER(abi.FitConfig), _I, _U32, _P, _P, _P, _P]
        L.lpmm_ref_fit_threads.argtypes = [C.POINTER(abi.FitConfig), _I, _U32, _P, _P, _P, _P, _I]
        L.lpmm_ref_update_distances.argtypes = [_U32, _P, _P, _P, _P]
        L.lpmm_ref_reposition.argtypes = [_P, _P]
        L.lpmm_ref_fastexp.argtypes = [_P, _P, _U32]
        L.lpmm_ref_postfit.argtypes = [C.POINTER(abi.FitConfig), C.POINTER(abi.SplitMergeConfig), _U32, _P, _P, _P,
                                       _P, _P]
        L.lpmm_ref_state_size.restype = _U32
        assert L.lpmm_ref_state_size() == abi.STATE_DTYPE.itemsize

    def init_states(self, cfg, n):
        s = np.zeros(n, dtype=abi.STATE_DTYPE)
        self.lib.lpmm_ref_init(C.byref(cfg), n, abi.ptr(s))
        return s

    def fit(self, cfg, dirw, offsets, states=None, mode=abi.PG_FIT_INIT, threads: int = 1):
        """Regions serial as the reference fits them (threads 1), or spread
        over host threads."""
        dirw = _f32(dirw)
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        R = offsets.shape[0] - 1
        st = np.zeros(R, dtype=abi.STATE_DTYPE) if states is None else states.copy()
        ll = np.zeros(R, dtype=np.float32)
        if threads > 1:
            self.lib.lpmm_ref_fit_threads(C.byref(cfg), mode, R, abi.ptr(dirw), abi.ptr(offsets), abi.ptr(st),
                                          abi.ptr(ll), threads)
        else:
            self.lib.lpmm_ref_fit(C.byref(cfg), mode, R, abi.ptr(dirw), abi.ptr(offsets), abi.ptr(st),
                                  abi.ptr(ll))
        return st, ll

    def postfit(self, cfg, sm, dirw, pdf, dist, offsets, states, extras):
        """PathGuiding::postFit with split/merge per region (regions without
        samples are skipped, as PathGuiding::update skips them)."""
        st, ex = states.copy(), extras.copy()
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        dirw, pdf = _f32(dirw), _f32(pdf)
        dist = _f32(dist) if dist is not None else None
        for r in range(offsets.shape[0] - 1):
            b, e = int(offsets[r]), int(offsets[r + 1])
            if e == b:
                continue
            one_st, one_ex = st[r:r + 1].copy(), ex[r:r + 1].copy()
            d = np.ascontiguousarray(dirw[b:e])
            p = np.ascontiguousarray(pdf[b:e])
            t = np.ascontiguousarray(dist[b:e]) if dist is not None else None
            self.lib.lpmm_ref_postfit(C.byref(cfg), C.byref(sm), e - b, abi.ptr(d), abi.ptr(p),
                                      abi.ptr(t) if t is not None else None, abi.ptr(one_st), abi.ptr(one_ex))
            st[r], ex[r] = one_st[0], one_ex[0]
        return st, ex

    def update_distances(self, dirw, dist, offsets, states):
        st = states.copy()
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        self.lib.lpmm_ref_update_distances(offsets.shape[0] - 1, abi.ptr(_f32(dirw)),
                                           abi.ptr(_f32(dist)), abi.ptr(offsets), abi.ptr(st))
        return st

    def reposition(self, state, new_to_old):
        s = np.array(state, dtype=abi.STATE_DTYPE).reshape(1).copy()
        self.lib.lpmm_ref_reposition(abi.ptr(s), abi.ptr(_f32(new_to_old)))
        return s[0]

    def fastexp(self, x):
        x = _f32(x)
        y = np.zeros_like(x)
        self.lib.lpmm_ref_fastexp(abi.ptr(x), abi.ptr(y), x.size)
        return y


class PgoScene(C.Structure):
    _fields_ = [("nodes", _P), ("n_nodes", _U32), ("tri_verts", _P), ("n_tris", _U32), ("pos", _P),
                ("n_vertices", _U32), ("idx", _P), ("tri_mat", _P), ("mats", _P), ("n_mats", _U32),
                ("spheres", _P), ("n_spheres", _U32), ("camera", abi.Camera), ("env", _P), ("env_w", _U32),
                ("env_h", _U32), ("tri_uv", _P), ("tex_info", _P), ("tex_data", _P), ("n_tex", _U32),
                ("alpha_salt", _U32)]


class PgoGuide(C.Structure):
    _fields_ = [("root", C.c_float * 6), ("split_count", _U32), ("nodes", _P), ("vmm", _P),
                ("use_parallax", C.c_int32)]


class TraceOracle:
    """CPU twins of the tracer (oracle/pg_oracle_trace.cpp, in liboracle.so)."""

    def __init__(self, path: Path | None = None):
        path = path or HERE / "liboracle.so"
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.pgo_trace_closest.argtypes = [C.POINTER(PgoScene), _P, _U32, _P, _I]
        L.pgo_trace_any.argtypes = [C.POINTER(PgoScene), _P, _U32, _P, _I]
        L.pgo_trace_closest_counted.argtypes = [C.POINTER(PgoScene), _P, _U32, _P, _P, _P, _I]
        L.pgo_render_f64.argtypes = [C.POINTER(PgoScene), C.POINTER(abi.RenderParams), C.POINTER(PgoGuide), _P, _U32,
                                     _U32, _I]
        L.pgo_rnd.argtypes = [_U32, _U32, _U32, _U32]
        L.pgo_rnd.restype = C.c_float
        L.pgo_probe_shading.argtypes = [_P, _U32, _P, _U32, _P, _U32, _P]

    def probe_shading(self, mats: np.ndarray, vmms: np.ndarray, probes: np.ndarray) -> np.ndarray:
        """The FP64 restatement of the renderer's shading functions on
        pg_probe_shading records; (n, 8) float64."""
        m = np.ascontiguousarray(mats, dtype=abi.MATERIAL_DTYPE)
        v = np.ascontiguousarray(vmms, dtype=abi.VMM_THETA_DTYPE)
        p = np.ascontiguousarray(probes, dtype=abi.PROBE_DTYPE)
        out = np.zeros((max(len(p), 1), 8), dtype=np.float64)
        self.lib.pgo_probe_shading(m.ctypes.data, len(m), v.ctypes.data, len(v), p.ctypes.data, len(p),
                                   out.ctypes.data)
        return out[:len(p)]

    @staticmethod
    def scene(exp: dict, camera: "abi.Camera | None" = None) -> tuple:
        keep = {k: np.ascontiguousarray(v) for k, v in exp.items() if isinstance(v, np.ndarray)}
        env = keep.get("env")
        s = PgoScene(keep["nodes"].ctypes.data, keep["nodes"].shape[0], keep["tri_verts"].ctypes.data,
                     keep["tri_verts"].shape[0], keep["pos"].ctypes.data, keep["pos"].shape[0],
                     keep["idx"].ctypes.data, keep["tri_mat"].ctypes.data, keep["mats"].ctypes.data,
                     keep["mats"].shape[0], keep["spheres"].ctypes.data, keep["spheres"].shape[0],
                     camera if camera is not None else exp["info"].camera,
                     env.ctypes.data if env is not None else None, env.shape[1] if env is not None else 0,
                     env.shape[0] if env is not None else 0)
        if "tri_uv" in keep and keep["tri_uv"].size:
            s.tri_uv = keep["tri_uv"].ctypes.data
        if "tex_info" in keep and keep["tex_info"].shape[0]:
            s.tex_info = keep["tex_info"].ctypes.data
            s.tex_data = keep["tex_data"].ctypes.data
            s.n_tex = keep["tex_info"].shape[0]
        return s, keep

    def closest(self, exp, rays, threads=None):
        s, keep = self.scene(exp)
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], dtype=abi.HIT_DTYPE)
        self.lib.pgo_trace_closest(C.byref(s), rays.ctypes.data, rays.shape[0], hits.ctypes.data,
                                   threads or (os.cpu_count() or 1))
        return hits

    def closest_counted(self, exp, rays, threads=None):
        """Closest hits plus per-ray BVH node fetches and triangle tests."""
        s, keep = self.scene(exp)
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        hits = np.zeros(n, dtype=abi.HIT_DTYPE)
        nodes = np.zeros(n, dtype=np.uint32)
        tris = np.zeros(n, dtype=np.uint32)
        self.lib.pgo_trace_closest_counted(C.byref(s), rays.ctypes.data, n, hits.ctypes.data, nodes.ctypes.data,
                                           tris.ctypes.data, threads or (os.cpu_count() or 1))
        return hits, nodes, tris

    def any(self, exp, rays, threads=None):
        s, keep = self.scene(exp)
        rays = np.ascontiguousarray(rays)
        occ = np.zeros(rays.shape[0], dtype=np.uint32)
        self.lib.pgo_trace_any(C.byref(s), rays.ctypes.data, rays.shape[0], occ.ctypes.data,
                               threads or (os.cpu_count() or 1))
        return occ

    def render(self, exp, params, guide=None, rows=None, threads=None, camera=None):
        """FP64 render: returns (H, W, 3) radiance sums over params.spp samples."""
        s, keep = self.scene(exp, camera)
        W, H = s.camera.width, s.camera.height
        img = np.zeros((H, W, 3), dtype=np.float64)
        r0, r1 = rows if rows is not None else (0, H)
        g = None
        if guide is not None:
            vmm = np.ascontiguousarray(guide["vmm"])
            keep["_vmm"] = vmm
            nodes = guide.get("nodes")
            nodes = np.ascontiguousarray(nodes, dtype=np.int32) if nodes is not None else None
            g = PgoGuide((C.c_float * 6)(*[float(x) for x in guide["root"]]), guide["split_count"],
                         nodes.ctypes.data if nodes is not None else None, vmm.ctypes.data,
                         int(guide.get("use_parallax", 1)))
        self.lib.pgo_render_f64(C.byref(s), C.byref(params), C.byref(g) if g is not None else None, img.ctypes.data,
                                r0, r1, threads or (os.cpu_count() or 1))
        return img

    def rnd(self, seed, pixel, sample, dim):
        return self.lib.pgo_rnd(seed, pixel, sample, dim)
