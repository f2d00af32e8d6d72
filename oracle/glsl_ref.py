"""TEST INFRASTRUCTURE: ctypes access to the reference's shader functions
compiled as host C++ (oracle/_ref/libglslref.so, built by
oracle/build_glsl_ref.py where the reference tree is present).

The functions are the reference's own (shaders/raytrace.rgen, guiding.glsl,
random.glsl, transform.glsl); this module maps the library's material and
mixture records onto the reference's, and turns the random state a sampling
function leaves behind into the list of numbers it drew, so the same numbers
can be handed to the project's implementations.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libglslref.so"

# the reference's MAT_* numbers (raytrace.rgen:21-27)
MAT_DIFFUSE, MAT_SPECULAR, MAT_DIELECTRIC, MAT_LIGHT, MAT_PHONG, MAT_CONDUCTOR, MAT_ROUGH_CONDUCTOR = range(7)
# the library's PG_MAT_* numbers (include/pathguide.h)
PG_MAT = dict(DIFFUSE=0, SPECULAR=1, DIELECTRIC=2, LIGHT=3, PHONG=4, CONDUCTOR=5, GGX=6, BECKMANN=7)
_PG_TO_REF = {0: MAT_DIFFUSE, 1: MAT_SPECULAR, 2: MAT_DIELECTRIC, 3: MAT_LIGHT, 4: MAT_PHONG, 5: MAT_CONDUCTOR,
              7: MAT_ROUGH_CONDUCTOR}


class RefMaterial(C.Structure):
    _fields_ = [("type", C.c_int32), ("light", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3), ("specular_highlight", C.c_float), ("refraction_index", C.c_float),
                ("eta", C.c_float), ("k", C.c_float), ("roughness", C.c_float)]


def ref_material(pg: np.void) -> RefMaterial:
    """The reference's Material for a library pg_material record (fields as
    the reference's SceneLoader fills them, src/SceneLoader.cpp:558-648)."""
    t = int(pg["type"])
    m = RefMaterial()
    m.type = _PG_TO_REF[t]
    m.light[:] = [float(x) for x in pg["emission"]]
    if t in (PG_MAT["SPECULAR"], PG_MAT["DIELECTRIC"]):
        m.specular[:] = [float(x) for x in pg["albedo"]]
    else:
        m.diffuse[:] = [float(x) for x in pg["albedo"]]
    if t == PG_MAT["PHONG"]:
        m.specular[:] = [float(x) for x in pg["specular"]]
    m.specular_highlight = float(pg["exponent"])
    m.refraction_index = float(pg["ior"]) if float(pg["ior"]) > 0 else 1.0
    m.eta, m.k, m.roughness = float(pg["eta"]), float(pg["k"]), float(pg["roughness"])
    return m


def available() -> bool:
    return LIB_PATH.exists()


class RenderConfig(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("max_follow_discrete", C.c_uint32),
                ("use_nee", C.c_uint32), ("use_mis", C.c_uint32), ("use_guiding", C.c_uint32),
                ("guiding_prob", C.c_float), ("use_parallax", C.c_uint32), ("frame_seed", C.c_uint32),
                ("region_splits", C.c_uint32), ("region_root", C.c_float * 6), ("use_ic", C.c_uint32),
                ("use_adrrs", C.c_uint32), ("adrrs_split", C.c_uint32), ("adrrs_s", C.c_float),
                ("estimate", C.c_void_p)]


class IcConfig(C.Structure):
    _fields_ = [("a", C.c_float), ("min_radius", C.c_float), ("gradients_max_length", C.c_float),
                ("use_gradients", C.c_uint32), ("visibility_check", C.c_uint32), ("use_on_glossy", C.c_uint32),
                ("capacity", C.c_uint32), ("num_nee", C.c_uint32)]


def ic_config(capacity, a=0.2, min_radius=0.1, gradients_max_length=5.0, use_gradients=0, visibility_check=0,
              use_on_glossy=0, num_nee=0) -> IcConfig:
    return IcConfig(a, min_radius, gradients_max_length, use_gradients, visibility_check, use_on_glossy, capacity,
                    num_nee)


class GlslRef:
    def __init__(self, path: Path = LIB_PATH):
        self.lib = C.CDLL(str(path))
        f, p, u, i = C.c_float, C.c_void_p, C.c_uint32, C.c_int
        P = C.POINTER
        sig = {
            "glslref_rnd_sequence": (None, [u, u, p]),
            "glslref_fresnel": (f, [f, f]),
            "glslref_fresnel_conductor": (f, [f, f, f]),
            "glslref_beckmann_D": (f, [p, p, p]),
            "glslref_beckmann_G1": (f, [p, p, p, p]),
            "glslref_power_heuristic": (f, [f, f]),
            "glslref_eval_bsdf": (f, [p, p, p, p, i, p]),
            "glslref_sample_bsdf": (f, [p, p, p, i, u, p, P(u)]),
            "glslref_vmm_pdf": (f, [p, p, p, i]),
            "glslref_sample_vmm": (None, [p, p, i, u, p, P(u)]),
            "glslref_new_direction": (f, [p, p, p, p, i, p, C.c_int32, i, f, i, u, p, p, P(u)]),
            "glslref_cosine_hemisphere": (None, [p, u, p, P(u)]),
            "glslref_cosine_power": (None, [p, f, u, p, P(u)]),
            "glslref_beckmann_normal": (None, [p, p, u, p, P(u)]),
            "glslref_to_world": (None, [p, p, p]),
            "glslref_almost_discrete": (i, [p]),
            "glslref_discrete": (i, [p]),
            "glslref_record_path": (u, [u, p, p, p, p, p, p, p]),
            "glslref_weight_window": (f, [p, p, p, f, u, P(C.c_int32), P(u)]),
            "glslref_approx_diffuse": (None, [p, p, p, p]),
            "glslref_render": (i, [p, P(RenderConfig), p, u, u, i, p]),
            "glslref_ic_set": (i, [p, u, P(IcConfig)]),
            "glslref_ic_get": (u, [p, u, P(u)]),
            "glslref_ic_query": (None, [p, p, u, p, p]),
            "glslref_ic_compute": (i, [p, P(RenderConfig), p, p, p, p, u, i, p]),
            "glslref_ic_create_update": (i, [p, P(RenderConfig), p, p, u, u]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args

    # ---- random numbers -------------------------------------------------
    def drawn(self, state: int, state_after: int, limit: int = 64) -> np.ndarray:
        """The rnd() values a call drew between two generator states."""
        seq = np.zeros(limit, dtype=np.float32)
        self.lib.glslref_rnd_sequence(state, limit, seq.ctypes.data)
        s = state
        for n in range(limit + 1):
            if s == state_after:
                return seq[:n].copy()
            s = (1664525 * s + 1013904223) & 0xFFFFFFFF
        raise RuntimeError("random state not reached")

    @staticmethod
    def _v(x) -> np.ndarray:
        return np.ascontiguousarray(x, dtype=np.float32)

    # ---- functions --------------------------------------------------------
    def fresnel(self, eta, cos_i):
        return self.lib.glslref_fresnel(eta, cos_i)

    def fresnel_conductor(self, cos_i, eta, k):
        return self.lib.glslref_fresnel_conductor(cos_i, eta, k)

    def eval_bsdf(self, mat: RefMaterial, n, wi, wo, front=True):
        """(evalBsdf, pdfBSDF)."""
        out = np.zeros(3, np.float32)
        n, wi, wo = self._v(n), self._v(wi), self._v(wo)
        pdf = self.lib.glslref_eval_bsdf(C.byref(mat), n.ctypes.data, wi.ctypes.data, wo.ctypes.data,
                                         int(front), out.ctypes.data)
        return out, pdf

    def sample_bsdf(self, mat: RefMaterial, wi, n, front, state):
        """(direction, pdf, numbers drawn)."""
        d = np.zeros(3, np.float32)
        after = C.c_uint32()
        wi, n = self._v(wi), self._v(n)
        pdf = self.lib.glslref_sample_bsdf(C.byref(mat), wi.ctypes.data, n.ctypes.data, int(front), state,
                                           d.ctypes.data, C.byref(after))
        return d, pdf, self.drawn(state, after.value)

    def vmm_pdf(self, vmm: np.ndarray, wo, pos, parallax):
        wo, pos = self._v(wo), self._v(pos)
        return self.lib.glslref_vmm_pdf(vmm.ctypes.data, wo.ctypes.data, pos.ctypes.data, int(parallax))

    def sample_vmm(self, vmm: np.ndarray, pos, parallax, state):
        d = np.zeros(3, np.float32)
        after = C.c_uint32()
        pos = self._v(pos)
        self.lib.glslref_sample_vmm(vmm.ctypes.data, pos.ctypes.data, int(parallax), state, d.ctypes.data,
                                    C.byref(after))
        return d, self.drawn(state, after.value)

    def new_direction(self, mat: RefMaterial, origin, n, wi, front, vmm, region, use_guiding, guiding_prob,
                      parallax, state):
        """getNewDirection: (direction, pdf, throughput change, numbers drawn)."""
        d = np.zeros(3, np.float32)
        tc = np.zeros(3, np.float32)
        after = C.c_uint32()
        origin, n, wi = self._v(origin), self._v(n), self._v(wi)
        pdf = self.lib.glslref_new_direction(C.byref(mat), origin.ctypes.data, n.ctypes.data, wi.ctypes.data,
                                             int(front), vmm.ctypes.data, int(region), int(use_guiding),
                                             guiding_prob, int(parallax), state, d.ctypes.data, tc.ctypes.data,
                                             C.byref(after))
        return d, pdf, tc, self.drawn(state, after.value)

    def cosine_hemisphere(self, n, state):
        d = np.zeros(3, np.float32)
        after = C.c_uint32()
        n = self._v(n)
        self.lib.glslref_cosine_hemisphere(n.ctypes.data, state, d.ctypes.data, C.byref(after))
        return d, self.drawn(state, after.value)

    def cosine_power(self, axis, p, state):
        d = np.zeros(3, np.float32)
        after = C.c_uint32()
        axis = self._v(axis)
        self.lib.glslref_cosine_power(axis.ctypes.data, p, state, d.ctypes.data, C.byref(after))
        return d, self.drawn(state, after.value)

    def beckmann_normal(self, mat, n, state):
        d = np.zeros(3, np.float32)
        after = C.c_uint32()
        n = self._v(n)
        self.lib.glslref_beckmann_normal(C.byref(mat), n.ctypes.data, state, d.ctypes.data, C.byref(after))
        return d, self.drawn(state, after.value)

    def to_world(self, v, n):
        out = np.zeros(3, np.float32)
        v, n = self._v(v), self._v(n)
        self.lib.glslref_to_world(v.ctypes.data, n.ctypes.data, out.ctypes.data)
        return out

    def almost_discrete(self, mat) -> bool:
        return bool(self.lib.glslref_almost_discrete(C.byref(mat)))

    def discrete(self, mat) -> bool:
        return bool(self.lib.glslref_discrete(C.byref(mat)))

    def record_path(self, kinds, pdfs, tcs, regions, lights):
        """Committed (weights, flags) of one path's recorded vertices."""
        n = len(kinds)
        k = np.ascontiguousarray(kinds, np.int32)
        p = np.ascontiguousarray(pdfs, np.float32)
        t = np.ascontiguousarray(tcs, np.float32).reshape(n, 3)
        r = np.ascontiguousarray(regions, np.uint32)
        L = np.ascontiguousarray(lights, np.float32).reshape(n, 3)
        w = np.zeros(16, np.float32)
        fl = np.zeros(16, np.uint32)
        m = self.lib.glslref_record_path(n, k.ctypes.data, p.ctypes.data, t.ctypes.data, r.ctypes.data,
                                         L.ctypes.data, w.ctypes.data, fl.ctypes.data)
        return w[:m].copy(), fl[:m].copy()

    def render(self, exp: dict, path_length: int, spp: int, frame_seed: int, use_nee=True, use_mis=True,
               guide: dict | None = None, guiding_prob=0.5, rows=None, threads=None, use_ic=False,
               adrrs: dict | None = None) -> np.ndarray:
        """The reference's estimator (raytrace() and the hit shaders compiled as
        C++) over an exported library scene: radiance sums (H, W, 3).
        path_length is the library's max_depth (paths of at most that many
        segments); the reference's maxDepth counts two fewer (its next-event
        estimation runs at the vertex after maxDepth).  use_ic: query the
        cache of ic_set at every cache-capable vertex (no entries are made).
        adrrs: {"estimate": (H, W, 3) mean radiance, "s", "split"} - ADRRS
        with the cache of ic_set."""
        import os
        from oracle.oracle import TraceOracle
        s, keep = TraceOracle.scene(exp)
        cam = exp["info"].camera
        W, H = cam.width, cam.height
        img = np.zeros((H, W, 3), dtype=np.float64)
        cfg = RenderConfig(spp=spp, max_depth=max(path_length - 2, 0), max_follow_discrete=0,
                           use_nee=int(use_nee), use_mis=int(use_mis), use_guiding=int(guide is not None),
                           guiding_prob=guiding_prob, frame_seed=frame_seed, use_ic=int(use_ic))
        est = None
        if adrrs is not None:
            est = np.ascontiguousarray(adrrs["estimate"], dtype=np.float32)
            cfg.use_adrrs, cfg.adrrs_split, cfg.adrrs_s = 1, int(adrrs["split"]), float(adrrs["s"])
            cfg.estimate = est.ctypes.data
        vmm = None
        if guide is not None:
            cfg.use_parallax = int(guide["use_parallax"])
            cfg.region_splits = int(guide["split_count"])
            cfg.region_root[:] = [float(x) for x in guide["root"]]
            vmm = np.ascontiguousarray(guide["vmm"])
        r0, r1 = rows if rows is not None else (0, H)
        st = self.lib.glslref_render(C.byref(s), C.byref(cfg), vmm.ctypes.data if vmm is not None else None, r0, r1,
                                     threads or os.cpu_count() or 1, img.ctypes.data)
        if st != 0:
            raise RuntimeError("glslref_render failed")
        return img

    # --- irradiance cache
    def ic_set(self, entries: np.ndarray, cfg: IcConfig):
        """The cache the reference's functions see (entries: pg_ic_entry rows)."""
        e = np.ascontiguousarray(entries)
        assert e.dtype.itemsize == 72
        if self.lib.glslref_ic_set(e.ctypes.data if len(e) else None, len(e), C.byref(cfg)) != 0:
            raise RuntimeError("glslref_ic_set failed")

    def ic_get(self, dtype) -> tuple[np.ndarray, int]:
        """The reference cache's entries and its round-robin update position."""
        nxt = C.c_uint32()
        n = self.lib.glslref_ic_get(None, 0, C.byref(nxt))
        out = np.zeros(n, dtype=dtype)
        self.lib.glslref_ic_get(out.ctypes.data if n else None, n, C.byref(nxt))
        return out, nxt.value

    def ic_query(self, pos, nrm):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        nrm = np.ascontiguousarray(nrm, dtype=np.float32)
        n = len(pos)
        rgb = np.zeros((n, 3), dtype=np.float32)
        found = np.zeros(n, dtype=np.uint32)
        self.lib.glslref_ic_query(pos.ctypes.data, nrm.ctypes.data, n, rgb.ctypes.data, found.ctypes.data)
        return rgb, found

    @staticmethod
    def _config(exp, use_nee, use_mis, guide, guiding_prob, frame_seed=0, spp=1, path_length=2, use_ic=0):
        cfg = RenderConfig(spp=spp, max_depth=max(path_length - 2, 0), max_follow_discrete=0,
                           use_nee=int(use_nee), use_mis=int(use_mis), use_guiding=int(guide is not None),
                           guiding_prob=guiding_prob, frame_seed=frame_seed, use_ic=int(use_ic))
        vmm = None
        if guide is not None:
            cfg.use_parallax = int(guide["use_parallax"])
            cfg.region_splits = int(guide["split_count"])
            cfg.region_root[:] = [float(x) for x in guide["root"]]
            vmm = np.ascontiguousarray(guide["vmm"])
        return cfg, vmm

    def ic_compute(self, exp: dict, pos, nrm, seeds, use_nee=True, use_mis=True, guide=None, guiding_prob=0.5,
                   threads=None) -> np.ndarray:
        """calculateCacheData at each (pos, nrm) with random state seeds[i]:
        (n, 10) colour, rotation gradient, translation gradient, harmonicR."""
        import os
        from oracle.oracle import TraceOracle
        s, keep = TraceOracle.scene(exp)
        cfg, vmm = self._config(exp, use_nee, use_mis, guide, guiding_prob)
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        nrm = np.ascontiguousarray(nrm, dtype=np.float32)
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        out = np.zeros((len(pos), 10), dtype=np.float32)
        st = self.lib.glslref_ic_compute(C.byref(s), C.byref(cfg), vmm.ctypes.data if vmm is not None else None,
                                         pos.ctypes.data, nrm.ctypes.data, seeds.ctypes.data, len(pos),
                                         threads or os.cpu_count() or 1, out.ctypes.data)
        if st != 0:
            raise RuntimeError("glslref_ic_compute failed")
        return out

    def ic_create_update(self, exp: dict, pos=None, nrm=None, updates=0, seed=1, use_nee=True, use_mis=True) -> int:
        """createIrradianceCache at (pos, nrm) (if given), then `updates`
        calls of updateIrradianceCache, on the cache of ic_set."""
        from oracle.oracle import TraceOracle
        s, keep = TraceOracle.scene(exp)
        cfg, _ = self._config(exp, use_nee, use_mis, None, 0.5)
        p = np.ascontiguousarray(pos, dtype=np.float32) if pos is not None else None
        q = np.ascontiguousarray(nrm, dtype=np.float32) if nrm is not None else None
        return self.lib.glslref_ic_create_update(C.byref(s), C.byref(cfg), p.ctypes.data if p is not None else None,
                                                 q.ctypes.data if q is not None else None, updates, seed)

    def approx_diffuse(self, mat: RefMaterial, n, wi) -> np.ndarray:
        out = np.zeros(3, np.float32)
        n, wi = self._v(n), self._v(wi)
        self.lib.glslref_approx_diffuse(C.byref(mat), n.ctypes.data, wi.ctypes.data, out.ctypes.data)
        return out

    def weight_window(self, estimate, throughput, adjoint, s, state):
        """applyWeightWindow: (q, n, numbers drawn)."""
        n = C.c_int32()
        after = C.c_uint32()
        e, t, a = self._v(estimate), self._v(throughput), self._v(adjoint)
        q = self.lib.glslref_weight_window(e.ctypes.data, t.ctypes.data, a.ctypes.data, s, state, C.byref(n),
                                           C.byref(after))
        return q, n.value, self.drawn(state, after.value)
