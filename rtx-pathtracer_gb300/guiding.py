"""Host-side mirror of the reference's guiding loop over the C ABI.

- SampleCollector (src/SampleCollector.h:36-39, src/SampleCollector.cpp:29-131):
  the tracer's record buffer, width * height * 16 DirectionalData slots on the
  device, and getSortedData as a host copy bucketed by region.
- PathGuiding (src/PathGuiding.h:132-136): regions from `splitCount` midpoint
  splits of the scene box, update(SampleCollector) fitting every region's
  vMF mixture on the device, getRegionCount().
- guided_sequence: the headless form of RayTracingApp's frame loop
  (src/RayTracingApp.cpp:125-157): training passes that render with sample
  recording and call PathGuiding::update, then a guided render.
- prepare_irradiance_cache / adrrs_estimate / adrrs_frames: the irradiance
  cache's prepare frames, the ADRRS estimate frame and the ADRRS frames
  (src/RayTracingApp.cpp:1129-1170, 1206-1217).

Device buffers are torch tensors (allocation and streams only); all work is in
the library.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import FitContext, Scene, abi

RECORD_BYTES = 40
RECORDS_PER_PIXEL = 16  # MAX_DIRECTIONAL_DATA_PER_PIXEL (shaders/limits.glsl:7)


def _torch():
    import torch
    return torch


class SampleCollector:
    """SampleCollector(regionCount, imageSize): one record slot per pixel and
    path vertex, written by pg_render with record_samples."""

    def __init__(self, region_count: int, width: int, height: int):
        torch = _torch()
        self.region_count = region_count
        self.width, self.height = width, height
        self.n_slots = width * height * RECORDS_PER_PIXEL
        self.buffer = torch.empty(self.n_slots * RECORD_BYTES, dtype=torch.uint8, device="cuda")

    def get_sorted_data(self, guiding: "PathGuiding", stream=None):
        """getSortedData (src/SampleCollector.cpp:76-131): records grouped by
        region (stable), with regionCount + 1 offsets; INVALID records are
        dropped.  Returns (records as a structured array, offsets)."""
        torch = _torch()
        R = guiding.get_region_count()  # regions may have been split since construction
        out = torch.empty(self.n_slots * RECORD_BYTES, dtype=torch.uint8, device="cuda")
        offs = torch.empty(R + 1, dtype=torch.int32, device="cuda")
        guiding.ctx.sort_samples(self.buffer, self.n_slots, R, out, offs, stream=stream)
        torch.cuda.synchronize()
        offsets = offs.cpu().numpy().view(np.uint32).copy()
        n = int(offsets[-1])
        from .workloads import RECORD_DTYPE
        rec = np.frombuffer(out[: n * RECORD_BYTES].cpu().numpy().tobytes(), dtype=RECORD_DTYPE).copy()
        return rec, offsets


class PathGuiding:
    """PathGuiding(splitCount, sceneAabb, useParallaxCompensation); split and
    merge of mixture components after each fit is on by default, as the
    reference's splitAndMerge (src/PathGuiding.h:124)."""

    def __init__(self, split_count: int, scene_aabb, use_parallax: bool = True, cfg: "abi.FitConfig | None" = None,
                 stream=None, split_and_merge: "bool | abi.SplitMergeConfig" = True, split_regions: bool = False,
                 samples_for_region_split: float = 10000.0, max_regions: int | None = None):
        cfg = cfg if cfg is not None else abi.default_fit_config()
        cfg.use_parallax = 1 if use_parallax else 0
        self.split_count = split_count
        self.ctx = FitContext(cfg, max_regions=max(max_regions or 0, 1 << split_count))
        self.ctx.set_regions(split_count, np.asarray(scene_aabb, dtype=np.float32), stream=stream)
        if isinstance(split_and_merge, abi.SplitMergeConfig):
            self.ctx.set_split_merge(split_and_merge)
        elif split_and_merge:
            self.ctx.set_split_merge()
        if split_regions:  # splitRegions / samplesForRegionSplit (src/PathGuiding.h:121-122), off by default
            self.ctx.set_region_split(abi.default_region_split_config(samples_for_region_split=samples_for_region_split))

    def get_region_count(self) -> int:
        return self.ctx.region_count()

    def update(self, collector: SampleCollector, stream=None) -> bool:
        """One guiding pass over the collector's records (bucket, parallax
        pre-pass, fit or stepwise update, split and merge, distances, VMM_Theta).  Returns
        whether a region was split (the reference's signal to rebind the
        tracer's region buffers; here the tracer picks the new tree up itself)."""
        before = self.ctx.region_count()
        self.ctx.update(collector.buffer, collector.n_slots, stream=stream)
        return self.ctx.region_count() != before

    def close(self):
        self.ctx.close()


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    """Relative MSE, mean over pixels and channels of (x - r)^2 / (r^2 + eps)."""
    img = np.asarray(img, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.mean((img - ref) ** 2 / (ref * ref + eps)))


def guided_sequence(scene: Scene, guiding: PathGuiding, collector: SampleCollector, image, train_spp=(1, 2, 4, 8, 16, 32),
                    final_spp: int = 64, max_depth: int = 10, seed: int = 1, guiding_prob: float = 0.5,
                    accumulate_training: bool = True, surrogate=None, judge_min_records: int = 32,
                    stream=None, render_flags: int = 0) -> dict:
    """Training passes (render with recording, then PathGuiding::update; the
    first pass is unguided), then a guided render of final_spp samples.  The
    image (cleared first) receives radiance sums: of every pass when
    accumulate_training (the reference keeps accumulating frames while it
    trains, src/RayTracingApp.cpp:125-157), else of the final render only.
    With a surrogate (a Surrogate), every pass's valid records also train the
    network online (one epoch each), and before the final render the network
    is judged against the fit region by region on the last pass's records
    (pg_mlp_judge_guide).  Returns CUDA-event times in ms and the number of
    samples per pixel summed.  render_flags go to every render
    (PG_RENDER_GUIDE_ALMOST_DISCRETE: the reference's rule of guiding every
    non-discrete material)."""
    torch = _torch()
    s = stream or torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    scratch = image if accumulate_training else torch.empty_like(image)
    R = guiding.get_region_count()
    if surrogate is not None:
        srt = torch.empty(collector.n_slots * RECORD_BYTES, dtype=torch.uint8, device="cuda")
        offs = torch.empty(R + 1, dtype=torch.int32, device="cuda")
    switched = None
    trained = []
    with torch.cuda.stream(s):
        image.zero_()
        ev[0].record(s)
        for i, spp in enumerate(train_spp):
            p = abi.render_params(spp=spp, max_depth=max_depth, seed=seed + 1000 * (i + 1),
                                  use_guiding=1 if i > 0 else 0, guiding_prob=guiding_prob, record_samples=1,
                                  flags=render_flags)
            scene.render(p, scratch, guide=guiding.ctx, records_dev=collector.buffer, stream=s, stats=False)
            guiding.update(collector, stream=s)
            if surrogate is not None:
                guiding.ctx.sort_samples(collector.buffer, collector.n_slots, R, srt, offs, stream=s)
                n_valid = int(offs[R].item())
                trained.append(n_valid)
                surrogate.train(srt, n_valid, stream=s, want_loss=False)
        if surrogate is not None:
            switched = surrogate.judge_guide(guiding.ctx, srt, n_valid, min_records=judge_min_records, stream=s)
        ev[1].record(s)
        p = abi.render_params(spp=final_spp, max_depth=max_depth, seed=seed, use_guiding=1,
                              guiding_prob=guiding_prob, flags=render_flags)
        scene.render(p, image, guide=guiding.ctx, stream=s, stats=False)
        ev[2].record(s)
    torch.cuda.synchronize()
    total = final_spp + (sum(train_spp) if accumulate_training else 0)
    out = {"train_ms": ev[0].elapsed_time(ev[1]), "render_ms": ev[1].elapsed_time(ev[2]),
           "total_ms": ev[0].elapsed_time(ev[2]), "spp": total}
    if switched is not None:
        out["regions_switched"] = switched
        out["records_trained_per_pass"] = trained
    return out


# --- irradiance cache and ADRRS frames (src/RayTracingApp.cpp:1129-1170, 1206-1217)
IRRADIANCE_PREPARE_FRAMES = 50  # irradianceCachePrepareFrames (src/RayTracingApp.h:175)


def prepare_irradiance_cache(scene: Scene, frames: int = IRRADIANCE_PREPARE_FRAMES, max_depth: int = 10, seed: int = 1,
                             cfg: "abi.IrradianceCacheConfig | None" = None, use_on_glossy: bool = False,
                             stream=None) -> np.ndarray:
    """The reference's prepare frames: `frames` frames of one sample per pixel
    that grow the scene's irradiance cache and whose images are not kept
    (isIrradiancePrepareFrame).  Sets a cache on the scene (cfg or the
    defaults, use_on_glossy as ADRRS's prepare frames set it) and returns its
    entries."""
    torch = _torch()
    if cfg is None:
        cfg = abi.IrradianceCacheConfig()
        scene.lib.pg_default_irradiance_cache_config(ctypes.byref(cfg))
    cfg.use_on_glossy = int(use_on_glossy)
    scene.set_irradiance_cache(cfg)
    cam = scene.info().camera
    scratch = torch.zeros(cam.width * cam.height * 3, dtype=torch.float32, device="cuda")
    for f in range(frames):
        params = abi.render_params(spp=1, max_depth=max_depth, seed=seed + f, use_nee=1, use_mis=1,
                                   flags=abi.PG_RENDER_IRRADIANCE_CACHE)
        scene.render(params, scratch, stream=stream, stats=False)
    torch.cuda.synchronize()
    return scene.irradiance_cache()


def adrrs_estimate(scene: Scene, spp: int = 16, max_depth: int = 3, seed: int = 7, stream=None):
    """The pixel estimate ADRRS compares against, rendered with the
    reference's estimate settings (setEstimateRTSettings: 16 samples per
    pixel, the irradiance cache used, next-event estimation, maxDepth 1 - a
    path length of 3 here): a device tensor of per-pixel mean radiance."""
    torch = _torch()
    cam = scene.info().camera
    img = torch.zeros(cam.width * cam.height * 3, dtype=torch.float32, device="cuda")
    params = abi.render_params(spp=spp, max_depth=max_depth, seed=seed, use_nee=1, use_mis=1,
                               flags=abi.PG_RENDER_IRRADIANCE_CACHE | abi.PG_RENDER_IC_FROZEN)
    scene.render(params, img, stream=stream, stats=False)
    torch.cuda.synchronize()
    return img / spp


def adrrs_frames(scene: Scene, image, frames: int, spp: int = 1, max_depth: int = 30, seed: int = 100,
                 s: float = 5.0, split: bool = True, prepare_frames: int = IRRADIANCE_PREPARE_FRAMES, stream=None):
    """RayTracingApp's ADRRS sequence: prepare frames growing the cache (on
    glossy surfaces too), the estimate frame, then `frames` frames of `spp`
    samples with adjoint-driven roulette and splitting added into image.
    Returns the estimate tensor (kept alive with the scene's ADRRS settings)."""
    prepare_irradiance_cache(scene, prepare_frames, seed=seed, use_on_glossy=True, stream=stream)
    est = adrrs_estimate(scene, stream=stream)
    scene.set_adrrs(est, s=s, split=split)
    for f in range(frames):
        params = abi.render_params(spp=spp, max_depth=max_depth, seed=seed + prepare_frames + f, use_nee=1,
                                   use_mis=1, flags=abi.PG_RENDER_ADRRS)
        scene.render(params, image, stream=stream, stats=False)
    return est
