// pathguiding.hpp - C++ facades with the reference's host interfaces over the
// C ABI of pathguide.h (header only; link libpathguide.so and cudart).
//
//   SceneLoader     src/SceneLoader.h:118-162   Mitsuba-XML scene, camera, scene box
//   SampleCollector src/SampleCollector.h:36-39 per-pixel guiding records on the device
//   PathGuiding     src/PathGuiding.h:121-136   spatial regions and their vMF mixtures
//   Tracer          (RayTracingApp's raytrace pass, src/RayTracingApp.cpp:99-112)
//
// The Vulkan objects of the reference constructors are replaced by a CUDA
// stream; errors become pg::Error exceptions (the reference's loaders throw
// std::runtime_error, src/SceneLoader.cpp:135-546).
#ifndef PATHGUIDING_HPP
#define PATHGUIDING_HPP

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pathguide.h"

namespace pg {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string &what)
        : std::runtime_error(std::string(pg_status_string(status)) + ": " + what), status(status) {}
    int status;
};

inline void check(int status, const pg_ctx *ctx = nullptr) {
    if (status != PG_OK) throw Error(status, pg_last_error(ctx));
}

inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(PG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

struct vec3 {
    float x = 0, y = 0, z = 0;
};

// Shapes.h Aabb: min and max corners.
struct Aabb {
    vec3 min, max;
    void to_array(float out[6]) const {
        out[0] = min.x, out[1] = min.y, out[2] = min.z;
        out[3] = max.x, out[4] = max.y, out[5] = max.z;
    }
};

// ---------------------------------------------------------------------------
// SceneLoader(filepath): geometry, materials, lights, camera and BVH.
// ---------------------------------------------------------------------------
class SceneLoader {
public:
    SceneLoader() = default;
    SceneLoader(const std::string &filepath, uint32_t width, uint32_t height) {
        check(pg_scene_load(filepath.c_str(), width, height, &scene_));
        read_camera();
    }
    static SceneLoader cornell(uint32_t width, uint32_t height, int ico_level = 5) {
        pg_cornell_params p{width, height, ico_level, 15.0f, 1.5f};
        SceneLoader s;
        check(pg_scene_create_cornell(&p, &s.scene_));
        s.read_camera();
        return s;
    }
    static SceneLoader plates(uint32_t width, uint32_t height, uint32_t occluder_grid = 707, uint32_t seed = 4) {
        pg_plates_params p{width, height, occluder_grid, seed};
        SceneLoader s;
        check(pg_scene_create_plates(&p, &s.scene_));
        s.read_camera();
        return s;
    }
    SceneLoader(SceneLoader &&o) noexcept { *this = std::move(o); }
    SceneLoader &operator=(SceneLoader &&o) noexcept {
        std::swap(scene_, o.scene_);
        origin = o.origin, target = o.target, upDir = o.upDir, vfov = o.vfov;
        return *this;
    }
    SceneLoader(const SceneLoader &) = delete;
    SceneLoader &operator=(const SceneLoader &) = delete;
    ~SceneLoader() { cleanup(); }

    // getSceneSize (src/SceneLoader.h:118)
    Aabb getSceneSize() const {
        pg_scene_info i{};
        check(pg_scene_get_info(scene_, &i));
        return Aabb{{i.aabb[0], i.aabb[1], i.aabb[2]}, {i.aabb[3], i.aabb[4], i.aabb[5]}};
    }
    pg_scene_info info() const {
        pg_scene_info i{};
        check(pg_scene_get_info(scene_, &i));
        return i;
    }
    // Writes origin / target / upDir / vfov back to the scene (the reference's
    // camera fields, src/SceneLoader.h:147-150).
    void applyCamera(uint32_t width, uint32_t height) {
        pg_camera c{};
        c.origin[0] = origin.x, c.origin[1] = origin.y, c.origin[2] = origin.z;
        c.target[0] = target.x, c.target[1] = target.y, c.target[2] = target.z;
        c.up[0] = upDir.x, c.up[1] = upDir.y, c.up[2] = upDir.z;
        c.vfov_deg = vfov;
        c.width = width;
        c.height = height;
        check(pg_scene_set_camera(scene_, &c));
    }
    pg_scene *handle() const { return scene_; }
    void cleanup() {
        if (scene_) pg_scene_destroy(scene_);
        scene_ = nullptr;
    }

    vec3 origin, target, upDir;
    float vfov = 45.0f;

private:
    void read_camera() {
        const pg_scene_info i = info();
        origin = {i.camera.origin[0], i.camera.origin[1], i.camera.origin[2]};
        target = {i.camera.target[0], i.camera.target[1], i.camera.target[2]};
        upDir = {i.camera.up[0], i.camera.up[1], i.camera.up[2]};
        vfov = i.camera.vfov_deg;
    }
    pg_scene *scene_ = nullptr;
};

// ---------------------------------------------------------------------------
// SampleCollector(regionCount, imageSize): the tracer's record buffer,
// MAX_DIRECTIONAL_DATA_PER_PIXEL (16) slots per pixel on the device.
// ---------------------------------------------------------------------------
class SampleCollector {
public:
    static constexpr uint32_t kPerPixel = 16;
    SampleCollector() = default;
    SampleCollector(uint32_t regionCount, uint32_t width, uint32_t height, cudaStream_t stream = nullptr)
        : region_count_(regionCount), slots_((uint64_t)width * height * kPerPixel), stream_(stream) {
        check_cuda(cudaMalloc(&records_, sizeof(pg_directional_data) * slots_), "SampleCollector buffer");
        pg_fit_config cfg;
        pg_default_fit_config(&cfg);
        check(pg_ctx_create(&cfg, regionCount, 0, &sorter_));
    }
    SampleCollector(SampleCollector &&o) noexcept { *this = std::move(o); }
    SampleCollector &operator=(SampleCollector &&o) noexcept {
        std::swap(region_count_, o.region_count_);
        std::swap(slots_, o.slots_);
        std::swap(records_, o.records_);
        std::swap(sorter_, o.sorter_);
        std::swap(stream_, o.stream_);
        return *this;
    }
    SampleCollector(const SampleCollector &) = delete;
    SampleCollector &operator=(const SampleCollector &) = delete;
    ~SampleCollector() { cleanup(); }

    pg_directional_data *deviceRecords() const { return records_; }
    uint64_t slotCount() const { return slots_; }
    uint32_t regionCount() const { return region_count_; }
    // After PathGuiding::update split regions (it returned true): bucket by the
    // new count from then on (the reference recreates its collector then).
    void setRegionCount(uint32_t regionCount) {
        if (regionCount == region_count_) return;
        pg_fit_config cfg;
        pg_default_fit_config(&cfg);
        pg_ctx *sorter = nullptr;
        check(pg_ctx_create(&cfg, regionCount, 0, &sorter));
        if (sorter_) pg_ctx_destroy(sorter_);
        sorter_ = sorter;
        region_count_ = regionCount;
    }

    // getSortedData (src/SampleCollector.cpp:76-131): a host copy of the
    // valid records grouped by region (stable), and regionCount + 1 offsets.
    std::shared_ptr<std::vector<pg_directional_data>> getSortedData(std::vector<uint32_t> &outRegionIndices) {
        pg_directional_data *sorted = nullptr;
        uint32_t *offsets = nullptr;
        check_cuda(cudaMalloc(&sorted, sizeof(pg_directional_data) * slots_), "sorted records");
        check_cuda(cudaMalloc(&offsets, sizeof(uint32_t) * (region_count_ + 1)), "region offsets");
        auto out = std::make_shared<std::vector<pg_directional_data>>();
        int st = pg_sort_samples(sorter_, records_, slots_, region_count_, sorted, offsets, stream_);
        if (st == PG_OK) {
            outRegionIndices.assign(region_count_ + 1, 0);
            cudaError_t e = cudaMemcpyAsync(outRegionIndices.data(), offsets, sizeof(uint32_t) * (region_count_ + 1),
                                            cudaMemcpyDeviceToHost, stream_);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
            if (e == cudaSuccess) {
                out->resize(outRegionIndices.back());
                if (!out->empty())
                    e = cudaMemcpy(out->data(), sorted, sizeof(pg_directional_data) * out->size(),
                                   cudaMemcpyDeviceToHost);
            }
            if (e != cudaSuccess) st = PG_ERR_CUDA;
        }
        cudaFree(sorted);
        cudaFree(offsets);
        check(st, sorter_);
        return out;
    }
    void cleanup() {
        if (records_) cudaFree(records_);
        if (sorter_) pg_ctx_destroy(sorter_);
        records_ = nullptr;
        sorter_ = nullptr;
    }

private:
    uint32_t region_count_ = 0;
    uint64_t slots_ = 0;
    pg_directional_data *records_ = nullptr;
    pg_ctx *sorter_ = nullptr;
    cudaStream_t stream_ = nullptr;
};

// ---------------------------------------------------------------------------
// PathGuiding(splitCount, sceneAabb, useParallaxCompensation)
// ---------------------------------------------------------------------------
class PathGuiding {
public:
    PathGuiding() = default;
    // splitAndMerge: the post-fit split and merge of mixture components
    // (src/PathGuiding.h:124, on by default there too).  maxRegions: room for
    // regions created by setSplitRegions (default: no more than splitCount gives).
    PathGuiding(uint32_t splitCount, const Aabb &sceneAabb, bool useParallaxCompensation,
                cudaStream_t stream = nullptr, uint32_t numInitialComponents = 8, bool splitAndMerge = true,
                uint32_t maxRegions = 0)
        : stream_(stream) {
        pg_fit_config cfg;
        pg_default_fit_config(&cfg);
        cfg.use_parallax = useParallaxCompensation ? 1u : 0u;
        cfg.num_initial_components = numInitialComponents;
        if (splitCount > 24) throw Error(PG_ERR_ARG, "splitCount must be <= 24");
        const uint32_t cap = maxRegions > (1u << splitCount) ? maxRegions : (1u << splitCount);
        check(pg_ctx_create(&cfg, cap, 0, &ctx_));
        float box[6];
        sceneAabb.to_array(box);
        check(pg_set_regions(ctx_, splitCount, box, stream_), ctx_);
        if (splitAndMerge) {
            pg_split_merge_config sm;
            pg_default_split_merge_config(&sm);
            check(pg_set_split_merge(ctx_, &sm), ctx_);
        }
    }
    PathGuiding(PathGuiding &&o) noexcept { *this = std::move(o); }
    PathGuiding &operator=(PathGuiding &&o) noexcept {
        std::swap(ctx_, o.ctx_);
        std::swap(stream_, o.stream_);
        return *this;
    }
    PathGuiding(const PathGuiding &) = delete;
    PathGuiding &operator=(const PathGuiding &) = delete;
    ~PathGuiding() { cleanup(); }

    // splitRegions / samplesForRegionSplit (src/PathGuiding.h:121-122; off by
    // default there and here).
    void setSplitRegions(bool splitRegions, float samplesForRegionSplit = 10000.0f) {
        pg_region_split_config rs{splitRegions ? 1u : 0u, samplesForRegionSplit};
        check(pg_set_region_split(ctx_, &rs), ctx_);
    }
    // update (src/PathGuiding.cpp:276-312): bucket the collector's records by
    // region, parallax pre-pass, fit (first pass) or stepwise update, split
    // and merge, lobe distances, the region split check and VMM_Theta packing,
    // all on the device and stream-ordered (a region split check synchronises).
    // Returns whether regions were split (the reference's signal to rebind
    // the tracer's buffers; the collector then needs setRegionCount).
    bool update(SampleCollector &sampleCollector) {
        const uint32_t before = getRegionCount();
        check(pg_update(ctx_, sampleCollector.deviceRecords(), sampleCollector.slotCount(), nullptr, stream_), ctx_);
        return getRegionCount() != before;
    }
    uint32_t getRegionCount() const {
        uint32_t n = 0;
        check(pg_region_count(ctx_, &n), ctx_);
        return n;
    }
    // Waits for the stream and reports device-side failures (non-finite fits,
    // bounded waits that ran out).
    void synchronize() { check(pg_sync_status(ctx_, stream_), ctx_); }
    pg_ctx *context() const { return ctx_; }
    void cleanup() {
        if (ctx_) pg_ctx_destroy(ctx_);
        ctx_ = nullptr;
    }

private:
    pg_ctx *ctx_ = nullptr;
    cudaStream_t stream_ = nullptr;
};

// ---------------------------------------------------------------------------
// Tracer: the wavefront renderer over a SceneLoader's scene.
// ---------------------------------------------------------------------------
class Tracer {
public:
    explicit Tracer(const SceneLoader &scene, cudaStream_t stream = nullptr) : scene_(&scene), stream_(stream) {}
    // Adds params.spp samples per pixel of radiance to image (device,
    // width * height * 3 floats); guiding and recording as params asks.
    pg_render_stats render(const pg_render_params &params, float *image, PathGuiding *guiding = nullptr,
                           SampleCollector *collector = nullptr, bool wait_for_stats = false) {
        pg_render_stats st{};
        check(pg_render(scene_->handle(), &params, guiding ? guiding->context() : nullptr, image,
                        collector ? collector->deviceRecords() : nullptr, wait_for_stats ? &st : nullptr, stream_));
        return st;
    }

private:
    const SceneLoader *scene_;
    cudaStream_t stream_;
};

// ---------------------------------------------------------------------------
// IrradianceCache(maxCaches) (src/IrradianceCache.h:33-64): the scene's
// irradiance cache with the reference's push-constant defaults; entries are
// made and updated by renders with PG_RENDER_IRRADIANCE_CACHE.
// ---------------------------------------------------------------------------
class IrradianceCache {
public:
    IrradianceCache(const SceneLoader &scene, uint32_t maxCaches, bool onGlossy = false) : scene_(&scene) {
        pg_default_irradiance_cache_config(&cfg_);
        cfg_.capacity = maxCaches;
        cfg_.use_on_glossy = onGlossy ? 1u : 0u;
        check(pg_scene_set_irradiance_cache(scene.handle(), &cfg_));
    }
    uint32_t size() const {
        uint32_t n = 0;
        check(pg_scene_get_irradiance_cache(scene_->handle(), nullptr, 0, &n));
        return n;
    }
    std::vector<pg_ic_entry> entries() const {
        std::vector<pg_ic_entry> out(size());
        uint32_t n = 0;
        check(pg_scene_get_irradiance_cache(scene_->handle(), out.data(), (uint32_t)out.size(), &n));
        out.resize(n);
        return out;
    }
    const pg_irradiance_cache_config &config() const { return cfg_; }

private:
    const SceneLoader *scene_;
    pg_irradiance_cache_config cfg_{};
};

inline pg_render_params render_params(uint32_t spp, uint32_t max_depth, uint32_t seed, bool guiding = false,
                                      bool record = false, float guiding_prob = 0.5f) {
    pg_render_params p{};
    p.spp = spp;
    p.max_depth = max_depth;
    p.seed = seed;
    p.use_nee = 1;
    p.use_mis = 1;
    p.use_guiding = guiding ? 1u : 0u;
    p.guiding_prob = guiding_prob;
    p.record_samples = record ? 1u : 0u;
    return p;
}

}  // namespace pg

#endif
