// pg_render - headless driver of the guided path tracer, through the C++
// facades of pathguiding.hpp.
//
// Arguments follow the reference's main (src/main.cpp:8-33): WIDTH HEIGHT
// IC_SIZE GUIDING_SPLITS SCENE.  IC_SIZE is the irradiance cache's capacity,
// used with --irradiance-cache or --adrrs.  SCENE is a Mitsuba-XML file, or
// "cornell" / "plates" for the procedural scenes.  The frame loop restates RayTracingApp's guiding phase
// (src/RayTracingApp.cpp:125-157): numGuidingOptimizations training frames
// that record samples and call PathGuiding::update, each accumulated into the
// image, then the remaining samples with guiding.  The mean radiance is
// written as a PFM image and a one-line JSON summary goes to stdout.
//
//   pg_render 1280 720 0 12 cornell --spp 64 --train 1,2,4,8,16,32 --out img.pfm
//
// Options: --spp N (final guided samples, default 64), --train LIST (training
// samples per frame, default 1,2,4,8,16,32), --depth N (10), --seed N (1),
// --prob P (guiding probability 0.5), --no-guiding (plain NEE + MIS with the
// same total samples), --no-parallax, --no-split-merge, --out FILE,
// --irradiance-cache (the cache's prepare frames, then every frame queries
// and grows it), --adrrs (prepare frames on glossy surfaces too, the
// estimate frame, then adjoint-driven roulette and splitting,
// src/RayTracingApp.cpp:1129-1170, 1206-1217), --prepare-frames N (50).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "pathguiding.hpp"

namespace {

std::vector<uint32_t> parse_list(const char *s) {
    std::vector<uint32_t> v;
    const char *p = s;
    while (*p) {
        char *end = nullptr;
        const unsigned long x = strtoul(p, &end, 10);
        if (end == p) break;
        v.push_back((uint32_t)x);
        p = *end == ',' ? end + 1 : end;
    }
    return v;
}

bool write_pfm(const std::string &path, const std::vector<float> &rgb, uint32_t w, uint32_t h) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    fprintf(f, "PF\n%u %u\n-1.0\n", w, h);
    for (uint32_t y = h; y-- > 0;)  // PFM stores the bottom row first
        if (fwrite(&rgb[(size_t)y * w * 3], sizeof(float), (size_t)w * 3, f) != (size_t)w * 3) {
            fclose(f);
            return false;
        }
    return fclose(f) == 0;
}

int usage() {
    fprintf(stderr, "Required parameters: WIDTH HEIGHT IC_SIZE GUIDING_SPLITS SCENE [--spp N] [--train LIST] "
                    "[--depth N] [--seed N] [--prob P] [--no-guiding] [--no-parallax] [--no-split-merge] "
                    "[--split-regions SAMPLES] [--out FILE] [--irradiance-cache] [--adrrs] [--prepare-frames N]\n");
    return EXIT_FAILURE;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 6) return usage();
    const uint32_t W = (uint32_t)strtoul(argv[1], nullptr, 10), H = (uint32_t)strtoul(argv[2], nullptr, 10);
    const uint32_t splits = (uint32_t)strtoul(argv[4], nullptr, 10);
    const std::string scene_arg = argv[5];
    uint32_t spp = 64, depth = 10, seed = 1;
    float prob = 0.5f;
    bool guiding = true, parallax = true, split_merge = true, use_ic = false, adrrs = false;
    uint32_t prepare_frames = 50;  // irradianceCachePrepareFrames (src/RayTracingApp.h:175)
    float split_regions = 0.0f;  // samplesForRegionSplit; 0: regions are not split (the reference's default)
    std::vector<uint32_t> train = {1, 2, 4, 8, 16, 32};
    std::string out;
    for (int i = 6; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> const char * { return i + 1 < argc ? argv[++i] : ""; };
        if (a == "--spp") spp = (uint32_t)strtoul(next(), nullptr, 10);
        else if (a == "--train") train = parse_list(next());
        else if (a == "--depth") depth = (uint32_t)strtoul(next(), nullptr, 10);
        else if (a == "--seed") seed = (uint32_t)strtoul(next(), nullptr, 10);
        else if (a == "--prob") prob = strtof(next(), nullptr);
        else if (a == "--no-guiding") guiding = false;
        else if (a == "--no-parallax") parallax = false;
        else if (a == "--no-split-merge") split_merge = false;
        else if (a == "--split-regions") split_regions = strtof(next(), nullptr);
        else if (a == "--out") out = next();
        else if (a == "--irradiance-cache") use_ic = true;
        else if (a == "--adrrs") adrrs = true;
        else if (a == "--prepare-frames") prepare_frames = (uint32_t)strtoul(next(), nullptr, 10);
        else return usage();
    }
    if (W == 0 || H == 0) return usage();
    const uint32_t ic_size = (uint32_t)strtoul(argv[3], nullptr, 10);
    if ((use_ic || adrrs) && ic_size == 0) {
        fprintf(stderr, "--irradiance-cache and --adrrs need IC_SIZE > 0\n");
        return EXIT_FAILURE;
    }
    try {
        pg::SceneLoader scene = scene_arg == "cornell"  ? pg::SceneLoader::cornell(W, H)
                                : scene_arg == "plates" ? pg::SceneLoader::plates(W, H)
                                                        : pg::SceneLoader(scene_arg, W, H);
        cudaStream_t stream;
        pg::check_cuda(cudaStreamCreate(&stream), "stream");
        float *image = nullptr;
        const size_t n = (size_t)W * H * 3;
        pg::check_cuda(cudaMalloc(&image, n * sizeof(float)), "image");
        pg::check_cuda(cudaMemsetAsync(image, 0, n * sizeof(float), stream), "image clear");
        pg::Tracer tracer(scene, stream);
        // irradiance cache: prepare frames of one sample per pixel into a scratch image
        // (isIrradiancePrepareFrame), for ADRRS on glossy surfaces too, then the estimate
        uint32_t flags = 0, ic_entries = 0;
        float *estimate = nullptr;
        std::unique_ptr<pg::IrradianceCache> ic;
        if (use_ic || adrrs) {
            ic.reset(new pg::IrradianceCache(scene, ic_size, adrrs));
            float *scratch = nullptr;
            pg::check_cuda(cudaMalloc(&scratch, n * sizeof(float)), "scratch image");
            for (uint32_t f = 0; f < prepare_frames; ++f) {
                pg_render_params p = pg::render_params(1, depth, seed + 7777u * (f + 1));
                p.flags = PG_RENDER_IRRADIANCE_CACHE;
                tracer.render(p, scratch);
            }
            if (adrrs) {
                // setEstimateRTSettings: 16 samples, the cache used, maxDepth 1
                pg::check_cuda(cudaMemsetAsync(scratch, 0, n * sizeof(float), stream), "estimate clear");
                pg_render_params p = pg::render_params(16, 3, seed + 99u);
                p.flags = PG_RENDER_IRRADIANCE_CACHE | PG_RENDER_IC_FROZEN;
                tracer.render(p, scratch);
                std::vector<float> est(n);
                pg::check_cuda(cudaMemcpyAsync(est.data(), scratch, n * sizeof(float), cudaMemcpyDeviceToHost, stream),
                               "estimate download");
                pg::check_cuda(cudaStreamSynchronize(stream), "estimate");
                for (float &v : est) v /= 16.0f;
                pg::check_cuda(cudaMalloc(&estimate, n * sizeof(float)), "estimate");
                pg::check_cuda(cudaMemcpy(estimate, est.data(), n * sizeof(float), cudaMemcpyHostToDevice),
                               "estimate upload");
                pg_adrrs_config ac{};
                ac.estimate = estimate;
                ac.s = 5.0f;
                ac.split = 1;
                pg::check(pg_scene_set_adrrs(scene.handle(), &ac));
                flags = PG_RENDER_ADRRS;
            } else {
                flags = PG_RENDER_IRRADIANCE_CACHE;
            }
            pg::check_cuda(cudaStreamSynchronize(stream), "prepare frames");
            cudaFree(scratch);
            ic_entries = ic->size();
        }
        cudaEvent_t e0, e1, e2;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventCreate(&e2);
        uint32_t total = 0;
        uint64_t sorted_records = 0, regions_with_samples = 0;
        uint32_t regions = 0;
        cudaEventRecord(e0, stream);
        if (guiding) {
            // room for 4x the initial regions when regions may split
            pg::PathGuiding pg(splits, scene.getSceneSize(), parallax, stream, 8, split_merge,
                               split_regions > 0.0f ? 4u << splits : 0u);
            if (split_regions > 0.0f) pg.setSplitRegions(true, split_regions);
            pg::SampleCollector collector(pg.getRegionCount(), W, H, stream);
            for (size_t f = 0; f < train.size(); ++f) {
                pg_render_params p = pg::render_params(train[f], depth, seed + 1000u * (uint32_t)(f + 1), f > 0, true, prob);
                p.flags = flags;
                tracer.render(p, image, &pg, &collector);
                // RayTracingApp rebuilds its buffers when update reports split regions
                if (pg.update(collector)) collector.setRegionCount(pg.getRegionCount());
                total += train[f];
            }
            regions = pg.getRegionCount();
            cudaEventRecord(e1, stream);
            pg_render_params p = pg::render_params(spp, depth, seed, true, false, prob);
            p.flags = flags;
            tracer.render(p, image, &pg);
            total += spp;
            cudaEventRecord(e2, stream);
            pg.synchronize();
            // the last training frame's records as SampleCollector::getSortedData returns them
            std::vector<uint32_t> offsets;
            const auto sorted = collector.getSortedData(offsets);
            sorted_records = sorted->size();
            for (size_t r = 0; r + 1 < offsets.size(); ++r) regions_with_samples += offsets[r + 1] > offsets[r];
        } else {
            uint32_t all = spp;
            for (uint32_t t : train) all += t;
            cudaEventRecord(e1, stream);
            pg_render_params p = pg::render_params(all, depth, seed);
            p.flags = flags;
            tracer.render(p, image);
            total = all;
            cudaEventRecord(e2, stream);
        }
        pg::check_cuda(cudaStreamSynchronize(stream), "render");
        float train_ms = 0, render_ms = 0;
        cudaEventElapsedTime(&train_ms, e0, e1);
        cudaEventElapsedTime(&render_ms, e1, e2);
        std::vector<float> rgb(n);
        pg::check_cuda(cudaMemcpy(rgb.data(), image, n * sizeof(float), cudaMemcpyDeviceToHost), "image download");
        double mean = 0.0;
        for (float &v : rgb) {
            v /= (float)total;
            mean += v;
        }
        mean /= (double)n;
        const bool exr = out.size() > 4 && out.compare(out.size() - 4, 4, ".exr") == 0;
        if (!out.empty() && exr) {
            // writeEXR (src/CommonOps.cpp:12-38): rows from the top
            if (pg_exr_write(out.c_str(), rgb.data(), W, H) != PG_OK) {
                fprintf(stderr, "cannot write %s\n", out.c_str());
                return EXIT_FAILURE;
            }
        } else if (!out.empty() && !write_pfm(out, rgb, W, H)) {
            fprintf(stderr, "cannot write %s\n", out.c_str());
            return EXIT_FAILURE;
        }
        printf("{\"scene\": \"%s\", \"width\": %u, \"height\": %u, \"guiding\": %s, \"spp\": %u, "
               "\"train_ms\": %.3f, \"render_ms\": %.3f, \"mean\": %.9g, \"sorted_records\": %llu, "
               "\"regions_with_samples\": %llu, \"regions\": %u, \"irradiance_cache_entries\": %u, \"adrrs\": %s}\n",
               scene_arg.c_str(), W, H, guiding ? "true" : "false", total, train_ms, render_ms, mean,
               (unsigned long long)sorted_records, (unsigned long long)regions_with_samples, regions, ic_entries,
               adrrs ? "true" : "false");
        cudaFree(image);
        cudaFree(estimate);
        cudaStreamDestroy(stream);
    } catch (const pg::Error &e) {
        fprintf(stderr, "pg_render: %s\n", e.what());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
