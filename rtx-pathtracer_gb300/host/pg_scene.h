// pg_scene.h - host-side scene: triangle meshes, analytic spheres, materials,
// lights, camera, and the binned-SAH BVH the traversal kernels walk.
//
// The reference keeps the same information in SceneLoader (src/SceneLoader.h:
// 118-162: vertices, indices, materials, spheres, lights, camera) and builds
// Vulkan BLAS/TLAS from it (src/SceneLoader.cpp:1101-1194); here the
// acceleration structure is our own BVH in device memory.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "pathguide.h"

namespace pg {

// Node of the four-wide BVH: the boxes of all four children live in the
// parent, slot-major per coordinate (lo[axis][slot]), so one 128-byte fetch
// tests four boxes.  Slot i: count[i] > 0 is a leaf with triangles
// [child[i], child[i] + count[i]) of the reordered list; count[i] == 0 and
// child[i] >= 0 an inner node; child[i] < 0 an empty slot (box +inf..-inf).
struct BvhNode {
    float lo[3][4];
    float hi[3][4];
    int32_t child[4];
    int32_t count[4];
};
static_assert(sizeof(BvhNode) == 128, "BvhNode is 128 bytes");

struct SceneData {
    std::vector<float> pos;        // 3 per vertex
    std::vector<float> nrm;        // 3 per vertex (shading normals; empty = geometric)
    std::vector<uint32_t> idx;     // 3 per triangle
    std::vector<uint32_t> tri_mat; // material per triangle
    std::vector<pg_material> mats;
    std::vector<pg_sphere> spheres;
    pg_camera camera{};
    // environment map (the reference's envmap emitter): lat-long RGB, row 0 = up
    uint32_t env_w = 0, env_h = 0;
    std::vector<float> env;
    // texture coordinates: 6 floats (u, v of the three corners) per triangle,
    // v flipped as the reference flips it (src/SceneLoader.cpp:288-291)
    std::vector<float> tri_uv;
    // material textures (RGBA8, sRGB colour, linear alpha; rows from the top);
    // pg_material::texture = index + 1
    struct Texture {
        uint32_t w = 0, h = 0;
        std::vector<uint8_t> rgba;
    };
    std::vector<Texture> textures;
    // built
    std::vector<BvhNode> nodes;
    std::vector<float> tri_verts;  // 12 floats per triangle in BVH order: v0.xyz id, v1.xyz 0, v2.xyz 0
    std::vector<uint32_t> tri_order;  // BVH order -> original triangle id
    std::string error;
};

// Binned SAH build (32 bins on centroid extents, leaves of at most max_leaf
// triangles) of a binary tree, collapsed into four-wide nodes (each node
// takes its binary children and repeatedly opens the inner child with the
// largest surface area until it holds four).  Deterministic: same input, same
// tree.
void build_bvh(SceneData &s, int max_leaf = 4);

// Procedural scenes of the benchmark workloads.
void make_cornell(SceneData &s, const pg_cornell_params &p);
void make_glossy_plates(SceneData &s, const pg_plates_params &p);

// Mitsuba-XML subset (SceneLoader::parseMitsubaSceneFile,
// src/SceneLoader.cpp:329-648): sensor (lookAt, fov), bsdf
// diffuse / dielectric / conductor / roughconductor / plastic-as-diffuse,
// shape obj / sphere / rectangle / cube with toWorld transforms, area emitters.
// Returns false and sets s.error on malformed input.
bool load_mitsuba(SceneData &s, const std::string &path, uint32_t width, uint32_t height);
bool load_obj(SceneData &s, const std::string &path, const float *to_world, uint32_t material);

// Icosphere: 20 * 4^level triangles, projected on the sphere.
void add_icosphere(SceneData &s, const float center[3], float radius, int level, uint32_t material);
void add_quad(SceneData &s, const float p0[3], const float p1[3], const float p2[3], const float p3[3],
              uint32_t material);

}  // namespace pg
