// Host-side construction of a scene's device tables from a cgpu_scene_desc:
// validation, rectangle expansion, BVH build, triangle records, materials,
// lights (area + environment distribution), camera.  cgpu_scene_upload copies
// the result to the device; the CPU check of the kernel logic uses it in
// place (host_view).
#pragma once

#include "../../include/cadise_gpu.h"
#include "bvh_build.h"
#include "scene_device.cuh"

#include <string>
#include <vector>

namespace cg {

struct HostScene {
    std::vector<Bvh4Node> nodes;
    std::vector<TriRecord> tris;
    std::vector<MaterialD> mats;
    std::vector<LightD> lights;      // area lights, then the environment light if any
    int num_area_lights = 0;
    int env_light = -1;
    int env_tex = -1;
    std::vector<float> env_marg, env_cond;
    std::vector<TextureD> textures;  // texel pointers into the caller's desc
    std::vector<float> rect_frames;  // vB, eA, eB per rectangle
    std::vector<uint32_t> prim_rank; // 8 per primitive (reference_visit_ranks)
    std::vector<float> light_cdf;    // power light cluster: num_lights + 1 CDF values; empty: uniform
    CameraD cam{};
    FilterD filter{};
    cgpu_scene_info info{};
    int wide_depth = 0;
    bool has_spheres = false;
};

// Resolves a cgpu_film_filter (defaults, derived constants); CGPU_OK or an
// error status with a message in *err.
cgpu_status resolve_filter(const cgpu_film_filter& f, FilterD* out, std::string* err);

// Returns CGPU_OK or an error status with a message in *err.  `bvh_builder`
// (optional) builds the BVH in place of the host builder.  `tie_ranks`:
// also build the reference's tie order (prim_rank, tie_order.h).
cgpu_status build_host_scene(const cgpu_scene_desc* d, HostScene* out, std::string* err,
                             BvhBuildFn bvh_builder = nullptr, void* bvh_user = nullptr, bool tie_ranks = true);

// A SceneD whose pointers are the host arrays (for running the kernel logic on the CPU).
SceneD host_view(HostScene& hs, const cgpu_scene_desc* d);

}  // namespace cg
