// Host BVH build into the 4-wide device layout (see scene_device.cuh).
#pragma once

#include "scene_device.cuh"

#include <cstdint>
#include <string>
#include <vector>

namespace cg {

struct Bvh4Result {
    std::vector<Bvh4Node> nodes;  // root at 0
    std::vector<uint32_t> order;  // leaf order -> input triangle index
    int binary_depth = 0;
    int wide_depth = 0;
};

// tri_vertices: 9 floats per triangle.  Returns false (with a message) on
// empty or oversized input.
bool build_bvh4(const float* tri_vertices, uint32_t num_tris, Bvh4Result* out, std::string* err);

// The same result from the GPU build (bvh_gpu.cu): tri_vertices in host
// memory, work on `stream`, nodes and leaf order copied back to `out`.
bool build_bvh4_gpu(const float* tri_vertices, uint32_t num_tris, cudaStream_t stream, Bvh4Result* out,
                    std::string* err);

// The host build's binned SAH on the GPU (bvh_sah_gpu.cu): same inputs and
// outputs as build_bvh4_gpu.
bool build_bvh4_gpu_sah(const float* tri_vertices, uint32_t num_tris, cudaStream_t stream, Bvh4Result* out,
                        std::string* err);

// A BVH builder the scene build can be handed instead of build_bvh4.
using BvhBuildFn = bool (*)(const float* tri_vertices, uint32_t num_tris, Bvh4Result* out, std::string* err,
                            void* user);

}  // namespace cg
