// Exact-tie order of closest hits.
//
// Where two primitives meet a ray at the same reference distance (coplanar,
// overlapping quads; a ray through an edge two triangles share), the
// reference keeps the one its BVH traversal reaches LAST: a primitive test
// accepts t == maxT (triangle.cpp:81-86, rectangle.cpp:49-75), and the
// traversal (bvhAccelerator.cpp:40-97) walks its binary tree depth first,
// the child on the near side of the node's split axis first
// (directionIsNegative[splitAxis] picks the second child first).  That order
// depends only on the tree and on the signs of the ray direction, so it is
// captured as one rank per primitive and direction octant; the closest-hit
// rule of the kernels (tie_prefers, traverse.cuh) compares ranks on an exact
// tie and reproduces the reference's answer without its tree on the device.
//
// The tree is the reference's own (bvhBuilder.cpp:59-169, :212-358): binned
// SAH over 12 buckets along the widest centroid axis, traversal cost 0.125 and
// intersection cost 1, an equal split of 2 primitives, a leaf of 1, the
// primitive boxes expanded by 0.0001 (triangle.cpp:45-52,
// rectangle.cpp:37-44, sphere.cpp:33-40) and the empty box's upper corner at
// FLT_MIN (tAabb.ipp:13-17).  Only the tree's shape is kept here.
#pragma once

#include "../../include/cadise_gpu.h"

#include <cstdint>
#include <vector>

namespace cg {

// Ranks of every primitive of `d`, 8 per primitive (primitive-major): entry
// 8 * p + o is the position of primitive p in the reference traversal's leaf
// order for rays of octant o (bit k of o set: direction component k is
// negative, -0 included).  Of two primitives hit at the same distance the
// reference keeps the higher rank.  Subtrees of large ranges are built on
// separate threads.
std::vector<uint32_t> reference_visit_ranks(const cgpu_scene_desc* d);

}  // namespace cg
