// SAH-optimal conversion of a binary BVH into 4-wide nodes, shared by the host
// build (bvh_build.cpp) and the GPU builds (bvh_gpu.cu, bvh_sah_gpu.cu).
//
// The dynamic programme of Ylitie, Karras & Laine, "Efficient Incoherent Ray
// Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017), for width 4:
// cost[i - 1] is the least SAH cost of a binary subtree that may fill at most
// i child slots of its parent - as one leaf (at most kMaxLeafTris triangles),
// as one inner wide node, or (i > 1) split between its two children's
// subtrees.  Node and triangle costs are 1 : 1 (0.3 or 0.5 per triangle made
// the trees trace slower).
#pragma once

#include "common.cuh"
#include "scene_device.cuh"

namespace cg {

constexpr float kWideCostNode = 1.0f;  // one wide-node visit (four box tests)
constexpr float kWideCostTri = 1.0f;   // one triangle test
constexpr float kWideInf = 3.402823466e38f;

struct WideCost {
    float cost[4];
    uint32_t split;  // byte i - 1 (i > 1): slots of the left child when distributing, 0 = i - 1 slots do
    uint32_t leaf;   // one slot: a leaf (else an inner wide node)
};

// A binary leaf (it cannot be split further).
CG_HD WideCost wide_cost_leaf(float half_area, uint32_t count) {
    const float c = count <= kMaxLeafTris ? half_area * float(count) * kWideCostTri : kWideInf;
    WideCost w;
    for (int i = 0; i < 4; ++i) w.cost[i] = c;
    w.split = 0;
    w.leaf = 1;
    return w;
}

// An inner binary node from its children's costs.
CG_HD WideCost wide_cost_inner(float half_area, uint32_t count, const WideCost& L, const WideCost& R) {
    const float leaf_cost = count <= kMaxLeafTris ? half_area * float(count) * kWideCostTri : kWideInf;
    float dist[5];
    uint32_t arg[5];
    for (int j = 2; j <= 4; ++j) {
        dist[j] = kWideInf;
        arg[j] = 1;
        for (int k = 1; k < j; ++k) {
            const float c = L.cost[k - 1] + R.cost[j - k - 1];
            if (c < dist[j]) {
                dist[j] = c;
                arg[j] = uint32_t(k);
            }
        }
    }
    const float inner = half_area * kWideCostNode + dist[4];
    WideCost w;
    w.leaf = leaf_cost <= inner ? 1u : 0u;
    w.cost[0] = w.leaf ? leaf_cost : inner;
    w.split = 0;
    for (int i = 2; i <= 4; ++i) {
        if (dist[i] < w.cost[i - 2]) {
            w.cost[i - 1] = dist[i];
            w.split |= arg[i] << (8 * (i - 1));
        } else {
            w.cost[i - 1] = w.cost[i - 2];
        }
    }
    return w;
}

// The binary nodes that fill the four slots of the wide node of an inner
// binary node with children l and r.  cost(x) gives node x's WideCost,
// left(x) / right(x) its children.  Returns the slot count.
template <typename Cost, typename Left, typename Right>
CG_HD int wide_slots(uint32_t l, uint32_t r, Cost&& cost, Left&& left, Right&& right, uint32_t (&kids)[4]) {
    int nk = 0;
    const WideCost Lc = cost(l), Rc = cost(r);
    uint32_t best_k = 1;
    float best = kWideInf;
    for (uint32_t k = 1; k < 4; ++k) {
        const float c = Lc.cost[k - 1] + Rc.cost[4 - k - 1];
        if (c < best) {
            best = c;
            best_k = k;
        }
    }
    // (node, slots) still to place; at most four are open at once
    uint32_t st_n[8], st_i[8];
    int sp = 0;
    st_n[sp] = r; st_i[sp++] = 4 - best_k;
    st_n[sp] = l; st_i[sp++] = best_k;
    while (sp > 0 && nk < 4) {
        --sp;
        const uint32_t x = st_n[sp];
        uint32_t slots = st_i[sp];
        const uint32_t sx = cost(x).split;
        while (slots > 1 && ((sx >> (8 * (slots - 1))) & 255u) == 0u) --slots;  // fewer slots do as well
        if (slots == 1) {
            kids[nk++] = x;
            continue;
        }
        const uint32_t q = (sx >> (8 * (slots - 1))) & 255u;
        if (sp + 2 > 8) break;  // cannot happen: at most four entries are open
        st_n[sp] = right(x); st_i[sp++] = slots - q;
        st_n[sp] = left(x); st_i[sp++] = q;
    }
    return nk;
}

}  // namespace cg
