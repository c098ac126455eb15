// GPU BVH build: PLOC clustering into a binary tree, SAH leaf choice,
// collapse into the 4-wide layout of scene_device.cuh.
//
// Replaces BvhBuilder (source/core/intersector/accelerator/bvh/bvhBuilder.cpp:18-358,
// serial recursive SAH) where set-up time matters more than trace speed: the
// host builder's (bvh_build.cpp) binned-SAH tree traces 12-25 % faster, so
// CGPU_BVH_BUILDER_AUTO picks this build only for scenes with many primitives
// per path sample.  Method: Meister & Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction"
// (IEEE TVCG 2018):
//   1. triangle boxes and the bounds of their centroids;
//   2. 63-bit Morton codes of the centroids, LSD radix sort (8 passes of 8
//      bits, stable block ranking with warp match);
//   3. clusters in Morton order; per iteration every cluster finds, within 64
//      positions either side, the one whose merged box has the smallest
//      surface area (ties to the lower position); mutual nearest neighbours
//      merge into a new binary node; prefix sums give the new node ids and
//      compact the cluster array, so the build is deterministic;
//   4. bottom-up (one thread per triangle, the second arrival at a node goes
//      on): triangle counts and the SAH-optimal 4-wide collapse costs of the
//      host builder (wide_costs in bvh_build.cpp);
//   5. top-down, one level of the 4-wide tree per launch: each wide node
//      takes the binary subtrees those costs assign to its four slots; leaf
//      subtrees (at most 8 triangles) become leaf entries whose triangles are
//      laid out contiguously in DFS order.
// No kernel waits on another thread: every loop is bounded by the data.
#include "bvh_build.h"
#include "radix.cuh"
#include "wide_collapse.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace cg {
namespace {

constexpr int kBlock = kRadixBlock;
// PLOC search radius.  On the 1,024,018-triangle icosphere field closest-hit
// rays visit 21.9 / 21.7 / 21.0 wide nodes with radius 16 / 32 / 64 (the
// host SAH tree: 18.9) for 9.5 / 9.9 / 10.4 ms of build.
constexpr int kRadius = 64;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kMaxIterations = 1 << 16;

__device__ __forceinline__ uint32_t order_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_value(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}
__device__ __forceinline__ float4 min4(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 max4(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f);
}

// ------------------------------------------------------------ boxes, codes --
__global__ void k_tri_boxes(const float* tv, uint32_t n, float4* lo, float4* hi, uint32_t* cb) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* v = tv + 9 * size_t(i);
        float l[3], h[3];
        for (int k = 0; k < 3; ++k) {
            l[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
            h[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
            const float c = 0.5f * (l[k] + h[k]);
            mn[k] = fminf(mn[k], c);
            mx[k] = fmaxf(mx[k], c);
        }
        lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
        hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
    }
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(cb + k, order_key(mn[k]));
            atomicMax(cb + 3 + k, order_key(mx[k]));
        }
    }
}

__device__ __forceinline__ uint64_t spread21(uint32_t v) {
    uint64_t x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* lo, const float4* hi, uint32_t n, const uint32_t* cb, uint64_t* keys,
                         uint32_t* vals) {
    const float mn[3] = {key_value(cb[0]), key_value(cb[1]), key_value(cb[2])};
    const float mx[3] = {key_value(cb[3]), key_value(cb[4]), key_value(cb[5])};
    float inv[3];
    for (int k = 0; k < 3; ++k) inv[k] = mx[k] > mn[k] ? 1.0f / (mx[k] - mn[k]) : 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = lo[i], h = hi[i];
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float u = fminf(fmaxf((c[k] - mn[k]) * inv[k], 0.0f), 1.0f);
            q[k] = min(uint32_t(u * 2097152.0f), 2097151u);
        }
        keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
        vals[i] = i;
    }
}

// ---------------------------------------------------------------------- PLOC --
// Cluster record: lo.w = binary node id (bits), hi.w unused.  Binary node:
// lo.w = left child, hi.w = right child (kNone for a triangle).
__global__ void k_ploc_init(const float4* tlo, const float4* thi, const uint32_t* vals, uint32_t n, float4* clo,
                            float4* chi, float4* blo, float4* bhi) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = tlo[vals[i]], h = thi[vals[i]];
        clo[i] = make_float4(l.x, l.y, l.z, __uint_as_float(i));
        chi[i] = make_float4(h.x, h.y, h.z, 0.0f);
        blo[i] = make_float4(l.x, l.y, l.z, __uint_as_float(kNone));
        bhi[i] = make_float4(h.x, h.y, h.z, __uint_as_float(kNone));
    }
}

__global__ void k_ploc_nn(const float4* clo, const float4* chi, uint32_t m, uint32_t* nn) {
    __shared__ float4 slo[kBlock + 2 * kRadius], shi[kBlock + 2 * kRadius];
    const int64_t base = int64_t(blockIdx.x) * kBlock;
    for (int j = threadIdx.x; j < kBlock + 2 * kRadius; j += kBlock) {
        const int64_t g = base - kRadius + j;
        if (g >= 0 && g < int64_t(m)) {
            slo[j] = clo[g];
            shi[j] = chi[g];
        }
    }
    __syncthreads();
    const int64_t i = base + threadIdx.x;
    if (i >= int64_t(m)) return;
    const int si = threadIdx.x + kRadius;
    const float4 a = slo[si], b = shi[si];
    float best = INFINITY;
    uint32_t bj = kNone;
    for (int o = -kRadius; o <= kRadius; ++o) {
        const int64_t j = i + o;
        if (o == 0 || j < 0 || j >= int64_t(m)) continue;
        const float c = half_area(min4(a, slo[si + o]), max4(b, shi[si + o]));
        if (c < best) {
            best = c;
            bj = uint32_t(j);
        }
    }
    nn[i] = bj == kNone ? uint32_t(i) : bj;
}

// f = 1 where cluster i merges as the lower of a mutual pair; k = 1 where it
// survives (unmerged, or the lower of a pair, which takes the new node).
__global__ void k_ploc_flags(const uint32_t* nn, uint32_t m, uint32_t* f, uint32_t* k) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint32_t j = nn[i];
        const bool mutual = j != i && nn[j] == i;
        f[i] = (mutual && i < j) ? 1u : 0u;
        k[i] = (mutual && i > j) ? 0u : 1u;
    }
}

__global__ void k_ploc_merge(const float4* clo, const float4* chi, const uint32_t* nn, uint32_t m, const uint32_t* fs,
                             const uint32_t* ks, uint32_t node_base, float4* olo, float4* ohi, float4* blo, float4* bhi,
                             uint32_t* parent, uint32_t* totals) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint32_t j = nn[i];
        const bool mutual = j != i && nn[j] == i;
        const bool merge = mutual && i < j, keep = !(mutual && i > j);
        if (merge) {
            const uint32_t id = node_base + fs[i];
            const float4 a0 = clo[i], a1 = chi[i], b0 = clo[j], b1 = chi[j];
            const float4 l = min4(a0, b0), h = max4(a1, b1);
            const uint32_t na = __float_as_uint(a0.w), nb = __float_as_uint(b0.w);
            blo[id] = make_float4(l.x, l.y, l.z, __uint_as_float(na));
            bhi[id] = make_float4(h.x, h.y, h.z, __uint_as_float(nb));
            parent[na] = id;
            parent[nb] = id;
            olo[ks[i]] = make_float4(l.x, l.y, l.z, __uint_as_float(id));
            ohi[ks[i]] = make_float4(h.x, h.y, h.z, 0.0f);
        } else if (keep) {
            olo[ks[i]] = clo[i];
            ohi[ks[i]] = chi[i];
        }
        if (i == m - 1) {
            totals[0] = fs[i] + (merge ? 1u : 0u);
            totals[1] = ks[i] + (keep ? 1u : 0u);
        }
    }
}

// ------------------------------------------------- bottom-up collapse costs --
// The SAH-optimal 4-wide collapse costs (wide_collapse.cuh) of every binary
// node, from the triangle leaves up: the second thread to reach a node
// computes it from its two children.
__global__ void k_bottom_up(uint32_t n, uint32_t root, const uint32_t* parent, const float4* blo, const float4* bhi,
                            uint32_t* count, WideCost* cost, uint32_t* visits) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        count[i] = 1;
        cost[i] = wide_cost_leaf(half_area(blo[i], bhi[i]), 1);
        uint32_t node = i;
        // each step climbs one level: at most the tree's node count
        for (uint32_t guard = 0; node != root && guard < 2 * n; ++guard) {
            const uint32_t p = parent[node];
            __threadfence();
            if (atomicAdd(visits + p, 1u) == 0u) break;  // the sibling's thread continues
            __threadfence();
            const float4 pl = blo[p], ph = bhi[p];
            const uint32_t l = __float_as_uint(pl.w), r = __float_as_uint(ph.w);
            const uint32_t c = __ldcg(count + l) + __ldcg(count + r);
            WideCost L, R;
            for (int k = 0; k < 4; ++k) {
                L.cost[k] = __ldcg(&cost[l].cost[k]);
                R.cost[k] = __ldcg(&cost[r].cost[k]);
            }
            L.split = __ldcg(&cost[l].split);
            R.split = __ldcg(&cost[r].split);
            L.leaf = R.leaf = 0;
            count[p] = c;
            cost[p] = wide_cost_inner(half_area(pl, ph), c, L, R);
            node = p;
        }
    }
}

// ------------------------------------------------------- top-down collapse --
struct Item {
    uint32_t bnode, wide, offset;
};

__global__ void k_collapse_select(const Item* items, uint32_t ni, const float4* blo, const float4* bhi,
                                  const WideCost* cost, uint4* kids, uint32_t* nkids, uint32_t* inner) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        const uint32_t b = items[i].bnode;
        uint32_t k[4] = {kNone, kNone, kNone, kNone};
        int nk = 0;
        if (cost[b].leaf) {
            k[nk++] = b;  // a root that is one leaf
        } else {
            nk = wide_slots(
                __float_as_uint(blo[b].w), __float_as_uint(bhi[b].w), [&](uint32_t x) { return cost[x]; },
                [&](uint32_t x) { return __float_as_uint(blo[x].w); }, [&](uint32_t x) { return __float_as_uint(bhi[x].w); },
                k);
        }
        uint32_t in = 0;
        for (int j = 0; j < nk; ++j) in += cost[k[j]].leaf ? 0u : 1u;
        kids[i] = make_uint4(k[0], k[1], k[2], k[3]);
        nkids[i] = uint32_t(nk);
        inner[i] = in;
    }
}

__global__ void k_collapse_emit(const Item* items, uint32_t ni, const uint4* kids, const uint32_t* nkids,
                                const uint32_t* slots, uint32_t wide_base, Item* next, Bvh4Node* nodes,
                                const uint32_t* count, const WideCost* cost, const float4* blo, const float4* bhi,
                                const uint32_t* vals, uint32_t n, uint32_t* order) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        const Item it = items[i];
        const uint4 k4 = kids[i];
        const uint32_t k[4] = {k4.x, k4.y, k4.z, k4.w};
        const int nk = int(nkids[i]);
        uint32_t off = it.offset, slot = slots[i];
        float lo[4][3] = {}, hi[4][3] = {};
        uint32_t child[4] = {0, 0, 0, 0};
        for (int j = 0; j < nk; ++j) {
            const uint32_t c = k[j];
            const float4 l = blo[c], h = bhi[c];
            lo[j][0] = l.x; lo[j][1] = l.y; lo[j][2] = l.z;
            hi[j][0] = h.x; hi[j][1] = h.y; hi[j][2] = h.z;
            const uint32_t cnt = count[c];
            if (cost[c].leaf) {
                child[j] = make_leaf(off, cnt);
                // the subtree's triangles (at most kMaxLeafTris) in DFS order
                uint32_t stack[2 * kMaxLeafTris], sp = 0, w = off;
                stack[sp++] = c;
                while (sp > 0 && w < off + cnt) {
                    const uint32_t x = stack[--sp];
                    if (x < n) {
                        order[w++] = vals[x];
                    } else if (sp + 2 <= 2 * kMaxLeafTris) {
                        stack[sp++] = __float_as_uint(bhi[x].w);
                        stack[sp++] = __float_as_uint(blo[x].w);
                    }
                }
            } else {
                child[j] = wide_base + slot;
                next[slot] = Item{c, wide_base + slot, off};
                ++slot;
            }
            off += cnt;
        }
        Bvh4Node wn;
        quantize_node(lo, hi, child, nk, &wn);
        nodes[it.wide] = wn;
    }
}

// ---------------------------------------------------------------- host side --
struct Pool {
    std::vector<void*> blocks;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* get(size_t count) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err == cudaSuccess) blocks.push_back(p);
        return static_cast<T*>(p);
    }
    ~Pool() {
        for (void* p : blocks) cudaFree(p);
    }
};

int grid_of(uint64_t work, int block = kBlock) {
    return int(std::max<uint64_t>(1, std::min<uint64_t>((work + block - 1) / block, 1u << 20)));
}

}  // namespace

bool build_bvh4_gpu(const float* tri_vertices, uint32_t n, cudaStream_t s, Bvh4Result* out, std::string* err) {
    out->nodes.clear();
    out->order.clear();
    if (n == 0) {
        *err = "scene has no triangles";
        return false;
    }
    if (n > kMaxTriSlots || n > 0x7FFFFFFFu / 2) {
        *err = "too many triangles for the 28-bit leaf encoding";
        return false;
    }
    Pool P;
    const uint32_t nb = radix_tiles(n);
    float* tv = P.get<float>(size_t(n) * 9);
    float4* tlo = P.get<float4>(n);
    float4* thi = P.get<float4>(n);
    uint32_t* cb = P.get<uint32_t>(8);
    uint64_t* keys[2] = {P.get<uint64_t>(n), P.get<uint64_t>(n)};
    uint32_t* vals[2] = {P.get<uint32_t>(n), P.get<uint32_t>(n)};
    uint32_t* hist = P.get<uint32_t>(size_t(nb) * 256);
    uint32_t* sums = P.get<uint32_t>(scan_scratch(std::max<uint32_t>(n, nb * 256)));
    float4* clo[2] = {P.get<float4>(n), P.get<float4>(n)};
    float4* chi[2] = {P.get<float4>(n), P.get<float4>(n)};
    uint32_t* nn = P.get<uint32_t>(n);
    uint32_t* fs = P.get<uint32_t>(n);
    uint32_t* ks = P.get<uint32_t>(n);
    uint32_t* totals = P.get<uint32_t>(2);
    const size_t nnodes = size_t(2) * n - 1;
    float4* blo = P.get<float4>(nnodes);
    float4* bhi = P.get<float4>(nnodes);
    uint32_t* parent = P.get<uint32_t>(nnodes);
    uint32_t* count = P.get<uint32_t>(nnodes);
    WideCost* cost = P.get<WideCost>(nnodes);
    uint32_t* visits = P.get<uint32_t>(nnodes);
    Item* items[2] = {P.get<Item>(n), P.get<Item>(n)};
    uint4* kids = P.get<uint4>(n);
    uint32_t* nkids = P.get<uint32_t>(n);
    uint32_t* inner = P.get<uint32_t>(n);
    Bvh4Node* nodes = P.get<Bvh4Node>(n);
    uint32_t* order = P.get<uint32_t>(n);
    if (P.err != cudaSuccess) {
        *err = std::string("GPU BVH build: ") + cudaGetErrorString(P.err);
        return false;
    }
    auto fail_cuda = [&](const char* what) {
        const cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) return false;
        *err = std::string("GPU BVH build (") + what + "): " + cudaGetErrorString(e);
        return true;
    };
    cudaMemcpyAsync(tv, tri_vertices, size_t(n) * 9 * sizeof(float), cudaMemcpyHostToDevice, s);
    const uint32_t cb_init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
    cudaMemcpyAsync(cb, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, s);
    k_tri_boxes<<<grid_of(n), kBlock, 0, s>>>(tv, n, tlo, thi, cb);
    k_morton<<<grid_of(n), kBlock, 0, s>>>(tlo, thi, n, cb, keys[0], vals[0]);
    radix_sort_pairs(keys, vals, n, nullptr, nb, 8, hist, sums, s);
    if (fail_cuda("sort")) return false;
    // 8 passes: the sorted pairs are back in keys[0] / vals[0]
    k_ploc_init<<<grid_of(n), kBlock, 0, s>>>(tlo, thi, vals[0], n, clo[0], chi[0], blo, bhi);
    uint32_t m = n, node_base = n;
    int cur = 0, iterations = 0;
    while (m > 1) {
        if (++iterations > kMaxIterations) {
            *err = "GPU BVH build: clustering did not converge";
            return false;
        }
        k_ploc_nn<<<(m + kBlock - 1) / kBlock, kBlock, 0, s>>>(clo[cur], chi[cur], m, nn);
        k_ploc_flags<<<grid_of(m), kBlock, 0, s>>>(nn, m, fs, ks);
        exclusive_scan(fs, m, sums, s);
        exclusive_scan(ks, m, sums, s);
        k_ploc_merge<<<grid_of(m), kBlock, 0, s>>>(clo[cur], chi[cur], nn, m, fs, ks, node_base, clo[cur ^ 1],
                                                   chi[cur ^ 1], blo, bhi, parent, totals);
        uint32_t t[2] = {0, 0};
        cudaMemcpyAsync(t, totals, sizeof(t), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess || fail_cuda("clustering")) {
            if (err->empty()) *err = "GPU BVH build: clustering failed";
            return false;
        }
        if (t[0] == 0 || t[1] >= m) {
            *err = "GPU BVH build: no cluster pair merged";
            return false;
        }
        node_base += t[0];
        m = t[1];
        cur ^= 1;
    }
    const uint32_t root = node_base - 1;  // n == 1: the single triangle
    cudaMemsetAsync(visits, 0, nnodes * sizeof(uint32_t), s);
    k_bottom_up<<<grid_of(n), kBlock, 0, s>>>(n, root, parent, blo, bhi, count, cost, visits);
    if (fail_cuda("bottom-up")) return false;
    // top-down, one wide level per round
    const Item first{root, 0, 0};
    cudaMemcpyAsync(items[0], &first, sizeof(Item), cudaMemcpyHostToDevice, s);
    uint32_t ni = 1, wide_count = 1;
    int depth = 0, ci = 0;
    while (ni > 0) {
        ++depth;
        k_collapse_select<<<grid_of(ni), kBlock, 0, s>>>(items[ci], ni, blo, bhi, cost, kids, nkids, inner);
        uint32_t last_inner = 0;
        cudaMemcpyAsync(&last_inner, inner + (ni - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        exclusive_scan(inner, ni, sums, s);
        uint32_t last_slot = 0;
        cudaMemcpyAsync(&last_slot, inner + (ni - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        k_collapse_emit<<<grid_of(ni), kBlock, 0, s>>>(items[ci], ni, kids, nkids, inner, wide_count, items[ci ^ 1],
                                                       nodes, count, cost, blo, bhi, vals[0], n, order);
        if (cudaStreamSynchronize(s) != cudaSuccess || fail_cuda("collapse")) {
            if (err->empty()) *err = "GPU BVH build: collapse failed";
            return false;
        }
        const uint32_t next_n = last_slot + last_inner;
        if (uint64_t(wide_count) + next_n > n) {
            *err = "GPU BVH build: wide node count out of range";
            return false;
        }
        wide_count += next_n;
        ni = next_n;
        ci ^= 1;
    }
    out->nodes.resize(wide_count);
    out->order.resize(n);
    cudaMemcpyAsync(out->nodes.data(), nodes, size_t(wide_count) * sizeof(Bvh4Node), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out->order.data(), order, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || fail_cuda("download")) {
        if (err->empty()) *err = "GPU BVH build: download failed";
        return false;
    }
    out->wide_depth = depth;
    out->binary_depth = 0;
    return true;
}

}  // namespace cg
