// Host BVH build: binned SAH binary tree, collapsed to the 4-wide layout of
// scene_device.cuh.
//
// Replaces BvhBuilder (source/core/intersector/accelerator/bvh/bvhBuilder.cpp:18-358),
// a serial recursive SAH over 12 buckets with one primitive per leaf that
// copies its BvhBoundInfo vectors at every level.  Here: 32 bins per axis on
// all three axes, leaves of up to 4 triangles (8 when the SAH cannot split),
// in-place partition of one index array, subtrees above 32k triangles built
// on separate host threads, then an SAH-optimal collapse (wide_costs) into
// 64-byte quantized 4-wide nodes.
#include "bvh_build.h"
#include "wide_collapse.cuh"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>

namespace cg {
namespace {

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int k = 0; k < 3; ++k) { lo[k] = FLT_MAX; hi[k] = -FLT_MAX; }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    float half_area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
        return dx * dy + dy * dz + dz * dx;
    }
};

// Every field is written by Builder::build: no initialisers, so the node
// array (2 n entries) is allocated without being filled first.
struct BinNode {
    Box box;
    int left, right;
    uint32_t first, count;  // leaf when left < 0
};

// A triangle as the build moves it: its box, its centroid and its index.
// The partition moves these records themselves, so the passes over a node
// read memory in order instead of through an index.
struct BuildPrim {
    Box box;
    float c[3];
    uint32_t t;
};

constexpr int kBins = 32;
constexpr uint32_t kLeafTarget = 4;
constexpr uint32_t kParallelMin = 32768;
constexpr uint32_t kParallelBinMin = 262144;  // nodes from this size bin on several threads
constexpr uint32_t kMaxChunks = 64;

struct Builder {
    BuildPrim* prims;
    BinNode* nodes;
    std::atomic<int> next_node{0};
    std::atomic<int> threads_live{0};
    int max_threads;
    int hw_threads = 1;
    std::atomic<int> max_depth{0};

    int alloc() { return next_node.fetch_add(1); }

    // Runs fn(chunk_begin, chunk_end, chunk) over [begin, end) in `chunks` pieces, one host thread each.
    template <typename F>
    static void for_chunks(uint32_t begin, uint32_t end, int chunks, F&& fn) {
        if (chunks <= 1) {
            fn(begin, end, 0);
            return;
        }
        const uint32_t n = end - begin;
        std::vector<std::thread> pool;
        for (int c = 1; c < chunks; ++c)
            pool.emplace_back([&, c]() {
                fn(begin + uint32_t(uint64_t(n) * c / chunks), begin + uint32_t(uint64_t(n) * (c + 1) / chunks), c);
            });
        fn(begin, begin + uint32_t(uint64_t(n) / chunks), 0);
        for (auto& t : pool) t.join();
    }

    void build(int ni, uint32_t begin, uint32_t end, int depth) {
        BinNode& node = nodes[ni];
        const uint32_t n = end - begin;
        // large nodes (the top of the tree, where few subtree threads run yet) bin on several host
        // threads; min / max and counts do not depend on the split, so the tree is the same
        const int chunks =
            n >= kParallelBinMin ? int(std::min<uint32_t>({uint32_t(hw_threads), n / (kParallelBinMin / 4), kMaxChunks}))
                                 : 1;
        Box cb_box[kMaxChunks], cb_cbox[kMaxChunks];
        for_chunks(begin, end, chunks, [&](uint32_t b0, uint32_t b1, int c) {
            Box bx, cx;
            bx.reset();
            cx.reset();
            for (uint32_t i = b0; i < b1; ++i) {
                bx.grow(prims[i].box);
                cx.grow(prims[i].c);
            }
            cb_box[c] = bx;
            cb_cbox[c] = cx;
        });
        Box box, cbox;
        box.reset();
        cbox.reset();
        for (int c = 0; c < chunks; ++c) {
            box.grow(cb_box[c]);
            cbox.grow(cb_cbox[c]);
        }
        node.box = box;
        int d = max_depth.load();
        while (depth > d && !max_depth.compare_exchange_weak(d, depth)) {
        }
        auto make_leaf = [&]() {
            node.left = node.right = -1;
            node.first = begin;
            node.count = n;
        };
        if (n <= 1) return make_leaf();
        // binned SAH over all three axes, binned in one pass over the node's triangles
        float scale[3];
        bool live[3];
        for (int ax = 0; ax < 3; ++ax) {
            const float ext = cbox.hi[ax] - cbox.lo[ax];
            live[ax] = ext > 0.0f;
            scale[ax] = live[ax] ? float(kBins) / ext : 0.0f;
        }
        struct Bins {
            Box bb[3][kBins];
            uint32_t bc[3][kBins];
        };
        // per-chunk bins on the heap only when several threads bin (small nodes are the many)
        Bins one;
        std::vector<Bins> many;
        if (chunks > 1) many.resize(size_t(chunks));
        Bins* cbins = chunks > 1 ? many.data() : &one;
        for_chunks(begin, end, chunks, [&](uint32_t b0, uint32_t b1, int c) {
            // a bin's box is set by its first triangle (counts zeroed here), so the many small
            // nodes do not reset 96 boxes; the sweeps skip empty bins
            Bins& B = cbins[c];
            std::memset(B.bc, 0, sizeof(B.bc));
            for (uint32_t i = b0; i < b1; ++i) {
                const BuildPrim& pr = prims[i];
                for (int ax = 0; ax < 3; ++ax) {
                    if (!live[ax]) continue;
                    int b = int((pr.c[ax] - cbox.lo[ax]) * scale[ax]);
                    b = std::min(std::max(b, 0), kBins - 1);
                    if (B.bc[ax][b]++ == 0) B.bb[ax][b] = pr.box;
                    else B.bb[ax][b].grow(pr.box);
                }
            }
        });
        for (int c = 1; c < chunks; ++c)
            for (int ax = 0; ax < 3; ++ax)
                for (int b = 0; b < kBins; ++b) {
                    if (cbins[c].bc[ax][b] == 0) continue;
                    if (cbins[0].bc[ax][b] == 0) cbins[0].bb[ax][b] = cbins[c].bb[ax][b];
                    else cbins[0].bb[ax][b].grow(cbins[c].bb[ax][b]);
                    cbins[0].bc[ax][b] += cbins[c].bc[ax][b];
                }
        float best_cost = FLT_MAX;
        int best_axis = -1, best_split = -1;
        for (int ax = 0; ax < 3; ++ax) {
            if (!live[ax]) continue;
            const Box* bb = cbins[0].bb[ax];
            const uint32_t* bc = cbins[0].bc[ax];
            float ra[kBins];
            uint32_t rc[kBins];
            Box acc;
            acc.reset();
            uint32_t cnt = 0;
            for (int b = kBins - 1; b > 0; --b) {
                if (bc[b]) acc.grow(bb[b]);
                cnt += bc[b];
                ra[b] = acc.half_area();
                rc[b] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                if (bc[b]) acc.grow(bb[b]);
                cnt += bc[b];
                if (cnt == 0 || rc[b + 1] == 0) continue;
                const float cost = acc.half_area() * float(cnt) + ra[b + 1] * float(rc[b + 1]);
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = ax;
                    best_split = b;
                }
            }
        }
        const float parent_area = box.half_area();
        const float leaf_cost = float(n);
        const float split_cost = parent_area > 0.0f ? 1.0f + best_cost / parent_area : FLT_MAX;
        uint32_t mid;
        if (best_axis < 0) {
            // all centroids coincide: object median by index
            if (n <= kMaxLeafTris) return make_leaf();
            mid = begin + n / 2;
        } else {
            if (n <= kLeafTarget && leaf_cost <= split_cost) return make_leaf();
            const float ext = cbox.hi[best_axis] - cbox.lo[best_axis];
            const float scale = float(kBins) / ext;
            BuildPrim* m = std::partition(prims + begin, prims + end, [&](const BuildPrim& pr) {
                int b = int((pr.c[best_axis] - cbox.lo[best_axis]) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_split;
            });
            mid = uint32_t(m - prims);
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        const int l = alloc(), r = alloc();
        node.left = l;
        node.right = r;
        node.first = begin;  // an inner node's triangles are prims[first, first + count) too
        node.count = n;
        const bool spawn = (mid - begin) >= kParallelMin && (end - mid) >= kParallelMin &&
                           threads_live.fetch_add(1) < max_threads;
        if (spawn) {
            std::thread t([this, l, begin, mid, depth]() { build(l, begin, mid, depth + 1); });
            build(r, mid, end, depth + 1);
            t.join();
            threads_live.fetch_sub(1);
        } else {
            if ((mid - begin) >= kParallelMin && (end - mid) >= kParallelMin) threads_live.fetch_sub(1);
            build(l, begin, mid, depth + 1);
            build(r, mid, end, depth + 1);
        }
    }
};

// SAH-optimal collapse into 4-wide nodes (wide_collapse.cuh): costs of every
// binary node, children before parents (children have larger ids).
void wide_costs(const BinNode* bn, int count, std::vector<WideCost>* out) {
    std::vector<WideCost>& wc = *out;
    wc.resize(size_t(count));
    for (int n = count - 1; n >= 0; --n) {
        const BinNode& b = bn[size_t(n)];
        wc[size_t(n)] = b.left < 0 ? wide_cost_leaf(b.box.half_area(), b.count)
                                   : wide_cost_inner(b.box.half_area(), b.count, wc[size_t(b.left)],
                                                     wc[size_t(b.right)]);
    }
}

// The binary nodes that fill the slots of the wide node of inner node n.
int wide_children(const BinNode* bn, const std::vector<WideCost>& wc, int n, int (&kids)[4]) {
    uint32_t k[4];
    const int nk = wide_slots(
        uint32_t(bn[size_t(n)].left), uint32_t(bn[size_t(n)].right), [&](uint32_t x) { return wc[x]; },
        [&](uint32_t x) { return uint32_t(bn[x].left); }, [&](uint32_t x) { return uint32_t(bn[x].right); }, k);
    for (int i = 0; i < nk; ++i) kids[i] = int(k[i]);
    return nk;
}

}  // namespace

bool build_bvh4(const float* tri_vertices, uint32_t num_tris, Bvh4Result* out, std::string* err) {
    out->nodes.clear();
    out->order.clear();
    if (num_tris == 0) {
        *err = "scene has no triangles";
        return false;
    }
    if (num_tris > kMaxTriSlots) {
        *err = "too many triangles for the 28-bit leaf encoding";
        return false;
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int setup_chunks = num_tris >= kParallelBinMin ? int(std::min<unsigned>(hw, kMaxChunks)) : 1;
    std::unique_ptr<BuildPrim[]> prims(new BuildPrim[num_tris]);
    out->order.resize(num_tris);
    Builder::for_chunks(0, num_tris, setup_chunks, [&](uint32_t t0, uint32_t t1, int) {
        for (uint32_t t = t0; t < t1; ++t) {
            BuildPrim& p = prims[t];
            p.box.reset();
            const float* v = tri_vertices + 9 * size_t(t);
            p.box.grow(v);
            p.box.grow(v + 3);
            p.box.grow(v + 6);
            for (int k = 0; k < 3; ++k) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
            p.t = t;
        }
    });
    std::unique_ptr<BinNode[]> nodes(new BinNode[size_t(num_tris) * 2]);
    Builder B;
    B.prims = prims.get();
    B.nodes = nodes.get();
    B.max_threads = int(hw) * 2;
    B.hw_threads = int(hw);
    const int root = B.alloc();
    B.build(root, 0, num_tris, 0);
    const BinNode* bn = nodes.get();
    Builder::for_chunks(0, num_tris, setup_chunks, [&](uint32_t t0, uint32_t t1, int) {
        for (uint32_t i = t0; i < t1; ++i) out->order[i] = prims[i].t;
    });
    out->binary_depth = B.max_depth.load();

    // SAH-optimal collapse into 4-wide nodes (breadth-first ids, root = 0)
    std::vector<WideCost> wc;
    wide_costs(bn, B.next_node.load(), &wc);
    struct Item { int bin; int wide; int depth; };
    std::vector<Item> work;
    // the tree's shape first (breadth-first), then the nodes' quantized boxes on all host threads
    struct Slots {
        int nk = 0;
        int bin[4] = {0, 0, 0, 0};
        uint32_t child[4] = {0, 0, 0, 0};
    };
    std::vector<Slots> slots(1);
    slots.reserve(size_t(num_tris) / 2 + 1);
    work.push_back({root, 0, 1});
    size_t head = 0;
    int wide_depth = 1;
    while (head < work.size()) {
        const Item it = work[head++];
        wide_depth = std::max(wide_depth, it.depth);
        int kids[4];
        int nk = 0;
        const BinNode& b = bn[it.bin];
        if (b.left < 0 || wc[it.bin].leaf) {
            kids[nk++] = it.bin;  // a root that is one leaf
        } else {
            nk = wide_children(bn, wc, it.bin, kids);
        }
        Slots sl;  // filled here, stored below: emplace_back may move the vector
        sl.nk = nk;
        for (int k = 0; k < nk; ++k) {
            const BinNode& c = bn[kids[k]];
            sl.bin[k] = kids[k];
            if (c.left < 0 || wc[kids[k]].leaf) {
                sl.child[k] = make_leaf(c.first, c.count);
            } else {
                const int id = int(slots.size());
                slots.emplace_back();
                work.push_back({kids[k], id, it.depth + 1});
                sl.child[k] = uint32_t(id);
            }
        }
        slots[size_t(it.wide)] = sl;
    }
    out->nodes.resize(slots.size());
    const int emit_chunks = slots.size() >= 65536 ? int(std::min<unsigned>(hw, kMaxChunks)) : 1;
    Builder::for_chunks(0, uint32_t(slots.size()), emit_chunks, [&](uint32_t w0, uint32_t w1, int) {
        for (uint32_t w = w0; w < w1; ++w) {
            const Slots& sl = slots[w];
            float lo[4][3] = {}, hi[4][3] = {};
            for (int k = 0; k < sl.nk; ++k)
                for (int a = 0; a < 3; ++a) {
                    lo[k][a] = bn[size_t(sl.bin[k])].box.lo[a];
                    hi[k][a] = bn[size_t(sl.bin[k])].box.hi[a];
                }
            quantize_node(lo, hi, sl.child, sl.nk, &out->nodes[w]);
        }
    });
    out->wide_depth = wide_depth;
    return true;
}

}  // namespace cg
