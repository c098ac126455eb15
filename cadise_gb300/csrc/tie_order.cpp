// Exact-tie ranks: the reference's binary BVH over the scene's primitives
// (shape only) and, per direction octant, the order in which its closest-hit
// traversal reaches their leaves.
#include "tie_order.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <future>
#include <thread>

namespace cg {
namespace {

struct Box3 {
    float lo[3], hi[3];
};

// TAABB's empty box (tAabb.ipp:13-17): the upper corner starts at FLT_MIN,
// the smallest positive float, and unionWith is a component min / max.
inline Box3 empty_box() {
    Box3 b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = FLT_MAX;
        b.hi[k] = FLT_MIN;
    }
    return b;
}
inline void grow(Box3& b, const float* lo, const float* hi) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], lo[k]);
        b.hi[k] = std::max(b.hi[k], hi[k]);
    }
}
// half the surface area; the reference's SAH divides full areas by a full
// area, which rounds to the same ratio (both scale by exactly 2)
inline float half_area(const Box3& b) {
    const float x = b.hi[0] - b.lo[0], y = b.hi[1] - b.lo[1], z = b.hi[2] - b.lo[2];
    return x * y + y * z + z * x;
}

struct Tree {
    // per node: split axis (internal) or -1 (leaf); children; range of `items`
    std::vector<int8_t> axis;
    std::vector<int32_t> first, second, begin, count;
};

// One primitive's box and index; the build partitions these in place
// (contiguous, as the reference's vectors of bound infos are), which gives
// the same orders as the reference's copies.  The centroid, (lo + hi) / 2,
// is recomputed where it is needed (the same bits; 28 bytes an item instead
// of 40 move through every level of the build).
struct Item {
    float lo[3], hi[3];
    int32_t idx;
    float c(int k) const { return (lo[k] + hi[k]) * 0.5f; }
};

class Builder {
public:
    Builder(const cgpu_scene_desc* d) : n_(d->num_primitives), items_(n_) {
        for (uint32_t i = 0; i < n_; ++i) prim_box(d, i);
        // at most 2n - 1 nodes; slots are taken with an atomic counter
        const size_t cap = n_ > 0 ? 2 * size_t(n_) - 1 : 1;
        tree_.axis.assign(cap, -1);
        tree_.first.assign(cap, -1);
        tree_.second.assign(cap, -1);
        tree_.begin.assign(cap, 0);
        tree_.count.assign(cap, 0);
    }

    void build() {
        next_.store(0);
        if (n_ > 0) node(0, int32_t(n_), 0);
    }

    // Ranks of all 8 octants in one pass down the tree: a node passes each
    // octant's first leaf position to its children, the child visited second
    // getting it plus the size of the one visited first; a leaf writes one
    // 32-byte row per primitive.  Large subtrees run on their own threads.
    std::vector<uint32_t> ranks() {
        std::vector<uint32_t> r(8 * size_t(n_));
        if (n_ == 0) return r;
        const std::array<uint32_t, 8> zero{};
        threads_.store(1);
        rank_rows(0, zero, r.data());
        return r;
    }

private:
    // Primitive bounds as the reference computes them: the vertices' box
    // expanded by 0.0001 (a rectangle's fourth corner is vB + eA + eB), a
    // sphere's (c - r, c + r) expanded by 0.0001.
    void prim_box(const cgpu_scene_desc* d, uint32_t i) {
        const int kind = d->prim_kind ? d->prim_kind[i] : CGPU_PRIM_TRIANGLE;
        const float* v = d->prim_vertices + 9 * size_t(i);
        Item& it = items_[i];
        it.idx = int32_t(i);
        float* lo = it.lo;
        float* hi = it.hi;
        if (kind == CGPU_PRIM_SPHERE) {
            for (int k = 0; k < 3; ++k) {
                lo[k] = (v[k] - v[3]) - 0.0001f;
                hi[k] = (v[k] + v[3]) + 0.0001f;
            }
        } else {
            float p[4][3];
            int np = 3;
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) p[j][k] = v[3 * j + k];
            if (kind == CGPU_PRIM_RECTANGLE) {  // v = (vA, vB, vC)
                for (int k = 0; k < 3; ++k) {
                    const float eA = v[k] - v[3 + k], eB = v[6 + k] - v[3 + k];
                    p[3][k] = (v[3 + k] + eA) + eB;
                }
                np = 4;
            }
            for (int k = 0; k < 3; ++k) {
                float a = p[0][k], b = p[0][k];
                for (int j = 1; j < np; ++j) {
                    a = std::min(a, p[j][k]);
                    b = std::max(b, p[j][k]);
                }
                lo[k] = a - 0.0001f;
                hi[k] = b + 0.0001f;
            }
        }
    }

    int32_t make_leaf(int32_t id, int32_t b, int32_t e) {
        tree_.axis[size_t(id)] = -1;
        tree_.begin[size_t(id)] = b;
        tree_.count[size_t(id)] = e - b;
        return id;
    }

    // BvhBuilder::_buildBinaryNodesRecursively on items_[b, e)
    int32_t node(int32_t b, int32_t e, int depth) {
        const int32_t id = next_.fetch_add(1);
        const int32_t count = e - b;
        if (count <= 1) return make_leaf(id, b, e);
        Item* it = items_.data();
        // bounds of the primitives and of their centroids (min / max: the
        // same result in any order, so large ranges are split over threads)
        struct Bounds {
            Box3 box = empty_box(), cbox = empty_box();
        };
        const Bounds bd = reduce<Bounds>(b, e, [it](int32_t i0, int32_t i1, Bounds& r) {
            for (int32_t i = i0; i < i1; ++i) {
                grow(r.box, it[i].lo, it[i].hi);
                const float c[3] = {it[i].c(0), it[i].c(1), it[i].c(2)};
                grow(r.cbox, c, c);
            }
        }, [](Bounds& r, const Bounds& x) {
            grow(r.box, x.box.lo, x.box.hi);
            grow(r.cbox, x.cbox.lo, x.cbox.hi);
        });
        const Box3 box = bd.box, cbox = bd.cbox;
        float ext[3];
        for (int k = 0; k < 3; ++k) ext[k] = cbox.hi[k] - cbox.lo[k];
        int axis = 0;
        if (ext[1] > ext[axis]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        if (cbox.lo[axis] == cbox.hi[axis]) return make_leaf(id, b, e);
        int32_t mid;
        if (count <= 2) {
            // the equal split (_canSplitWithEqual): the lower centroid first
            mid = b + (count + 1) / 2;
            std::nth_element(it + b, it + mid, it + e,
                             [axis](const Item& x, const Item& y) { return x.c(axis) < y.c(axis); });
        } else {
            constexpr int kBuckets = 12;
            const float cmin = cbox.lo[axis];
            const float inv_ext = 1.0f / ext[axis];
            auto bucket = [axis, cmin, inv_ext](const Item& x) {
                const size_t k = size_t((x.c(axis) - cmin) * inv_ext * float(kBuckets));
                return k == size_t(kBuckets) ? size_t(kBuckets - 1) : k;
            };
            struct Bins {
                int32_t n[kBuckets] = {0};
                Box3 box[kBuckets];
                Bins() {
                    for (auto& x : box) x = empty_box();
                }
            };
            const Bins bins = reduce<Bins>(b, e, [it, &bucket](int32_t i0, int32_t i1, Bins& r) {
                for (int32_t i = i0; i < i1; ++i) {
                    const size_t k = bucket(it[i]);
                    ++r.n[k];
                    grow(r.box[k], it[i].lo, it[i].hi);
                }
            }, [](Bins& r, const Bins& x) {
                for (int k = 0; k < kBuckets; ++k) {
                    r.n[k] += x.n[k];
                    grow(r.box[k], x.box[k].lo, x.box[k].hi);
                }
            });
            const int32_t* bn = bins.n;
            const Box3* bb = bins.box;
            const float inv_area = 1.0f / half_area(box);
            float best = FLT_MAX;
            size_t best_split = size_t(kBuckets);
            for (int s = 0; s < kBuckets - 1; ++s) {
                Box3 A = empty_box(), B = empty_box();
                int32_t na = 0, nb = 0;
                for (int k = 0; k <= s; ++k) {
                    grow(A, bb[k].lo, bb[k].hi);
                    na += bn[k];
                }
                for (int k = s + 1; k < kBuckets; ++k) {
                    grow(B, bb[k].lo, bb[k].hi);
                    nb += bn[k];
                }
                // an empty side has an infinite area and its cost 0 x inf is
                // NaN in the reference, which never compares below the best
                if (na == 0 || nb == 0) continue;
                const float cost = 0.125f + (half_area(A) * inv_area * float(na) + half_area(B) * inv_area * float(nb));
                if (cost < best) {
                    best = cost;
                    best_split = size_t(s);
                }
            }
            if (best >= float(count)) return make_leaf(id, b, e);
            mid = int32_t(std::partition(it + b, it + e, [&](const Item& x) { return bucket(x) <= best_split; }) - it);
            if (mid == b || mid == e) return make_leaf(id, b, e);
        }
        tree_.axis[size_t(id)] = int8_t(axis);
        tree_.begin[size_t(id)] = b;
        tree_.count[size_t(id)] = count;
        int32_t f;
        if (count >= kParallelRange && take_thread()) {
            auto left = std::async(std::launch::async, [this, b, mid, depth] {
                const int32_t r = node(b, mid, depth + 1);
                threads_.fetch_sub(1);
                return r;
            });
            tree_.second[size_t(id)] = node(mid, e, depth + 1);
            f = left.get();
        } else {
            f = node(b, mid, depth + 1);
            tree_.second[size_t(id)] = node(mid, e, depth + 1);
        }
        tree_.first[size_t(id)] = f;
        return id;
    }

    uint32_t size_of(int32_t id) const { return uint32_t(tree_.count[size_t(id)]); }

    void rank_rows(int32_t id, const std::array<uint32_t, 8>& start, uint32_t* r) {
        const int ax = tree_.axis[size_t(id)];
        if (ax < 0) {
            const int32_t b = tree_.begin[size_t(id)], n = tree_.count[size_t(id)];
            for (int32_t i = 0; i < n; ++i) {
                uint32_t* row = r + 8 * size_t(items_[size_t(b + i)].idx);
                for (int o = 0; o < 8; ++o) row[o] = start[size_t(o)] + uint32_t(i);
            }
            return;
        }
        const int32_t f = tree_.first[size_t(id)], sc = tree_.second[size_t(id)];
        std::array<uint32_t, 8> sf, ss;
        for (int o = 0; o < 8; ++o) {
            // the reference takes the second child first when the ray runs towards -axis
            const bool second_first = ((o >> ax) & 1) != 0;
            sf[size_t(o)] = start[size_t(o)] + (second_first ? size_of(sc) : 0u);
            ss[size_t(o)] = start[size_t(o)] + (second_first ? 0u : size_of(f));
        }
        if (size_of(id) >= uint32_t(kParallelRange) && take_thread()) {
            auto first = std::async(std::launch::async, [this, f, sf, r] {
                rank_rows(f, sf, r);
                threads_.fetch_sub(1);
            });
            rank_rows(sc, ss, r);
            first.get();
        } else {
            rank_rows(f, sf, r);
            rank_rows(sc, ss, r);
        }
    }

    // A thread for the first child of a range of at least kParallelRange
    // primitives, while fewer than 2 x the hardware threads build.
    bool take_thread() {
        int cur = threads_.load();
        while (cur < max_threads_)
            if (threads_.compare_exchange_weak(cur, cur + 1)) return true;
        return false;
    }

    // f(i0, i1, partial) over [b, e) in chunks, partials combined by g; ranges
    // of at least kSplitRange use all hardware threads.
    template <class R, class F, class G>
    static R reduce(int32_t b, int32_t e, F f, G g) {
        R out;
        const int32_t n = e - b;
        const int nt = n >= kSplitRange ? hw_threads() : 1;
        if (nt <= 1) {
            f(b, e, out);
            return out;
        }
        std::vector<R> part(static_cast<size_t>(nt));
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) {
            const int32_t i0 = b + int32_t(int64_t(n) * t / nt), i1 = b + int32_t(int64_t(n) * (t + 1) / nt);
            th.emplace_back([&, t, i0, i1] { f(i0, i1, part[size_t(t)]); });
        }
        for (auto& x : th) x.join();
        for (const R& x : part) g(out, x);
        return out;
    }
    static int hw_threads() {
        const unsigned h = std::thread::hardware_concurrency();
        return h ? int(h) : 4;
    }

    static constexpr int32_t kParallelRange = 1 << 15;
    static constexpr int32_t kSplitRange = 1 << 20;

    uint32_t n_;
    std::vector<Item> items_;
    Tree tree_;
    std::atomic<int32_t> next_{0};
    std::atomic<int> threads_{1};
    const int max_threads_ = 2 * hw_threads();
};

}  // namespace

std::vector<uint32_t> reference_visit_ranks(const cgpu_scene_desc* d) {
    Builder b(d);
    b.build();
    return b.ranks();
}

}  // namespace cg
