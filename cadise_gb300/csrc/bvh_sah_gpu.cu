// GPU BVH build by binned SAH: the host build's algorithm (bvh_build.cpp) run
// on the GPU, then the shared SAH-optimal collapse (wide_collapse.cuh) and the
// 64-byte quantized nodes.
//
// Replaces BvhBuilder (source/core/intersector/accelerator/bvh/bvhBuilder.cpp:18-358,
// serial recursive SAH).  The same decisions as the host build: per node 32
// bins on every axis with a non-empty centroid extent, the same FP32 sweep and
// costs, leaves of up to 4 triangles where the SAH says so (8 when the
// centroids coincide), a median by position when the centroids coincide or the
// best split leaves one side empty.  The partition is stable (the host's is
// not), so the two trees differ only below such median splits.
//   * nodes of more than kSmall triangles, one tree level per round: the node's
//     triangles in chunks of kChunk, one block per chunk for the bounds, the
//     bins and the stable partition (prefix sums over the chunks of a node),
//     one block per node for the split;
//   * nodes of at most kSmall triangles: one block builds the whole subtree in
//     shared memory, depth first.
// No kernel waits on another thread; every loop is bounded by the data.
#include "bvh_build.h"
#include "radix.cuh"
#include "wide_collapse.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace cg {
namespace {

constexpr int kSahBins = 32;
constexpr int kNumBins = 3 * kSahBins;
constexpr uint32_t kSahLeafTarget = 4;  // bvh_build.cpp kLeafTarget
constexpr uint32_t kChunk = 4096;       // triangles per block in the large-node rounds
constexpr uint32_t kSmall = 512;        // nodes up to this size build in one block
constexpr int kSmallThreads = 128;
constexpr uint32_t kNil = 0xFFFFFFFFu;
constexpr float kFltMax = 3.402823466e38f;

__device__ __forceinline__ int fkey(float f) {  // order-preserving int image of a float
    const int i = __float_as_int(f);
    return i >= 0 ? i : int(0x80000000u ^ ~uint32_t(i));
}
__device__ __forceinline__ float fval(int k) { return __int_as_float(k >= 0 ? k : int(~(uint32_t(k) ^ 0x80000000u))); }

// Box::half_area of bvh_build.cpp: 0 for an empty (inverted) box.
__device__ __forceinline__ float box_half_area(const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0.0f || dy < 0.0f || dz < 0.0f) return 0.0f;
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
    const int b = int((c - lo) * scale);
    return min(max(b, 0), kSahBins - 1);
}

// A node's split: mode 0 leaf, 1 by bins (axis, bin: left = bins <= bin), 2 by position (left = [begin, mid)).
struct Split {
    uint32_t mode, axis, bin, mid;
};

struct SegInfo {  // a large node of the current round
    uint32_t begin, count, node, chunk0, nchunks, pad[3];
};
struct Chunk {
    uint32_t seg, begin, end, pad;
};
struct SmallSeg {
    uint32_t begin, count, node, pad;
};

// The per-node bounds (box, centroid box) and bin scales of a large node.
struct SegBounds {
    float lo[3], hi[3], clo[3], chi[3], scale[3];
    uint32_t live;  // bit a: the centroid extent on axis a is positive
};

// The host build's leaf rules and the split of a node of n triangles in [begin, begin + n)
// once the sweep found its cheapest bin split (best_axis < 0: none);
// `left` is the triangle count of bins <= best_split of best_axis.
__device__ Split finish_split(const SegBounds& sb, uint32_t begin, uint32_t n, int best_axis, int best_split,
                              float best_cost, uint32_t left, uint32_t* left_count) {
    Split sp{0, 0, 0, begin};
    *left_count = 0;
    const float parent_area = box_half_area(sb.lo, sb.hi);
    const float leaf_cost = float(n);
    const float split_cost = parent_area > 0.0f ? 1.0f + best_cost / parent_area : kFltMax;
    if (best_axis < 0) {
        if (n <= kMaxLeafTris) return sp;  // leaf
        sp.mode = 2;
        sp.mid = begin + n / 2;
        *left_count = n / 2;
        return sp;
    }
    if (n <= kSahLeafTarget && leaf_cost <= split_cost) return sp;  // leaf
    if (left == 0 || left == n) {
        sp.mode = 2;
        sp.mid = begin + n / 2;
        *left_count = n / 2;
        return sp;
    }
    sp.mode = 1;
    sp.axis = uint32_t(best_axis);
    sp.bin = uint32_t(best_split);
    sp.mid = begin + left;
    *left_count = left;
    return sp;
}

// The host build's SAH sweep (bvh_build.cpp) over bins already reduced
// (counts + boxes), by the 32 lanes of one warp, lane b holding bin b of each
// axis.  The left (prefix) and right (suffix) box unions are min / max scans
// and the counts integer scans, exact in any order, so every candidate's
// cost is the host's serial sweep's to the bit; the argmin keeps, among equal
// costs, the first in (axis, bin) order, as the serial sweep does.  Every
// lane of the warp must call it and gets the same split.
__device__ Split choose_split_warp(const SegBounds& sb, const uint32_t* bcnt, const float (*bbox)[6], uint32_t begin,
                                   uint32_t n, uint32_t* left_count) {
    static_assert(kSahBins == 32, "one bin per lane");
    *left_count = 0;
    if (n <= 1) return Split{0, 0, 0, begin};
    const int lane = int(threadIdx.x & 31u);
    float best_cost = kFltMax;
    int best_idx = 0x7FFFFFFF;  // axis * kSahBins + bin of this lane's cheapest candidate
    uint32_t best_left = 0;
    for (int ax = 0; ax < 3; ++ax) {
        if (!((sb.live >> ax) & 1u)) continue;
        const int j = ax * kSahBins + lane;
        const uint32_t c = bcnt[j];
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {  // an empty bin is the union's identity
            lo[k] = c ? bbox[j][k] : kFltMax;
            hi[k] = c ? bbox[j][3 + k] : -kFltMax;
        }
        float plo[3] = {lo[0], lo[1], lo[2]}, phi[3] = {hi[0], hi[1], hi[2]};  // bins <= lane
        float slo[3] = {lo[0], lo[1], lo[2]}, shi[3] = {hi[0], hi[1], hi[2]};  // bins >= lane
        uint32_t pc = c, sc = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            for (int k = 0; k < 3; ++k) {
                const float ul = __shfl_up_sync(0xFFFFFFFFu, plo[k], off), uh = __shfl_up_sync(0xFFFFFFFFu, phi[k], off);
                const float dl = __shfl_down_sync(0xFFFFFFFFu, slo[k], off), dh = __shfl_down_sync(0xFFFFFFFFu, shi[k], off);
                if (lane >= off) {
                    plo[k] = fminf(plo[k], ul);
                    phi[k] = fmaxf(phi[k], uh);
                }
                if (lane + off < 32) {
                    slo[k] = fminf(slo[k], dl);
                    shi[k] = fmaxf(shi[k], dh);
                }
            }
            const uint32_t ucnt = __shfl_up_sync(0xFFFFFFFFu, pc, off), dcnt = __shfl_down_sync(0xFFFFFFFFu, sc, off);
            if (lane >= off) pc += ucnt;
            if (lane + off < 32) sc += dcnt;
        }
        // the right side of split `lane` is bins >= lane + 1
        const float ra = __shfl_down_sync(0xFFFFFFFFu, box_half_area(slo, shi), 1);
        const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, sc, 1);
        if (lane < kSahBins - 1 && pc != 0 && rc != 0) {
            const float cost = box_half_area(plo, phi) * float(pc) + ra * float(rc);
            if (cost < best_cost) {
                best_cost = cost;
                best_idx = j;
                best_left = pc;
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oc = __shfl_xor_sync(0xFFFFFFFFu, best_cost, off);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, best_idx, off);
        const uint32_t ol = __shfl_xor_sync(0xFFFFFFFFu, best_left, off);
        if (oc < best_cost || (oc == best_cost && oi < best_idx)) {
            best_cost = oc;
            best_idx = oi;
            best_left = ol;
        }
    }
    const bool found = best_idx != 0x7FFFFFFF;
    return finish_split(sb, begin, n, found ? best_idx / kSahBins : -1, found ? best_idx % kSahBins : -1, best_cost,
                        best_left, left_count);
}

__device__ __forceinline__ bool goes_left(const Split& sp, const SegBounds& sb, float4 lo, float4 hi, uint32_t pos) {
    if (sp.mode == 2) return pos < sp.mid;
    const int a = int(sp.axis);
    const float l = a == 0 ? lo.x : a == 1 ? lo.y : lo.z, h = a == 0 ? hi.x : a == 1 ? hi.y : hi.z;
    return uint32_t(bin_of(0.5f * (l + h), sb.clo[a], sb.scale[a])) <= sp.bin;
}

// Children of a split node: ids, links and counts; each child goes to the
// next round's large nodes or to the small-node list.
__device__ void make_children(uint32_t node, uint32_t begin, uint32_t n, uint32_t left, uint32_t* node_counter,
                              float4* blo, float4* bhi, uint32_t* parent, uint32_t* count, uint32_t* first,
                              SegInfo* next, uint32_t* next_count, SmallSeg* small, uint32_t* small_count) {
    const uint32_t l = atomicAdd(node_counter, 2u), r = l + 1;
    blo[node].w = __uint_as_float(l);
    bhi[node].w = __uint_as_float(r);
    const uint32_t cb[2] = {begin, begin + left}, cn[2] = {left, n - left}, id[2] = {l, r};
    for (int k = 0; k < 2; ++k) {
        parent[id[k]] = node;
        count[id[k]] = cn[k];
        first[id[k]] = cb[k];
        if (cn[k] > kSmall) {
            const uint32_t s = atomicAdd(next_count, 1u);
            next[s] = SegInfo{cb[k], cn[k], id[k], 0, 0, {0, 0, 0}};
        } else {
            const uint32_t s = atomicAdd(small_count, 1u);
            small[s] = SmallSeg{cb[k], cn[k], id[k], 0};
        }
    }
}

// ------------------------------------------------------------ large nodes --
__global__ void k_sah_init(const float* tv, uint32_t n, float4* plo, float4* phi) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* v = tv + 9 * size_t(i);
        float l[3], h[3];
        for (int k = 0; k < 3; ++k) {
            l[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
            h[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
        }
        plo[i] = make_float4(l[0], l[1], l[2], __uint_as_float(i));
        phi[i] = make_float4(h[0], h[1], h[2], 0.0f);
    }
}

// Block-wide min / max of 12 floats (box lo, hi, centroid lo, hi) into red[12].
__device__ void block_bounds(float (&v)[12], float* red) {
    for (int k = 0; k < 12; ++k) {
        const bool mx = (k >= 3 && k < 6) || k >= 9;
        for (int o = 16; o > 0; o >>= 1) {
            const float u = __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
            v[k] = mx ? fmaxf(v[k], u) : fminf(v[k], u);
        }
    }
    __shared__ float part[32][12];
    const int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 12; ++k) part[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        const bool mx = (k >= 3 && k < 6) || k >= 9;
        float r = part[0][k];
        for (int w = 1; w < nw; ++w) r = mx ? fmaxf(r, part[w][k]) : fminf(r, part[w][k]);
        red[k] = r;
    }
    __syncthreads();
}

__device__ __forceinline__ void bounds_init(float (&v)[12]) {
    for (int k = 0; k < 12; ++k) v[k] = ((k >= 3 && k < 6) || k >= 9) ? -kFltMax : kFltMax;
}
__device__ __forceinline__ void bounds_add(float (&v)[12], float4 lo, float4 hi) {
    const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
    for (int k = 0; k < 3; ++k) {
        const float c = 0.5f * (l[k] + h[k]);
        v[k] = fminf(v[k], l[k]);
        v[3 + k] = fmaxf(v[3 + k], h[k]);
        v[6 + k] = fminf(v[6 + k], c);
        v[9 + k] = fmaxf(v[9 + k], c);
    }
}

__global__ void k_chunk_bounds(const Chunk* chunks, const float4* plo, const float4* phi, float* cbounds) {
    __shared__ float red[12];
    const Chunk ch = chunks[blockIdx.x];
    float v[12];
    bounds_init(v);
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) bounds_add(v, plo[i], phi[i]);
    block_bounds(v, red);
    if (threadIdx.x < 12) cbounds[12 * blockIdx.x + threadIdx.x] = red[threadIdx.x];
}

__global__ void k_seg_bounds(const SegInfo* segs, const float* cbounds, SegBounds* sbs, float4* blo, float4* bhi) {
    __shared__ float red[12];
    const SegInfo sg = segs[blockIdx.x];
    float v[12];
    bounds_init(v);
    for (uint32_t c = threadIdx.x; c < sg.nchunks; c += blockDim.x) {
        const float* b = cbounds + 12 * size_t(sg.chunk0 + c);
        for (int k = 0; k < 12; ++k) v[k] = ((k >= 3 && k < 6) || k >= 9) ? fmaxf(v[k], b[k]) : fminf(v[k], b[k]);
    }
    block_bounds(v, red);
    if (threadIdx.x == 0) {
        SegBounds sb;
        sb.live = 0;
        for (int k = 0; k < 3; ++k) {
            sb.lo[k] = red[k];
            sb.hi[k] = red[3 + k];
            sb.clo[k] = red[6 + k];
            sb.chi[k] = red[9 + k];
            const float ext = sb.chi[k] - sb.clo[k];
            const bool live = ext > 0.0f;
            sb.scale[k] = live ? float(kSahBins) / ext : 0.0f;
            sb.live |= live ? (1u << k) : 0u;
        }
        sbs[blockIdx.x] = sb;
        blo[sg.node] = make_float4(sb.lo[0], sb.lo[1], sb.lo[2], __uint_as_float(kNil));
        bhi[sg.node] = make_float4(sb.hi[0], sb.hi[1], sb.hi[2], __uint_as_float(kNil));
    }
}

// Bins of one chunk: counts and boxes (as order-preserving ints, so shared
// atomics give the exact min / max) on every live axis.
__global__ void k_chunk_bins(const Chunk* chunks, const SegBounds* sbs, const float4* plo, const float4* phi,
                             uint32_t* bcnt, int* bkey) {
    __shared__ uint32_t cnt[kNumBins];
    __shared__ int key[kNumBins][6];
    const Chunk ch = chunks[blockIdx.x];
    const SegBounds sb = sbs[ch.seg];
    for (int j = threadIdx.x; j < kNumBins; j += blockDim.x) {
        cnt[j] = 0;
        for (int k = 0; k < 3; ++k) {
            key[j][k] = fkey(kFltMax);
            key[j][3 + k] = fkey(-kFltMax);
        }
    }
    __syncthreads();
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        const float4 lo = plo[i], hi = phi[i];
        const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
        for (int a = 0; a < 3; ++a) {
            if (!((sb.live >> a) & 1u)) continue;
            const int j = a * kSahBins + bin_of(0.5f * (l[a] + h[a]), sb.clo[a], sb.scale[a]);
            atomicAdd(&cnt[j], 1u);
            for (int k = 0; k < 3; ++k) {
                atomicMin(&key[j][k], fkey(l[k]));
                atomicMax(&key[j][3 + k], fkey(h[k]));
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kNumBins; j += blockDim.x) {
        bcnt[size_t(blockIdx.x) * kNumBins + j] = cnt[j];
        for (int k = 0; k < 6; ++k) bkey[(size_t(blockIdx.x) * kNumBins + j) * 6 + k] = key[j][k];
    }
}

// One block of kNumBins threads per large node: the bins of its chunks, the
// split, the children.
__global__ void k_seg_split(const SegInfo* segs, const SegBounds* sbs, const uint32_t* bcnt, const int* bkey,
                            Split* splits, uint32_t* node_counter, float4* blo, float4* bhi, uint32_t* parent,
                            uint32_t* count, uint32_t* first, uint32_t* leaves, uint32_t* leaf_count, SegInfo* next,
                            uint32_t* next_count, SmallSeg* small, uint32_t* small_count) {
    __shared__ uint32_t cnt[kNumBins];
    __shared__ float box[kNumBins][6];
    const SegInfo sg = segs[blockIdx.x];
    const int j = threadIdx.x;
    if (j < kNumBins) {
        uint32_t c = 0;
        int k6[6];
        for (int k = 0; k < 3; ++k) {
            k6[k] = fkey(kFltMax);
            k6[3 + k] = fkey(-kFltMax);
        }
        for (uint32_t q = 0; q < sg.nchunks; ++q) {
            const size_t at = size_t(sg.chunk0 + q) * kNumBins + j;
            const uint32_t cq = bcnt[at];
            if (cq == 0) continue;
            c += cq;
            for (int k = 0; k < 3; ++k) {
                k6[k] = min(k6[k], bkey[at * 6 + k]);
                k6[3 + k] = max(k6[3 + k], bkey[at * 6 + 3 + k]);
            }
        }
        cnt[j] = c;
        for (int k = 0; k < 6; ++k) box[j][k] = fval(k6[k]);
    }
    __syncthreads();
    if (j >= 32) return;
    const SegBounds sb = sbs[blockIdx.x];
    uint32_t left = 0;
    const Split sp = choose_split_warp(sb, cnt, box, sg.begin, sg.count, &left);
    if (j != 0) return;
    splits[blockIdx.x] = sp;
    count[sg.node] = sg.count;
    first[sg.node] = sg.begin;
    if (sp.mode == 0) {
        leaves[atomicAdd(leaf_count, 1u)] = sg.node;
        return;
    }
    make_children(sg.node, sg.begin, sg.count, left, node_counter, blo, bhi, parent, count, first, next, next_count,
                  small, small_count);
}

// Left / right counts of every chunk (leaf nodes: all left, nothing moves).
__global__ void k_chunk_count(const Chunk* chunks, const SegBounds* sbs, const Split* splits, const float4* plo,
                              const float4* phi, uint32_t* chunk_left) {
    __shared__ uint32_t total;
    const Chunk ch = chunks[blockIdx.x];
    const Split sp = splits[ch.seg];
    const SegBounds sb = sbs[ch.seg];
    if (threadIdx.x == 0) total = 0;
    __syncthreads();
    uint32_t mine = 0;
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x)
        mine += (sp.mode == 0 || goes_left(sp, sb, plo[i], phi[i], i)) ? 1u : 0u;
    atomicAdd(&total, mine);
    __syncthreads();
    if (threadIdx.x == 0) chunk_left[blockIdx.x] = total;
}

// Per node, the first left and right slot of each of its chunks.
__global__ void k_seg_offsets(const SegInfo* segs, uint32_t nseg, const Chunk* chunks, const uint32_t* chunk_left,
                              uint32_t* lbase, uint32_t* rbase) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) {
        const SegInfo sg = segs[s];
        uint32_t l = 0, r = 0;
        for (uint32_t q = 0; q < sg.nchunks; ++q) {
            const uint32_t c = sg.chunk0 + q;
            lbase[c] = l;
            rbase[c] = r;
            l += chunk_left[c];
            r += (chunks[c].end - chunks[c].begin) - chunk_left[c];
        }
    }
}

// Stable partition of one chunk into tlo / thi: rounds of blockDim
// consecutive triangles, ranked by a block prefix sum.
__global__ void k_chunk_scatter(const Chunk* chunks, const SegInfo* segs, const SegBounds* sbs, const Split* splits,
                                const uint32_t* lbase, const uint32_t* rbase, const float4* plo, const float4* phi,
                                float4* tlo, float4* thi) {
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t run_l, run_r;
    const Chunk ch = chunks[blockIdx.x];
    const SegInfo sg = segs[ch.seg];
    const Split sp = splits[ch.seg];
    const SegBounds sb = sbs[ch.seg];
    const uint32_t lstart = sg.begin + lbase[blockIdx.x];
    const uint32_t mid = sp.mode == 0 ? sg.begin + sg.count : sp.mid;
    const uint32_t rstart = mid + rbase[blockIdx.x];
    if (threadIdx.x == 0) run_l = run_r = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (uint32_t base = ch.begin; base < ch.end; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < ch.end;
        float4 lo = make_float4(0, 0, 0, 0), hi = lo;
        bool left = false;
        if (valid) {
            lo = plo[i];
            hi = phi[i];
            left = sp.mode == 0 || goes_left(sp, sb, lo, hi, i);
        }
        const unsigned ball = __ballot_sync(0xFFFFFFFFu, valid && left);
        const uint32_t before_in_warp = __popc(ball & ((1u << lane) - 1u));
        if (lane == 0) warp_sum[warp] = __popc(ball);
        __syncthreads();
        uint32_t warp_before = 0, round_left = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < warp) warp_before += warp_sum[w];
            round_left += warp_sum[w];
        }
        const uint32_t lrank = warp_before + before_in_warp;
        const uint32_t valid_before = min(uint32_t(threadIdx.x), ch.end - base > blockDim.x ? blockDim.x : ch.end - base);
        if (valid) {
            const uint32_t dst = left ? lstart + run_l + lrank : rstart + run_r + (valid_before - lrank);
            tlo[dst] = lo;
            thi[dst] = hi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t round_n = min(uint32_t(blockDim.x), ch.end - base);
            run_l += round_left;
            run_r += round_n - round_left;
        }
        __syncthreads();
    }
}

__global__ void k_chunk_copy(const Chunk* chunks, const float4* tlo, const float4* thi, float4* plo, float4* phi) {
    const Chunk ch = chunks[blockIdx.x];
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        plo[i] = tlo[i];
        phi[i] = thi[i];
    }
}

// ------------------------------------------------------------ small nodes --
// One block builds the subtree of a node of at most kSmall triangles in
// shared memory, depth first, with the large rounds' rules.
__global__ void __launch_bounds__(kSmallThreads) k_small_build(const SmallSeg* segs, float4* plo, float4* phi,
                                                               uint32_t* node_counter, float4* blo, float4* bhi,
                                                               uint32_t* parent, uint32_t* count, uint32_t* first,
                                                               uint32_t* leaves, uint32_t* leaf_count) {
    __shared__ float4 slo[kSmall], shi[kSmall], tlo[kSmall], thi[kSmall];
    __shared__ uint32_t st_b[kSmall], st_e[kSmall], st_n[kSmall];
    __shared__ uint32_t cnt[kNumBins];
    __shared__ int key[kNumBins][6];
    __shared__ float fbox[kNumBins][6];
    __shared__ float red[12];
    __shared__ SegBounds sb;
    __shared__ Split split;
    __shared__ uint32_t sp, cur_b, cur_e, cur_node, done, warp_sum[kSmallThreads / 32], run_l, run_r;
    const SmallSeg sg = segs[blockIdx.x];
    const uint32_t tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    for (uint32_t i = tid; i < sg.count; i += blockDim.x) {
        slo[i] = plo[sg.begin + i];
        shi[i] = phi[sg.begin + i];
    }
    if (tid == 0) {
        st_b[0] = 0;
        st_e[0] = sg.count;
        st_n[0] = sg.node;
        sp = 1;
    }
    __syncthreads();
    // at most one iteration per node of the subtree (fewer than 2 kSmall)
    for (uint32_t guard = 0; guard < 2 * kSmall; ++guard) {
        if (tid == 0) {
            done = sp == 0 ? 1u : 0u;
            if (sp > 0) {
                --sp;
                cur_b = st_b[sp];
                cur_e = st_e[sp];
                cur_node = st_n[sp];
            }
        }
        __syncthreads();
        if (done) break;
        const uint32_t b = cur_b, e = cur_e, node = cur_node, n = e - b;
        float v[12];
        bounds_init(v);
        for (uint32_t i = b + tid; i < e; i += blockDim.x) bounds_add(v, slo[i], shi[i]);
        block_bounds(v, red);
        if (tid == 0) {
            sb.live = 0;
            for (int k = 0; k < 3; ++k) {
                sb.lo[k] = red[k];
                sb.hi[k] = red[3 + k];
                sb.clo[k] = red[6 + k];
                sb.chi[k] = red[9 + k];
                const float ext = sb.chi[k] - sb.clo[k];
                const bool live = ext > 0.0f;
                sb.scale[k] = live ? float(kSahBins) / ext : 0.0f;
                sb.live |= live ? (1u << k) : 0u;
            }
            blo[node] = make_float4(sb.lo[0], sb.lo[1], sb.lo[2], __uint_as_float(kNil));
            bhi[node] = make_float4(sb.hi[0], sb.hi[1], sb.hi[2], __uint_as_float(kNil));
            count[node] = n;
            first[node] = sg.begin + b;
        }
        for (int j = tid; j < kNumBins; j += blockDim.x) {
            cnt[j] = 0;
            for (int k = 0; k < 3; ++k) {
                key[j][k] = fkey(kFltMax);
                key[j][3 + k] = fkey(-kFltMax);
            }
        }
        __syncthreads();
        if (n > 1) {
            for (uint32_t i = b + tid; i < e; i += blockDim.x) {
                const float4 lo = slo[i], hi = shi[i];
                const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
                for (int a = 0; a < 3; ++a) {
                    if (!((sb.live >> a) & 1u)) continue;
                    const int j = a * kSahBins + bin_of(0.5f * (l[a] + h[a]), sb.clo[a], sb.scale[a]);
                    atomicAdd(&cnt[j], 1u);
                    for (int k = 0; k < 3; ++k) {
                        atomicMin(&key[j][k], fkey(l[k]));
                        atomicMax(&key[j][3 + k], fkey(h[k]));
                    }
                }
            }
        }
        __syncthreads();
        for (int j = tid; j < kNumBins; j += blockDim.x)
            for (int k = 0; k < 6; ++k) fbox[j][k] = fval(key[j][k]);
        __syncthreads();
        uint32_t left = 0;
        Split chosen{};
        if (warp == 0) chosen = choose_split_warp(sb, cnt, fbox, b, n, &left);
        if (tid == 0) {
            split = chosen;
            if (split.mode == 0) {
                leaves[atomicAdd(leaf_count, 1u)] = node;
            } else {
                const uint32_t l = atomicAdd(node_counter, 2u), r = l + 1;
                blo[node].w = __uint_as_float(l);
                bhi[node].w = __uint_as_float(r);
                parent[l] = node;
                parent[r] = node;
                // right below left on the stack: the left subtree builds first
                if (sp + 2 <= kSmall) {
                    st_b[sp] = b + left; st_e[sp] = e; st_n[sp] = r; ++sp;
                    st_b[sp] = b; st_e[sp] = b + left; st_n[sp] = l; ++sp;
                }
            }
            run_l = run_r = 0;
        }
        __syncthreads();
        if (split.mode != 1) continue;  // a leaf or a split by position: nothing moves
        // stable partition of [b, e) through tlo / thi, rounds of blockDim triangles
        const uint32_t mid = split.mid;
        for (uint32_t base = b; base < e; base += blockDim.x) {
            const uint32_t i = base + tid;
            const bool valid = i < e;
            const bool left = valid && goes_left(split, sb, slo[i], shi[i], i);
            const unsigned ball = __ballot_sync(0xFFFFFFFFu, left);
            const uint32_t before = __popc(ball & ((1u << lane) - 1u));
            if (lane == 0) warp_sum[warp] = __popc(ball);
            __syncthreads();
            uint32_t wb = 0, rl = 0;
            for (int w = 0; w < kSmallThreads / 32; ++w) {
                if (w < warp) wb += warp_sum[w];
                rl += warp_sum[w];
            }
            const uint32_t lrank = wb + before;
            if (valid) {
                const uint32_t dst = left ? b + run_l + lrank : mid + run_r + (tid - lrank);
                tlo[dst] = slo[i];
                thi[dst] = shi[i];
            }
            __syncthreads();
            if (tid == 0) {
                const uint32_t rn = min(uint32_t(blockDim.x), e - base);
                run_l += rl;
                run_r += rn - rl;
            }
            __syncthreads();
        }
        for (uint32_t i = b + tid; i < e; i += blockDim.x) {
            slo[i] = tlo[i];
            shi[i] = thi[i];
        }
        __syncthreads();
    }
    __syncthreads();
    for (uint32_t i = tid; i < sg.count; i += blockDim.x) {
        plo[sg.begin + i] = slo[i];
        phi[sg.begin + i] = shi[i];
    }
}

// --------------------------------------------------------------- collapse --
__device__ __forceinline__ float node_half_area(float4 lo, float4 hi) {
    const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
    return box_half_area(l, h);
}

// Collapse costs from the binary leaves up (wide_collapse.cuh).
__global__ void k_sah_bottom_up(const uint32_t* leaves, const uint32_t* leaf_count, uint32_t root, uint32_t max_steps,
                                const uint32_t* parent, const float4* blo, const float4* bhi, const uint32_t* count,
                                WideCost* cost, uint32_t* visits) {
    const uint32_t nl = *leaf_count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x) {
        uint32_t node = leaves[i];
        cost[node] = wide_cost_leaf(node_half_area(blo[node], bhi[node]), count[node]);
        for (uint32_t guard = 0; node != root && guard < max_steps; ++guard) {
            const uint32_t p = parent[node];
            if (p >= max_steps) break;  // no parent recorded: a broken tree, refused by the collapse check
            __threadfence();
            if (atomicAdd(visits + p, 1u) == 0u) break;  // the sibling's thread continues
            __threadfence();
            const float4 pl = blo[p], ph = bhi[p];
            const uint32_t l = __float_as_uint(pl.w), r = __float_as_uint(ph.w);
            if (l >= max_steps || r >= max_steps) break;
            WideCost L, R;
            for (int k = 0; k < 4; ++k) {
                L.cost[k] = __ldcg(&cost[l].cost[k]);
                R.cost[k] = __ldcg(&cost[r].cost[k]);
            }
            L.split = __ldcg(&cost[l].split);
            R.split = __ldcg(&cost[r].split);
            L.leaf = R.leaf = 0;
            cost[p] = wide_cost_inner(node_half_area(pl, ph), count[p], L, R);
            node = p;
        }
    }
}

struct Item {
    uint32_t bnode, wide;
};

// Node ids are checked against the node count (nn): a broken tree sets *bad
// instead of reading out of range.
__global__ void k_sah_select(const Item* items, uint32_t ni, uint32_t nn, const float4* blo, const float4* bhi,
                             const WideCost* cost, uint4* kids, uint32_t* nkids, uint32_t* inner, uint32_t* bad) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        const uint32_t b = items[i].bnode;
        uint32_t k[4] = {kNil, kNil, kNil, kNil};
        int nk = 0;
        auto ok = [&](uint32_t x) {
            if (x < nn) return x;
            *bad = 1u;
            return 0u;
        };
        if (cost[b].leaf) {
            k[nk++] = b;  // a root that is one leaf
        } else {
            nk = wide_slots(
                ok(__float_as_uint(blo[b].w)), ok(__float_as_uint(bhi[b].w)), [&](uint32_t x) { return cost[x]; },
                [&](uint32_t x) { return ok(__float_as_uint(blo[x].w)); },
                [&](uint32_t x) { return ok(__float_as_uint(bhi[x].w)); }, k);
        }
        uint32_t in = 0;
        for (int j = 0; j < nk; ++j) in += cost[k[j]].leaf ? 0u : 1u;
        kids[i] = make_uint4(k[0], k[1], k[2], k[3]);
        nkids[i] = uint32_t(nk);
        inner[i] = in;
    }
}

// Leaves keep their triangle ranges (a binary subtree's triangles are
// contiguous after the in-place partitions).
__global__ void k_sah_emit(const Item* items, uint32_t ni, const uint4* kids, const uint32_t* nkids,
                           const uint32_t* slots, uint32_t wide_base, Item* next, Bvh4Node* nodes,
                           const uint32_t* count, const uint32_t* first, const WideCost* cost, const float4* blo,
                           const float4* bhi) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
        const Item it = items[i];
        const uint4 k4 = kids[i];
        const uint32_t k[4] = {k4.x, k4.y, k4.z, k4.w};
        const int nk = int(nkids[i]);
        uint32_t slot = slots[i];
        float lo[4][3] = {}, hi[4][3] = {};
        uint32_t child[4] = {0, 0, 0, 0};
        for (int j = 0; j < nk; ++j) {
            const uint32_t c = k[j];
            const float4 l = blo[c], h = bhi[c];
            lo[j][0] = l.x; lo[j][1] = l.y; lo[j][2] = l.z;
            hi[j][0] = h.x; hi[j][1] = h.y; hi[j][2] = h.z;
            if (cost[c].leaf) {
                child[j] = make_leaf(first[c], count[c]);
            } else {
                child[j] = wide_base + slot;
                next[slot] = Item{c, wide_base + slot};
                ++slot;
            }
        }
        Bvh4Node wn;
        quantize_node(lo, hi, child, nk, &wn);
        nodes[it.wide] = wn;
    }
}

__global__ void k_sah_order(const float4* plo, uint32_t n, uint32_t* order) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        order[i] = __float_as_uint(plo[i].w);
}

// ---------------------------------------------------------------- host side --
struct SahPool {
    std::vector<void*> blocks;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* get(size_t count) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err == cudaSuccess) blocks.push_back(p);
        return static_cast<T*>(p);
    }
    ~SahPool() {
        for (void* p : blocks) cudaFree(p);
    }
};

int sah_grid(uint64_t work, int block = 256) {
    return int(std::max<uint64_t>(1, std::min<uint64_t>((work + block - 1) / block, 1u << 20)));
}

}  // namespace

bool build_bvh4_gpu_sah(const float* tri_vertices, uint32_t n, cudaStream_t s, Bvh4Result* out, std::string* err) {
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
    const uint32_t seg_cap = n / kSmall + 2;
    const uint32_t chunk_cap = n / kChunk + seg_cap + 2;
    const size_t nnodes = size_t(2) * n;
    SahPool P;
    float* tv = P.get<float>(size_t(n) * 9);
    float4* plo = P.get<float4>(n);
    float4* phi = P.get<float4>(n);
    float4* tlo = P.get<float4>(n);
    float4* thi = P.get<float4>(n);
    float4* blo = P.get<float4>(nnodes);
    float4* bhi = P.get<float4>(nnodes);
    uint32_t* parent = P.get<uint32_t>(nnodes);
    uint32_t* count = P.get<uint32_t>(nnodes);
    uint32_t* first = P.get<uint32_t>(nnodes);
    WideCost* cost = P.get<WideCost>(nnodes);
    uint32_t* visits = P.get<uint32_t>(nnodes);
    uint32_t* leaves = P.get<uint32_t>(n);
    uint32_t* counters = P.get<uint32_t>(4);  // node counter, leaves, next large nodes, small nodes
    SegInfo* segs = P.get<SegInfo>(seg_cap);
    SegInfo* next = P.get<SegInfo>(seg_cap);
    Chunk* chunks = P.get<Chunk>(chunk_cap);
    float* cbounds = P.get<float>(size_t(chunk_cap) * 12);
    SegBounds* sbs = P.get<SegBounds>(seg_cap);
    uint32_t* bcnt = P.get<uint32_t>(size_t(chunk_cap) * kNumBins);
    int* bkey = P.get<int>(size_t(chunk_cap) * kNumBins * 6);
    Split* splits = P.get<Split>(seg_cap);
    uint32_t* chunk_left = P.get<uint32_t>(chunk_cap);
    uint32_t* lbase = P.get<uint32_t>(chunk_cap);
    uint32_t* rbase = P.get<uint32_t>(chunk_cap);
    SmallSeg* small = P.get<SmallSeg>(n);
    Item* items[2] = {P.get<Item>(n), P.get<Item>(n)};
    uint4* kids = P.get<uint4>(n);
    uint32_t* nkids = P.get<uint32_t>(n);
    uint32_t* inner = P.get<uint32_t>(n);
    uint32_t* sums = P.get<uint32_t>(scan_scratch(n));
    Bvh4Node* nodes = P.get<Bvh4Node>(n);
    uint32_t* order = P.get<uint32_t>(n);
    if (P.err != cudaSuccess) {
        *err = std::string("GPU SAH build: ") + cudaGetErrorString(P.err);
        return false;
    }
    auto failed = [&](const char* what) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) return false;
        *err = std::string("GPU SAH build (") + what + "): " + cudaGetErrorString(e);
        return true;
    };
    // node arrays start as zeros (parent as none): no entry is ever read uninitialised
    cudaMemsetAsync(blo, 0, nnodes * sizeof(float4), s);
    cudaMemsetAsync(bhi, 0, nnodes * sizeof(float4), s);
    cudaMemsetAsync(count, 0, nnodes * sizeof(uint32_t), s);
    cudaMemsetAsync(first, 0, nnodes * sizeof(uint32_t), s);
    cudaMemsetAsync(cost, 0, nnodes * sizeof(WideCost), s);
    cudaMemsetAsync(parent, 0xFF, nnodes * sizeof(uint32_t), s);
    cudaMemcpyAsync(tv, tri_vertices, size_t(n) * 9 * sizeof(float), cudaMemcpyHostToDevice, s);
    k_sah_init<<<sah_grid(n), 256, 0, s>>>(tv, n, plo, phi);
    // the root
    const uint32_t root_info[3] = {n, 0u, kNil};
    cudaMemcpyAsync(count, &root_info[0], 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(first, &root_info[1], 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(parent, &root_info[2], 4, cudaMemcpyHostToDevice, s);
    std::vector<SegInfo> cur;
    uint32_t host_counters[4] = {1u, 0u, 0u, 0u};
    if (n > kSmall) {
        cur.push_back(SegInfo{0, n, 0, 0, 0, {0, 0, 0}});
    } else {
        const SmallSeg r{0, n, 0, 0};
        cudaMemcpyAsync(small, &r, sizeof(r), cudaMemcpyHostToDevice, s);
        host_counters[3] = 1;
    }
    cudaMemcpyAsync(counters, host_counters, sizeof(host_counters), cudaMemcpyHostToDevice, s);
    // large nodes, one level per round (a round splits every node: at most n rounds)
    std::vector<Chunk> hchunks;
    for (uint32_t round = 0; !cur.empty(); ++round) {
        if (round > n) {
            *err = "GPU SAH build: too many rounds";
            return false;
        }
        hchunks.clear();
        for (size_t k = 0; k < cur.size(); ++k) {
            SegInfo& g = cur[k];
            g.chunk0 = uint32_t(hchunks.size());
            for (uint32_t b = g.begin; b < g.begin + g.count; b += kChunk)
                hchunks.push_back(Chunk{uint32_t(k), b, std::min(b + kChunk, g.begin + g.count), 0});
            g.nchunks = uint32_t(hchunks.size()) - g.chunk0;
        }
        const uint32_t nseg = uint32_t(cur.size()), nch = uint32_t(hchunks.size());
        if (nseg > seg_cap || nch > chunk_cap) {
            *err = "GPU SAH build: round larger than its buffers";
            return false;
        }
        cudaMemcpyAsync(segs, cur.data(), nseg * sizeof(SegInfo), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(chunks, hchunks.data(), nch * sizeof(Chunk), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(counters + 2, 0, sizeof(uint32_t), s);
        k_chunk_bounds<<<nch, 256, 0, s>>>(chunks, plo, phi, cbounds);
        k_seg_bounds<<<nseg, 256, 0, s>>>(segs, cbounds, sbs, blo, bhi);
        k_chunk_bins<<<nch, 256, 0, s>>>(chunks, sbs, plo, phi, bcnt, bkey);
        k_seg_split<<<nseg, kNumBins, 0, s>>>(segs, sbs, bcnt, bkey, splits, counters, blo, bhi, parent, count, first,
                                              leaves, counters + 1, next, counters + 2, small, counters + 3);
        k_chunk_count<<<nch, 256, 0, s>>>(chunks, sbs, splits, plo, phi, chunk_left);
        k_seg_offsets<<<sah_grid(nseg, 128), 128, 0, s>>>(segs, nseg, chunks, chunk_left, lbase, rbase);
        k_chunk_scatter<<<nch, 256, 0, s>>>(chunks, segs, sbs, splits, lbase, rbase, plo, phi, tlo, thi);
        k_chunk_copy<<<nch, 256, 0, s>>>(chunks, tlo, thi, plo, phi);
        uint32_t nn = 0;
        cudaMemcpyAsync(&nn, counters + 2, sizeof(nn), cudaMemcpyDeviceToHost, s);
        if (failed("large nodes")) return false;
        if (nn > seg_cap) {
            *err = "GPU SAH build: too many large nodes";
            return false;
        }
        cur.resize(nn);
        if (nn) cudaMemcpyAsync(cur.data(), next, nn * sizeof(SegInfo), cudaMemcpyDeviceToHost, s);
        if (failed("large nodes")) return false;
    }
    // small nodes: one block each
    cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost, s);
    if (failed("counters")) return false;
    if (host_counters[3] > 0) k_small_build<<<host_counters[3], kSmallThreads, 0, s>>>(small, plo, phi, counters, blo, bhi,
                                                                                     parent, count, first, leaves,
                                                                                     counters + 1);
    cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost, s);
    if (failed("small nodes")) return false;
    if (host_counters[0] > nnodes || host_counters[1] > n) {
        *err = "GPU SAH build: node count out of range";
        return false;
    }
    cudaMemsetAsync(visits, 0, nnodes * sizeof(uint32_t), s);
    cudaMemsetAsync(counters + 2, 0, sizeof(uint32_t), s);  // from here: the broken-tree flag
    k_sah_bottom_up<<<sah_grid(host_counters[1]), 256, 0, s>>>(leaves, counters + 1, 0u, uint32_t(nnodes), parent, blo,
                                                                bhi, count, cost, visits);
    // top-down, one wide level per round
    const Item first_item{0, 0};
    cudaMemcpyAsync(items[0], &first_item, sizeof(Item), cudaMemcpyHostToDevice, s);
    uint32_t ni = 1, wide_count = 1;
    int depth = 0, ci = 0;
    while (ni > 0) {
        ++depth;
        k_sah_select<<<sah_grid(ni), 256, 0, s>>>(items[ci], ni, host_counters[0], blo, bhi, cost, kids, nkids, inner,
                                                  counters + 2);
        uint32_t last_inner = 0, last_slot = 0;
        cudaMemcpyAsync(&last_inner, inner + (ni - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        exclusive_scan(inner, ni, sums, s);
        cudaMemcpyAsync(&last_slot, inner + (ni - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        k_sah_emit<<<sah_grid(ni), 256, 0, s>>>(items[ci], ni, kids, nkids, inner, wide_count, items[ci ^ 1], nodes,
                                                count, first, cost, blo, bhi);
        uint32_t broken = 0;
        cudaMemcpyAsync(&broken, counters + 2, sizeof(broken), cudaMemcpyDeviceToHost, s);
        if (failed("collapse")) return false;
        if (broken) {
            *err = "GPU SAH build: broken tree";
            return false;
        }
        const uint32_t next_n = last_slot + last_inner;
        if (uint64_t(wide_count) + next_n > n) {
            *err = "GPU SAH build: wide node count out of range";
            return false;
        }
        wide_count += next_n;
        ni = next_n;
        ci ^= 1;
    }
    k_sah_order<<<sah_grid(n), 256, 0, s>>>(plo, n, order);
    out->nodes.resize(wide_count);
    out->order.resize(n);
    cudaMemcpyAsync(out->nodes.data(), nodes, size_t(wide_count) * sizeof(Bvh4Node), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(out->order.data(), order, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (failed("download")) return false;
    out->wide_depth = depth;
    out->binary_depth = 0;
    return true;
}

}  // namespace cg
