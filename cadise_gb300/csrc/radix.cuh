// Device-wide LSD radix sort of (key, value) pairs and exclusive prefix sum,
// shared by the GPU BVH build (64-bit Morton keys) and the ray reordering of
// the wavefront extend pass (32-bit keys).
//
// Sort: per pass of 8 bits, digit counts per tile of 2048 keys (digit-major,
// so one exclusive scan of the counts gives every tile's first output slot
// per digit), then a stable scatter: each tile in rounds of 256 consecutive
// keys, ranked within a warp by match_any and across the block's warps by
// per-digit counts in shared memory.  The key count may live in device memory
// (n_dev, read by every kernel; grids then cover `tiles` tiles of capacity),
// so the passes can sit in a captured graph.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace cg {

constexpr int kRadixBlock = 256;
constexpr int kRadixItems = 8;
constexpr uint32_t kRadixTile = kRadixBlock * kRadixItems;  // 2048

inline uint32_t radix_tiles(uint64_t n) { return uint32_t((n + kRadixTile - 1) / kRadixTile); }

__device__ __forceinline__ uint32_t radix_count(uint32_t n, const uint32_t* n_dev) { return n_dev ? *n_dev : n; }

template <typename K>
__global__ void k_radix_hist(const K* keys, uint32_t n, const uint32_t* n_dev, int shift, uint32_t* hist) {
    __shared__ uint32_t h[256];
    const uint32_t cnt = radix_count(n, n_dev);
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kRadixTile;
    if (base < cnt) {
        for (int r = 0; r < kRadixItems; ++r) {
            const uint32_t i = base + r * kRadixBlock + threadIdx.x;
            if (i < cnt) atomicAdd(&h[uint32_t(keys[i] >> shift) & 255u], 1u);
        }
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void k_radix_scatter(const K* kin, const uint32_t* vin, K* kout, uint32_t* vout, uint32_t n,
                                const uint32_t* n_dev, int shift, const uint32_t* offs) {
    __shared__ uint32_t wc[kRadixBlock / 32][256];
    __shared__ uint32_t run[256];
    const uint32_t cnt = radix_count(n, n_dev);
    const uint32_t base = blockIdx.x * kRadixTile;
    if (base >= cnt) return;  // the whole block: no barrier is left waiting
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    run[t] = offs[t * gridDim.x + blockIdx.x];
    for (int w = 0; w < kRadixBlock / 32; ++w) wc[w][t] = 0;
    __syncthreads();
    for (int r = 0; r < kRadixItems; ++r) {
        const uint32_t i = base + r * kRadixBlock + t;
        const bool valid = i < cnt;
        const K k = valid ? kin[i] : K(0);
        const uint32_t v = valid ? vin[i] : 0u;
        const int d = valid ? int(uint32_t(k >> shift) & 255u) : 256;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wc[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = run[t];
            for (int w = 0; w < kRadixBlock / 32; ++w) {
                const uint32_t c = wc[w][t];
                wc[w][t] = acc;
                acc += c;
            }
            run[t] = acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wc[warp][d] + uint32_t(rank);
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        for (int w = 0; w < kRadixBlock / 32; ++w) wc[w][t] = 0;
        __syncthreads();
    }
}

// Exclusive scan of one tile of 2048 values in place; the tile's total to sums.
static __global__ void k_scan_tile(uint32_t* data, uint32_t n, uint32_t* sums) {
    __shared__ uint32_t warp_tot[kRadixBlock / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t base = blockIdx.x * kRadixTile + uint32_t(t) * kRadixItems;
    uint32_t v[kRadixItems], local = 0;
    for (int k = 0; k < kRadixItems; ++k) {
        v[k] = base + k < n ? data[base + k] : 0u;
        local += v[k];
    }
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0, total = 0;
    for (int w = 0; w < kRadixBlock / 32; ++w) {
        if (w < warp) wpre += warp_tot[w];
        total += warp_tot[w];
    }
    uint32_t run = wpre + incl - local;
    for (int k = 0; k < kRadixItems; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
    if (t == 0) sums[blockIdx.x] = total;
}

static __global__ void k_scan_add(uint32_t* data, uint32_t n, const uint32_t* offs) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        data[i] += offs[i / kRadixTile];
}

inline int radix_grid(uint64_t work, int block = kRadixBlock) {
    const uint64_t g = (work + block - 1) / block;
    return int(g < 1 ? 1 : (g > (1u << 20) ? (1u << 20) : g));
}

// In-place exclusive scan of n values (n known on the host); `sums` holds
// scan_scratch(n) words.
inline void exclusive_scan(uint32_t* data, uint32_t n, uint32_t* sums, cudaStream_t s) {
    if (n == 0) return;
    const uint32_t nb = radix_tiles(n);
    k_scan_tile<<<nb, kRadixBlock, 0, s>>>(data, n, sums);
    if (nb > 1) {
        exclusive_scan(sums, nb, sums + nb, s);
        k_scan_add<<<radix_grid(n), kRadixBlock, 0, s>>>(data, n, sums);
    }
}

inline size_t scan_scratch(uint64_t n) {
    size_t total = 0;
    while (n > 1) {
        n = (n + kRadixTile - 1) / kRadixTile;
        total += size_t(n);
    }
    return total + 1;
}

// Sorts keys[0] / vals[0] by the low 8 * passes bits (the result is in
// keys[passes & 1] / vals[passes & 1]).  n_dev (optional): the count
// in device memory, at most tiles * 2048; hist holds 256 * tiles words, sums
// scan_scratch(256 * tiles).
template <typename K>
void radix_sort_pairs(K* const keys[2], uint32_t* const vals[2], uint32_t n, const uint32_t* n_dev, uint32_t tiles,
                      int passes, uint32_t* hist, uint32_t* sums, cudaStream_t s) {
    for (int pass = 0; pass < passes; ++pass) {
        const int cur = pass & 1;
        k_radix_hist<K><<<tiles, kRadixBlock, 0, s>>>(keys[cur], n, n_dev, 8 * pass, hist);
        exclusive_scan(hist, tiles * 256, sums, s);
        k_radix_scatter<K><<<tiles, kRadixBlock, 0, s>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, n_dev,
                                                          8 * pass, hist);
    }
}

}  // namespace cg
