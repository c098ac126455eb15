// Autotuner for the wavefront schedule: threads per block of the traversal
// and shade kernels and the number of paths in flight, picked by timing
// wavefront passes of the caller's own scenes (CUDA events on the context
// stream), cached per GPU and scene size as JSON lines.
#include "internal.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

bool valid_tuning(const cgpu_tuning& t) {
    auto ok_block = [](int b) { return b >= 32 && b <= 1024 && b % 32 == 0; };
    return ok_block(t.block_trace) && ok_block(t.block_shade) && (t.traversal >= 0 && t.traversal <= 3) &&
           (t.reorder >= 0 && t.reorder <= 4) && (t.refill_closest >= 0 && t.refill_closest <= 32) &&
           (t.refill_any >= 0 && t.refill_any <= 32);
}

void apply(cgpu_ctx* ctx, const cgpu_tuning& t) {
    const bool realloc = t.max_paths != ctx->tuning.max_paths;
    ctx->tuning = t;
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    ctx->graph_depth = -1;
    if (realloc) cg_free_render_state(ctx);
}

std::string cache_key(cgpu_ctx* ctx, const int32_t* scenes, uint32_t n, uint32_t samples) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, ctx->device);
    uint64_t tris = 0, pix = 0;
    int depth = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const SceneSlot& sl = ctx->scenes[size_t(scenes[i])];
        tris += sl.info.num_triangles;
        pix += uint64_t(sl.width) * sl.height;
        depth = std::max(depth, sl.max_depth);
    }
    std::ostringstream os;
    os << prop.name << "|sm" << prop.multiProcessorCount << "|tris" << tris << "|pix" << pix << "|depth" << depth
       << "|scenes" << n << "|samples" << samples;
    return os.str();
}

bool cache_lookup(const char* path, const std::string& key, cgpu_tuning* out) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        const std::string tag = "\"key\": \"" + key + "\"";
        if (line.find(tag) == std::string::npos) continue;
        cgpu_tuning t{};
        int a = 0, b = 0;
        unsigned c = 0;
        const char* p = std::strstr(line.c_str(), "\"block_trace\":");
        const char* q = std::strstr(line.c_str(), "\"block_shade\":");
        const char* r = std::strstr(line.c_str(), "\"max_paths\":");
        const char* tv = std::strstr(line.c_str(), "\"traversal\":");
        const char* ro = std::strstr(line.c_str(), "\"reorder\":");
        const char* rc = std::strstr(line.c_str(), "\"refill_closest\":");
        const char* ra = std::strstr(line.c_str(), "\"refill_any\":");
        if (!p || !q || !r) continue;
        int trav = 0, reord = 0, refc = 0, refa = 0;
        if (tv) std::sscanf(tv, "\"traversal\": %d", &trav);
        if (ro) std::sscanf(ro, "\"reorder\": %d", &reord);
        if (rc) std::sscanf(rc, "\"refill_closest\": %d", &refc);
        if (ra) std::sscanf(ra, "\"refill_any\": %d", &refa);
        if (std::sscanf(p, "\"block_trace\": %d", &a) != 1 || std::sscanf(q, "\"block_shade\": %d", &b) != 1 ||
            std::sscanf(r, "\"max_paths\": %u", &c) != 1)
            continue;
        t.block_trace = a;
        t.block_shade = b;
        t.max_paths = c;
        t.traversal = trav;
        t.reorder = reord;
        t.refill_closest = refc;
        t.refill_any = refa;
        if (valid_tuning(t)) {
            *out = t;
            found = true;  // the last matching line wins
        }
    }
    return found;
}

}  // namespace

extern "C" {

cgpu_status cgpu_tuning_get(cgpu_ctx* ctx, cgpu_tuning* out) {
    if (!ctx || !out) return CGPU_ERR_INVALID_ARGUMENT;
    *out = ctx->tuning;
    return CGPU_OK;
}

cgpu_status cgpu_tuning_set(cgpu_ctx* ctx, const cgpu_tuning* t) {
    if (!ctx || !t) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_tuning(*t))
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT,
                       "tuning: block sizes must be multiples of 32 in [32, 1024], traversal 0 to 3, reorder 0 to 4, "
                       "refill thresholds 0 to 32");
    cudaStreamSynchronize(ctx->stream);
    apply(ctx, *t);
    return CGPU_OK;
}

cgpu_status cgpu_autotune(cgpu_ctx* ctx, const int32_t* scenes, uint32_t n, uint32_t samples, const char* cache_path,
                          cgpu_tuning* out) {
    if (!ctx || !scenes || n == 0) return CGPU_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; ++i)
        if (scenes[i] < 0 || scenes[i] >= int32_t(ctx->scenes.size()) || !ctx->scenes[size_t(scenes[i])].live)
            return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "autotune: unknown scene id");
    cudaSetDevice(ctx->device);
    if (samples == 0) samples = 1;
    const std::string key = cache_key(ctx, scenes, n, samples);
    cgpu_tuning best = ctx->tuning;
    if (cache_path && cache_lookup(cache_path, key, &best)) {
        cudaStreamSynchronize(ctx->stream);
        apply(ctx, best);
        if (out) *out = best;
        return CGPU_OK;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // The films of the scenes are saved and restored around the timing renders.
    std::vector<std::vector<double>> saved(n);
    for (uint32_t i = 0; i < n; ++i) {
        const SceneSlot& sl = ctx->scenes[size_t(scenes[i])];
        const size_t bytes = size_t(sl.width) * sl.height * 7 * sizeof(double);
        saved[i].resize(bytes / sizeof(double));
        cudaMemcpy(saved[i].data(), sl.film.sum, bytes, cudaMemcpyDeviceToHost);
    }
    auto time_one = [&](const cgpu_tuning& t, float* ms) -> cgpu_status {
        apply(ctx, t);
        cgpu_render_params p{};
        p.scenes = scenes;
        p.num_scenes = n;
        p.first_sample = 0;
        p.num_samples = samples;
        p.seed = 99;
        p.mode = CGPU_MODE_WAVEFRONT;
        p.use_graph = 1;
        cgpu_status st = cg_render_batches(ctx, &p);  // warm (capture + allocation)
        if (st != CGPU_OK) return st;
        // the faster of two timed renders: one render alone is too noisy to
        // separate candidates a few percent apart
        *ms = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            st = cg_render_batches(ctx, &p);
            if (st != CGPU_OK) return st;
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float t = 0.0f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep == 0 || t < *ms) *ms = t;
        }
        return CGPU_OK;
    };
    float best_ms = 0.0f;
    cgpu_status st = time_one(best, &best_ms);
    const int blocks[] = {64, 128, 256};
    // paths in flight: larger batches hold several samples per pixel and
    // share one tail of short late-bounce queues among them
    const uint32_t caps[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24};
    // (ray reordering is not searched: on the 1 M-triangle field its sort costs about what it saves in
    // the closest-hit passes, so the search would pick it by noise)
    // queue compaction of the persistent passes: refill a warp's finished
    // lanes once fewer than this many lanes still trace
    const int refills[] = {8, 16, 24, 28, 32};
    const int options[] = {4, 3, 3, 5, 5, 5};
    for (int pass = 0; pass < 6 && st == CGPU_OK; ++pass) {
        // the thresholds only act in the persistent while-while passes
        if (pass == 4 && best.traversal < 2) continue;
        if (pass == 5 && best.traversal < 3) continue;
        for (int k = 0; k < options[pass] && st == CGPU_OK; ++k) {
            cgpu_tuning t = best;
            if (pass == 0) t.traversal = k;
            if (pass == 1) t.block_trace = blocks[k];
            if (pass == 2) t.block_shade = blocks[k];
            if (pass == 3) t.max_paths = caps[k];
            if (pass == 4) t.refill_closest = refills[k];
            if (pass == 5) t.refill_any = refills[k];
            if (cg::refill_lanes(t.refill_closest) == cg::refill_lanes(best.refill_closest) &&
                cg::refill_lanes(t.refill_any) == cg::refill_lanes(best.refill_any) && pass >= 4)
                continue;
            if (std::memcmp(&t, &best, sizeof(t)) == 0) continue;
            float ms = 0.0f;
            st = time_one(t, &ms);
            if (st == CGPU_OK && ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply(ctx, best);
    for (uint32_t i = 0; i < n; ++i) {
        const SceneSlot& sl = ctx->scenes[size_t(scenes[i])];
        cudaMemcpy(sl.film.sum, saved[i].data(), saved[i].size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (st != CGPU_OK) return st;
    if (cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        f << "{\"key\": \"" << key << "\", \"block_trace\": " << best.block_trace << ", \"block_shade\": "
          << best.block_shade << ", \"max_paths\": " << best.max_paths << ", \"traversal\": " << best.traversal
          << ", \"reorder\": " << best.reorder << ", \"refill_closest\": " << best.refill_closest
          << ", \"refill_any\": " << best.refill_any << ", \"ms\": " << best_ms << "}\n";
    }
    if (out) *out = best;
    return CGPU_OK;
}

}  // extern "C"
