// Library-internal state behind the C ABI (not installed, not part of the ABI).
#pragma once

#include "../../include/cadise_gpu.h"
#include "scene_device.cuh"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace cg {

// One render chunk: samples [sample0, sample0 + nsamples) of every pixel of
// one scene; its paths occupy [path_begin, path_begin + npix * nsamples) of
// the batch, sample-major (path = path_begin + s * npix + pixel).
struct Chunk {
    int scene;
    uint32_t path_begin;
    uint32_t npix;
    uint32_t width;
    uint32_t sample0;
    uint32_t nsamples;
    uint32_t pix_begin;  // prefix over chunks of npix (film splat index space)
    uint32_t pad;
};
constexpr int kMaxChunks = 256;

struct BatchHeader {
    uint32_t num_chunks;
    uint32_t total_paths;
    uint32_t total_pixels;
    int max_depth;
    uint64_t seed;
};

struct FilmD {
    double* sum;    // 3 per pixel
    double* sumsq;  // 3 per pixel
    double* count;  // 1 per pixel
};

// Counters per bounce b at cnt[b * kCntStride + k]:
//   k = 0 continuation rays to extend, 1 MIS rays to extend, 2 shadow rays,
//   3 + kind: hits waiting for the shade kernel of that BSDF kind,
//   8 / 9: rays handed out so far by the persistent extend / shadow kernels,
//   10: adjoint vertices of bounce b - 1 (the wavefront adjoint's gradient kernel),
//   11: MIS rays whose direction meets the sampled light's primitive (or that
//       sampled the environment), left for the MIS occlusion pass,
//   12: closest-hit rays of the persistent pass left for k_wf_ties (q_tie).
constexpr int kCntStride = 16;

struct WfBuffers {
    // L.w and Ls.w hold the sample's film position (x, y) for the film filter;
    // the passes update L and Ls in place and leave .w as it is.
    float4 *ray_o, *ray_d, *hit, *thr, *L, *Ls, *mis_a, *mis_b, *mis_d, *sh_d, *sh_c;
    // Sky radiance picked up by an escaped continuation ray.  Kept apart from
    // L: the MIS ray of the same path's last vertex adds to L in the same
    // extend pass.  A path sample is (L + Le) + Ls.
    float4* Le;
    // MIS ray resolved against its light at the vertex: (t, record slot, u, v)
    // of the light's hit, slot -1 for the environment.
    float4* mis_h;
    uint4* meta;      // scene, pixel, sample, rng counter
    int* q_cont[2];
    int* q_mis[2];
    int* q_shadow[2];
    int* q_mocc[2];   // MIS occlusion queries, ping-pong on the bounce
    int* q_mat[kNumBsdfKinds];
    // closest-hit rays whose persistent traversal met two primitives within
    // the tie window (k_wf_extend_pww), for k_wf_ties: path, | 0x80000000 for
    // a MIS ray; room for every ray of a pass (2 per path)
    int* q_tie;
    int* cnt;
    int cnt_depth;    // bounces the counter array covers
};

// Lays the path state of `cap` paths and the counters of `cnt_rows` bounces
// out from `base` (256-byte aligned arrays) and returns the bytes used.  With
// base == nullptr it only measures: the allocation is sized by the same walk
// that carves it.
inline size_t wf_layout(char* base, size_t cap, int cnt_rows, WfBuffers* w) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* r = base ? base + off : nullptr;
        off += (bytes + 255) & ~size_t(255);
        return r;
    };
    float4** f4s[] = {&w->ray_o, &w->ray_d, &w->hit, &w->thr, &w->L, &w->Le, &w->Ls,
                      &w->mis_a, &w->mis_b, &w->mis_d, &w->mis_h, &w->sh_d, &w->sh_c};
    for (float4** f : f4s) *f = reinterpret_cast<float4*>(take(cap * sizeof(float4)));
    w->meta = reinterpret_cast<uint4*>(take(cap * sizeof(uint4)));
    for (int k = 0; k < 2; ++k) {
        w->q_cont[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
        w->q_mis[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
        w->q_shadow[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
        w->q_mocc[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
    }
    for (int k = 0; k < kNumBsdfKinds; ++k) w->q_mat[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
    w->q_tie = reinterpret_cast<int*>(take(2 * cap * sizeof(int)));
    w->cnt = reinterpret_cast<int*>(take(size_t(cnt_rows) * kCntStride * sizeof(int)));
    w->cnt_depth = cnt_rows;
    return off;
}

// Static scratch of cgpu_render_noalloc: every device buffer of that call
// lives in one file-scope array of kNoAllocScratchBytes, laid out by
// noalloc_layout.  Limits: a frame of at most kNoAllocMaxPaths pixels (one
// path per pixel per batch), max_depth <= kNoAllocMaxDepth, scene ids below
// kNoAllocMaxScenes (the scene and film tables are indexed by scene id).
constexpr uint32_t kNoAllocMaxPaths = 1u << 18;
constexpr int kNoAllocMaxDepth = 62;
constexpr int kNoAllocMaxScenes = 64;
constexpr size_t kNoAllocScratchBytes = size_t(80) << 20;

struct NoAllocView {
    BatchHeader* header;
    Chunk* chunk;
    SceneD* scenes;               // kNoAllocMaxScenes entries
    FilmD* films;                 // kNoAllocMaxScenes entries
    unsigned long long* counters; // 8
    WfBuffers wf;                 // kNoAllocMaxPaths paths, kNoAllocMaxDepth + 2 counter rows
};

inline size_t noalloc_layout(char* base, NoAllocView* v) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* r = base ? base + off : nullptr;
        off += (bytes + 255) & ~size_t(255);
        return r;
    };
    v->header = reinterpret_cast<BatchHeader*>(take(sizeof(BatchHeader)));
    v->chunk = reinterpret_cast<Chunk*>(take(sizeof(Chunk)));
    v->scenes = reinterpret_cast<SceneD*>(take(sizeof(SceneD) * kNoAllocMaxScenes));
    v->films = reinterpret_cast<FilmD*>(take(sizeof(FilmD) * kNoAllocMaxScenes));
    v->counters = reinterpret_cast<unsigned long long*>(take(8 * sizeof(unsigned long long)));
    return off + wf_layout(base ? base + off : nullptr, kNoAllocMaxPaths, kNoAllocMaxDepth + 2, &v->wf);
}

// Wavefront adjoint (path replay in wavefront form): per path the radiance
// of the whole path from a first wavefront pass (Ltot), the radiance of the
// vertices replayed so far (acc), and what one vertex leaves for the gradient
// kernel that runs once its shadow and MIS rays are traced: st_a = textured
// albedo and texel index, st_b = d ln f / d roughness towards the shadow,
// MIS and continuation directions + material | flags, st_c = the shadow
// contribution without the light's radiance + the light; mis_B / mis_X = the
// MIS half and its radiance derivative (with the light) once resolved.
struct AdjBufs {
    float4 *Ltot, *acc, *st_a, *st_b, *st_c, *mis_B, *mis_X;
    int* q_vtx[2];          // paths with a vertex at bounce b, ping-pong on b
    const float* dLdI;      // d loss / d pixel, 3 per pixel
    double* g_tex;
    const int* tex_offset;  // per texture: first float of its block in g_tex
    double* g_rough;        // per material
    double* g_rad;          // 3 per area light
    int nmat, nlight;
    float inv_spp;
};
// st_b.w bits above the 16-bit material index
constexpr uint32_t kAdjShadow = 1u << 16, kAdjMis = 1u << 17, kAdjCont = 1u << 18, kAdjTexel = 1u << 19,
                   kAdjGgx = 1u << 20;

inline size_t adj_layout(char* base, size_t cap, AdjBufs* a) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* r = base ? base + off : nullptr;
        off += (bytes + 255) & ~size_t(255);
        return r;
    };
    float4** f4s[] = {&a->Ltot, &a->acc, &a->st_a, &a->st_b, &a->st_c, &a->mis_B, &a->mis_X};
    for (float4** f : f4s) *f = reinterpret_cast<float4*>(take(cap * sizeof(float4)));
    for (int k = 0; k < 2; ++k) a->q_vtx[k] = reinterpret_cast<int*>(take(cap * sizeof(int)));
    return off;
}

struct RenderArgs {
    const SceneD* scenes;
    const Chunk* chunks;
    const BatchHeader* header;
    FilmD* films;     // per scene id
    WfBuffers wf;
    unsigned long long* counters;  // closest rays, any rays, nodes, tris, paths
    AdjBufs adj;      // wavefront adjoint only
    // reordered closest-hit queue (tuning.reorder): path | 0x80000000 for a MIS ray
    const uint32_t* sorted;
    // persistent traversal passes: a warp refills its finished lanes once
    // fewer than this many of its lanes still trace (cgpu_tuning)
    int refill_closest, refill_any;
};

// The refill thresholds of a tuning, 0 replaced by the default.
constexpr int kDefaultRefillLanes = 24;
inline int refill_lanes(int32_t v) { return v > 0 ? v : kDefaultRefillLanes; }

// Buffers of the ray reordering: keys / values ping-pong for 2 * path_cap
// queue entries, digit counts, scan scratch, the entry count.
struct SortBufs {
    uint32_t* keys[2];
    uint32_t* vals[2];
    uint32_t* hist;
    uint32_t* sums;
    uint32_t* n;
    uint32_t tiles;
};

}  // namespace cg

struct SceneSlot {
    bool live = false;
    cg::SceneD d{};
    // host copies of the differentiable tables (cgpu_params_get / _set)
    std::vector<cg::MaterialD> h_mats;
    std::vector<cg::LightD> h_lights;
    std::vector<cg::TextureD> h_texs;  // device texel pointers
    cg::MaterialD* d_mats = nullptr;
    cg::LightD* d_lights = nullptr;
    int num_area_lights = 0;  // h_lights[0, num_area_lights) are area lights
    std::vector<void*> allocations;
    cgpu_scene_info info{};
    cg::FilmD film{};
    int width = 0, height = 0, spp = 1, max_depth = 1;
    bool has_spheres = false;  // renders of this scene use the kernels with the sphere test
};

struct cgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // second stream for graph branches
    bool own_stream = false;
    std::string last_error;
    std::vector<SceneSlot> scenes;
    int num_sms = 0;
    bool counting = false;
    cgpu_tuning tuning{128, 128, 0, 0, 0, 0, 0};

    // device tables (rebuilt when the scene set changes)
    cg::SceneD* d_scenes = nullptr;
    cg::FilmD* d_films = nullptr;
    int table_cap = 0;
    bool tables_dirty = true;

    // batch description
    cg::Chunk* d_chunks = nullptr;
    cg::BatchHeader* d_header = nullptr;
    cg::Chunk* h_chunks = nullptr;        // pinned
    cg::BatchHeader* h_header = nullptr;  // pinned

    // per-path buffers
    uint32_t path_cap = 0;
    cg::WfBuffers wf{};
    void* wf_block = nullptr;
    // wavefront adjoint state (allocated by the first wavefront adjoint)
    // ray reordering buffers (allocated while tuning.reorder is on)
    uint32_t sort_cap = 0;
    cg::SortBufs sort{};
    void* sort_block = nullptr;
    uint32_t adj_cap = 0;
    cg::AdjBufs adj{};
    void* adj_block = nullptr;
    int adjoint_schedule = CGPU_MODE_WAVEFRONT;
    int bvh_builder = CGPU_BVH_BUILDER_AUTO;
    int tie_order = CGPU_TIE_ORDER_REFERENCE;
    unsigned long long* d_counters = nullptr;
    // device status word: rays whose traversal ran out of its visit budget
    // since the last check (cg_check_status); 0 = automatic budget per scene
    uint32_t* d_status = nullptr;
    uint32_t visit_budget = 0;

    // captured wavefront graph
    cudaGraphExec_t graph = nullptr;
    int graph_depth = -1;
    uint32_t graph_paths = 0;
    bool graph_spheres = false;
    uint32_t graph_launches = 0;  // kernel launches one replay of the graph makes
    bool batch_spheres = false;  // a scene of the current render holds spheres

    cgpu_render_stats stats{};

    // per-kernel event timing (cgpu_set_profiling)
    bool profiling = false;
    struct ProfEvent { int cls; cudaEvent_t a, b; };
    std::vector<ProfEvent> prof;
    cgpu_kernel_times times{};
};

// implemented in render.cu
cgpu_status cg_render_batches(cgpu_ctx* ctx, const cgpu_render_params* p);
cgpu_status cg_adjoint_wavefront(cgpu_ctx* ctx, int scene, uint32_t spp, uint64_t seed, const cg::AdjBufs& params);
cgpu_status cg_render_paths_raw(cgpu_ctx* ctx, int scene, int mode, uint32_t first, uint32_t count, uint64_t seed,
                                float* host_rgb);
cgpu_status cg_path_radiance(cgpu_ctx* ctx, int scene, int mode, const double* film_xy, const uint64_t* keys,
                             uint32_t n, float* out_rgb);
cgpu_status cg_trace(cgpu_ctx* ctx, int scene, const cgpu_ray* d_rays, uint32_t n, cgpu_hit* d_hits,
                     uint8_t* d_occ, bool any);
cgpu_status cg_camera(cgpu_ctx* ctx, int scene, const double* d_xy, uint32_t n, float* d_out);
cgpu_status cg_film_clear(cgpu_ctx* ctx, int scene);
void cg_free_render_state(cgpu_ctx* ctx);

// implemented in api.cu
cgpu_status cg_fail(cgpu_ctx* ctx, cgpu_status s, const std::string& msg);
cgpu_status cg_cuda(cgpu_ctx* ctx, cudaError_t e, const char* what);
cgpu_status cg_sync_tables(cgpu_ctx* ctx);
// After the context stream is synchronised: CGPU_ERR_TIMEOUT (and a reset
// count) if a traversal ran out of its device-side visit budget.
cgpu_status cg_check_status(cgpu_ctx* ctx);
