// C ABI entry points (include/cadise_gpu.h): context, scene upload, ray
// queries, camera rays, render, film.
#include "internal.h"
#include "scene_build.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

using namespace cg;

// ------------------------------------------------------------------ errors --
cgpu_status cg_fail(cgpu_ctx* ctx, cgpu_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

cgpu_status cg_cuda(cgpu_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return CGPU_OK;
    const cgpu_status s = e == cudaErrorMemoryAllocation ? CGPU_ERR_OUT_OF_MEMORY
                          : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? CGPU_ERR_NO_DEVICE
                                                                                          : CGPU_ERR_CUDA;
    return cg_fail(ctx, s, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

template <typename T>
cgpu_status upload(cgpu_ctx* ctx, SceneSlot& sl, const T* host, size_t count, T** dev) {
    *dev = nullptr;
    if (count == 0) return CGPU_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) return cg_cuda(ctx, e, "scene upload");
    sl.allocations.push_back(p);
    e = cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cg_cuda(ctx, e, "scene upload copy");
    *dev = static_cast<T*>(p);
    sl.info.device_bytes += count * sizeof(T);
    return CGPU_OK;
}

void free_slot(SceneSlot& sl) {
    for (void* p : sl.allocations) cudaFree(p);
    sl.allocations.clear();
    sl.live = false;
}

bool check_ctx(cgpu_ctx* ctx) { return ctx != nullptr; }

bool valid_scene(cgpu_ctx* ctx, int32_t s) { return s >= 0 && s < int32_t(ctx->scenes.size()) && ctx->scenes[s].live; }

}  // namespace

cgpu_status cg_check_status(cgpu_ctx* ctx) {
    if (!ctx->d_status) return CGPU_OK;
    uint32_t ran_out = 0;
    cudaError_t e = cudaMemcpyAsync(&ran_out, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cg_cuda(ctx, e, "status read");
    if (ran_out == 0) return CGPU_OK;
    cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    const std::string budget =
        ctx->visit_budget ? std::to_string(ctx->visit_budget) + " node and leaf visits per ray"
                          : "the automatic budget of 5 x nodes + 64 node and leaf visits per ray";
    return cg_fail(ctx, CGPU_ERR_TIMEOUT,
                   std::to_string(ran_out) + " ray traversal(s) ran out of the device-side iteration budget (" +
                       budget + ") and stopped early since the last check: their results are not valid");
}

cgpu_status cg_sync_tables(cgpu_ctx* ctx) {
    if (!ctx->tables_dirty) return CGPU_OK;
    const int n = int(ctx->scenes.size());
    if (n > ctx->table_cap) {
        if (ctx->d_scenes) cudaFree(ctx->d_scenes);
        if (ctx->d_films) cudaFree(ctx->d_films);
        ctx->d_scenes = nullptr;
        ctx->d_films = nullptr;
        const int cap = std::max(8, n * 2);
        cudaError_t e = cudaMalloc(&ctx->d_scenes, sizeof(SceneD) * cap);
        if (e == cudaSuccess) e = cudaMalloc(&ctx->d_films, sizeof(FilmD) * cap);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "scene table");
        ctx->table_cap = cap;
    }
    std::vector<SceneD> sd(size_t(std::max(n, 1)));
    std::vector<FilmD> fd(size_t(std::max(n, 1)));
    for (int i = 0; i < n; ++i) {
        if (ctx->scenes[i].live) {
            sd[i] = ctx->scenes[i].d;
            fd[i] = ctx->scenes[i].film;
        } else {
            std::memset(&sd[i], 0, sizeof(SceneD));
            std::memset(&fd[i], 0, sizeof(FilmD));
        }
    }
    cudaError_t e = cudaMemcpyAsync(ctx->d_scenes, sd.data(), sizeof(SceneD) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->d_films, fd.data(), sizeof(FilmD) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cg_cuda(ctx, e, "scene table upload");
    ctx->tables_dirty = false;
    return CGPU_OK;
}

extern "C" {

int32_t cgpu_abi_version(void) { return CGPU_ABI_VERSION; }

const char* cgpu_status_string(cgpu_status s) {
    switch (s) {
        case CGPU_OK: return "CGPU_OK";
        case CGPU_ERR_INVALID_ARGUMENT: return "CGPU_ERR_INVALID_ARGUMENT";
        case CGPU_ERR_CUDA: return "CGPU_ERR_CUDA";
        case CGPU_ERR_OUT_OF_MEMORY: return "CGPU_ERR_OUT_OF_MEMORY";
        case CGPU_ERR_TIMEOUT: return "CGPU_ERR_TIMEOUT";
        case CGPU_ERR_UNSUPPORTED: return "CGPU_ERR_UNSUPPORTED";
        case CGPU_ERR_NOT_FOUND: return "CGPU_ERR_NOT_FOUND";
        case CGPU_ERR_PARSE: return "CGPU_ERR_PARSE";
        case CGPU_ERR_NO_DEVICE: return "CGPU_ERR_NO_DEVICE";
    }
    return "CGPU_ERR_UNKNOWN";
}

const char* cgpu_last_error(const cgpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

cgpu_status cgpu_create(cgpu_ctx** out_ctx, const cgpu_options* options) {
    if (!out_ctx) return CGPU_ERR_INVALID_ARGUMENT;
    *out_ctx = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return CGPU_ERR_NO_DEVICE;
    cgpu_ctx* ctx = new (std::nothrow) cgpu_ctx();
    if (!ctx) return CGPU_ERR_OUT_OF_MEMORY;
    ctx->device = options ? options->device : 0;
    if (ctx->device < 0 || ctx->device >= count) {
        delete ctx;
        return CGPU_ERR_INVALID_ARGUMENT;
    }
    e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) {
        if (options && options->stream) {
            ctx->stream = static_cast<cudaStream_t>(options->stream);
        } else {
            e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
            ctx->own_stream = true;
        }
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, 4 * sizeof(uint32_t));
    if (e != cudaSuccess) {
        if (ctx->d_status) cudaFree(ctx->d_status);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return CGPU_ERR_CUDA;
    }
    ctx->tuning.max_paths = options ? options->max_paths : 0;
    *out_ctx = ctx;
    return CGPU_OK;
}

void cgpu_destroy(cgpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cg_free_render_state(ctx);
    for (SceneSlot& sl : ctx->scenes) free_slot(sl);
    if (ctx->d_scenes) cudaFree(ctx->d_scenes);
    if (ctx->d_films) cudaFree(ctx->d_films);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_chunks) cudaFree(ctx->d_chunks);
    if (ctx->d_header) cudaFree(ctx->d_header);
    if (ctx->h_chunks) cudaFreeHost(ctx->h_chunks);
    if (ctx->h_header) cudaFreeHost(ctx->h_header);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

cgpu_status cgpu_synchronize(cgpu_ctx* ctx) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    const cgpu_status st = cg_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
    return st != CGPU_OK ? st : cg_check_status(ctx);
}

cgpu_status cgpu_set_visit_budget(cgpu_ctx* ctx, uint32_t visits) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(ctx->stream);
    ctx->visit_budget = visits;
    for (SceneSlot& sl : ctx->scenes)
        if (sl.live) sl.d.visit_budget = visits ? visits : auto_visit_budget(sl.info.num_bvh_nodes);
    ctx->tables_dirty = true;
    return CGPU_OK;
}

cgpu_status cgpu_set_tie_order(cgpu_ctx* ctx, int32_t order) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (order != CGPU_TIE_ORDER_REFERENCE && order != CGPU_TIE_ORDER_INDEX)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "set_tie_order: unknown order");
    ctx->tie_order = order;
    return CGPU_OK;
}

cgpu_status cgpu_set_bvh_builder(cgpu_ctx* ctx, int32_t builder) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (builder < CGPU_BVH_BUILDER_AUTO || builder > CGPU_BVH_BUILDER_GPU_SAH)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "set_bvh_builder: unknown builder");
    ctx->bvh_builder = builder;
    return CGPU_OK;
}

namespace {
bool gpu_ploc_builder(const float* tv, uint32_t n, Bvh4Result* out, std::string* err, void* user) {
    return build_bvh4_gpu(tv, n, static_cast<cgpu_ctx*>(user)->stream, out, err);
}
bool gpu_sah_builder(const float* tv, uint32_t n, Bvh4Result* out, std::string* err, void* user) {
    return build_bvh4_gpu_sah(tv, n, static_cast<cgpu_ctx*>(user)->stream, out, err);
}
}  // namespace

cgpu_status cgpu_scene_upload(cgpu_ctx* ctx, const cgpu_scene_desc* d, int32_t* out_scene) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!d || !out_scene) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: null argument");
    cudaSetDevice(ctx->device);
    const auto t0 = std::chrono::steady_clock::now();
    HostScene hs;
    std::string err;
    // AUTO: the PLOC tree renders 12-25 % slower, which its build time (0.08 s for 20 M triangles,
    // against 0.5 s for the SAH build on the GPU) outweighs only above ~0.01 primitives per path
    // sample of a full render; else the SAH tree, built on the GPU from 65,536 primitives up
    const double samples = double(d->width) * double(d->height) * double(d->spp > 0 ? d->spp : 1);
    int builder = ctx->bvh_builder;
    if (builder == CGPU_BVH_BUILDER_AUTO)
        builder = d->num_primitives >= CGPU_BVH_GPU_MIN_PRIMITIVES &&
                          double(d->num_primitives) > CGPU_BVH_GPU_MIN_PRIMS_PER_SAMPLE * samples
                      ? CGPU_BVH_BUILDER_GPU_PLOC
                  : d->num_primitives >= CGPU_BVH_GPU_SAH_MIN_PRIMITIVES ? CGPU_BVH_BUILDER_GPU_SAH
                                                                         : CGPU_BVH_BUILDER_HOST_SAH;
    const bool ranks = ctx->tie_order == CGPU_TIE_ORDER_REFERENCE;
    cgpu_status st = builder == CGPU_BVH_BUILDER_GPU_PLOC  ? build_host_scene(d, &hs, &err, gpu_ploc_builder, ctx, ranks)
                     : builder == CGPU_BVH_BUILDER_GPU_SAH ? build_host_scene(d, &hs, &err, gpu_sah_builder, ctx, ranks)
                                                           : build_host_scene(d, &hs, &err, nullptr, nullptr, ranks);
    if (st != CGPU_OK) return cg_fail(ctx, st, "scene_upload: " + err);
    hs.info.bvh_builder = builder;
    if (3 * hs.wide_depth + 1 > kStackSize)
        return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "scene_upload: BVH too deep for the traversal stack");
    SceneSlot sl;
    sl.info = hs.info;
    // textures first: the texture table holds their device pointers
    std::vector<TextureD> texs = hs.textures;
    for (size_t i = 0; i < texs.size() && st == CGPU_OK; ++i) {
        float* dev = nullptr;
        st = upload(ctx, sl, texs[i].texels, size_t(texs[i].width) * texs[i].height * 3, &dev);
        texs[i].texels = dev;
    }
    if (st == CGPU_OK && hs.env_light >= 0) {
        float *dm_cdf = nullptr, *dc_cdf = nullptr;
        st = upload(ctx, sl, hs.env_marg.data(), hs.env_marg.size(), &dm_cdf);
        if (st == CGPU_OK) st = upload(ctx, sl, hs.env_cond.data(), hs.env_cond.size(), &dc_cdf);
        hs.lights[size_t(hs.env_light)].marg_cdf = dm_cdf;
        hs.lights[size_t(hs.env_light)].cond_cdf = dc_cdf;
    }
    const uint32_t np = d->num_primitives;
    Bvh4Node* dn = nullptr;
    TriRecord* dt = nullptr;
    MaterialD* dm = nullptr;
    LightD* dl = nullptr;
    TextureD* dtex = nullptr;
    float *dnorm = nullptr, *duvw = nullptr, *drect = nullptr;
    if (st == CGPU_OK) st = upload(ctx, sl, hs.nodes.data(), hs.nodes.size(), &dn);
    if (st == CGPU_OK) st = upload(ctx, sl, hs.tris.data(), hs.tris.size(), &dt);
    if (st == CGPU_OK) st = upload(ctx, sl, hs.mats.data(), hs.mats.size(), &dm);
    if (st == CGPU_OK) st = upload(ctx, sl, hs.lights.data(), hs.lights.size(), &dl);
    if (st == CGPU_OK) st = upload(ctx, sl, texs.data(), texs.size(), &dtex);
    if (st == CGPU_OK && d->prim_normals) st = upload(ctx, sl, d->prim_normals, size_t(np) * 9, &dnorm);
    if (st == CGPU_OK && d->prim_uvws) st = upload(ctx, sl, d->prim_uvws, size_t(np) * 9, &duvw);
    if (st == CGPU_OK) st = upload(ctx, sl, hs.rect_frames.data(), hs.rect_frames.size(), &drect);
    uint32_t* drank = nullptr;
    if (st == CGPU_OK) st = upload(ctx, sl, hs.prim_rank.data(), hs.prim_rank.size(), &drank);
    float* dlcdf = nullptr;
    if (st == CGPU_OK && !hs.light_cdf.empty()) st = upload(ctx, sl, hs.light_cdf.data(), hs.light_cdf.size(), &dlcdf);
    const size_t npix = size_t(d->width) * size_t(d->height);
    double* film = nullptr;
    if (st == CGPU_OK) {
        cudaError_t e = cudaMalloc(&film, npix * 7 * sizeof(double));
        if (e != cudaSuccess) st = cg_cuda(ctx, e, "film");
        else {
            sl.allocations.push_back(film);
            e = cudaMemset(film, 0, npix * 7 * sizeof(double));
            if (e != cudaSuccess) st = cg_cuda(ctx, e, "film clear");
        }
    }
    if (st != CGPU_OK) {
        free_slot(sl);
        return st;
    }
    sl.film = FilmD{film, film + 3 * npix, film + 6 * npix};
    sl.h_mats = hs.mats;
    sl.h_lights = hs.lights;
    sl.h_texs = texs;
    sl.d_mats = dm;
    sl.d_lights = dl;
    sl.num_area_lights = hs.num_area_lights;
    SceneD& S = sl.d;
    S.nodes = dn;
    S.tris = dt;
    S.materials = dm;
    S.lights = dl;
    S.textures = dtex;
    S.prim_normals = dnorm;
    S.prim_uvws = duvw;
    S.rect_frames = drect;
    S.prim_rank = drank;
    S.light_cdf = dlcdf;
    S.num_lights = int(hs.lights.size());
    S.env_light = hs.env_light;
    S.num_tris = int(hs.tris.size());
    S.width = d->width;
    S.height = d->height;
    S.max_depth = d->max_depth;
    S.spp = d->spp > 0 ? d->spp : 1;
    S.cam = hs.cam;
    S.filter = hs.filter;
    S.visit_budget = ctx->visit_budget ? ctx->visit_budget : auto_visit_budget(hs.nodes.size());
    S.status = ctx->d_status;
    {
        const float c[3] = {hs.cam.pos.x, hs.cam.pos.y, hs.cam.pos.z};
        S.tie_abs = tie_window_abs(hs.info.bounds_min, hs.info.bounds_max, c);
    }
    S.bounds_lo = make_float3(hs.info.bounds_min[0], hs.info.bounds_min[1], hs.info.bounds_min[2]);
    {
        float inv[3];
        for (int k = 0; k < 3; ++k) {
            const float e = hs.info.bounds_max[k] - hs.info.bounds_min[k];
            inv[k] = e > 0.0f ? 1.0f / e : 0.0f;
        }
        S.bounds_inv = make_float3(inv[0], inv[1], inv[2]);
    }
    sl.width = d->width;
    sl.height = d->height;
    sl.spp = S.spp;
    sl.max_depth = d->max_depth;
    sl.has_spheres = hs.has_spheres;
    sl.live = true;
    sl.info.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int id = -1;
    for (size_t i = 0; i < ctx->scenes.size(); ++i)
        if (!ctx->scenes[i].live) { id = int(i); break; }
    if (id < 0) {
        id = int(ctx->scenes.size());
        ctx->scenes.push_back(SceneSlot());
    }
    ctx->scenes[size_t(id)] = std::move(sl);
    ctx->tables_dirty = true;
    *out_scene = id;
    return CGPU_OK;
}

cgpu_status cgpu_scene_release(cgpu_ctx* ctx, int32_t scene) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "scene_release: unknown scene id");
    cudaStreamSynchronize(ctx->stream);
    free_slot(ctx->scenes[size_t(scene)]);
    ctx->tables_dirty = true;
    return CGPU_OK;
}

cgpu_status cgpu_scene_info_get(cgpu_ctx* ctx, int32_t scene, cgpu_scene_info* out) {
    if (!check_ctx(ctx) || !out) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "scene_info: unknown scene id");
    *out = ctx->scenes[size_t(scene)].info;
    return CGPU_OK;
}

static cgpu_status trace_host(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* rays, uint32_t n, cgpu_hit* hits,
                              uint8_t* occ, bool any) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "trace: unknown scene id");
    if (n == 0) return CGPU_OK;
    if (!rays || (any ? !occ : !hits)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "trace: null buffer");
    cudaSetDevice(ctx->device);
    cgpu_ray* dr = nullptr;
    void* dout = nullptr;
    const size_t out_bytes = any ? size_t(n) : size_t(n) * sizeof(cgpu_hit);
    cudaError_t e = cudaMalloc(&dr, size_t(n) * sizeof(cgpu_ray));
    if (e == cudaSuccess) e = cudaMalloc(&dout, out_bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dr, rays, size_t(n) * sizeof(cgpu_ray), cudaMemcpyHostToDevice, ctx->stream);
    cgpu_status st = cg_cuda(ctx, e, "trace buffers");
    if (st == CGPU_OK)
        st = cg_trace(ctx, scene, dr, n, any ? nullptr : static_cast<cgpu_hit*>(dout), any ? static_cast<uint8_t*>(dout) : nullptr, any);
    if (st == CGPU_OK) {
        e = cudaMemcpyAsync(any ? static_cast<void*>(occ) : static_cast<void*>(hits), dout, out_bytes, cudaMemcpyDeviceToHost,
                            ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        st = cg_cuda(ctx, e, "trace readback");
    }
    cudaFree(dr);
    cudaFree(dout);
    return st != CGPU_OK ? st : cg_check_status(ctx);
}

cgpu_status cgpu_trace_closest(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* rays, uint32_t n, cgpu_hit* hits) {
    return trace_host(ctx, scene, rays, n, hits, nullptr, false);
}

cgpu_status cgpu_trace_any(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* rays, uint32_t n, uint8_t* occluded) {
    return trace_host(ctx, scene, rays, n, nullptr, occluded, true);
}

cgpu_status cgpu_trace_closest_device(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* d_rays, uint32_t n, cgpu_hit* d_hits) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "trace: unknown scene id");
    if (n && (!d_rays || !d_hits)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "trace: null buffer");
    return cg_trace(ctx, scene, d_rays, n, d_hits, nullptr, false);
}

cgpu_status cgpu_trace_any_device(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* d_rays, uint32_t n, uint8_t* d_occ) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "trace: unknown scene id");
    if (n && (!d_rays || !d_occ)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "trace: null buffer");
    return cg_trace(ctx, scene, d_rays, n, nullptr, d_occ, true);
}

cgpu_status cgpu_camera_rays(cgpu_ctx* ctx, int32_t scene, const double* film_xy, uint32_t n, float* out) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "camera_rays: unknown scene id");
    if (n == 0) return CGPU_OK;
    if (!film_xy || !out) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "camera_rays: null buffer");
    double* dxy = nullptr;
    float* dout = nullptr;
    cudaError_t e = cudaMalloc(&dxy, size_t(n) * 16);
    if (e == cudaSuccess) e = cudaMalloc(&dout, size_t(n) * 24);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dxy, film_xy, size_t(n) * 16, cudaMemcpyHostToDevice, ctx->stream);
    cgpu_status st = cg_cuda(ctx, e, "camera buffers");
    if (st == CGPU_OK) st = cg_camera(ctx, scene, dxy, n, dout);
    if (st == CGPU_OK) {
        e = cudaMemcpyAsync(out, dout, size_t(n) * 24, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        st = cg_cuda(ctx, e, "camera readback");
    }
    cudaFree(dxy);
    cudaFree(dout);
    return st;
}

cgpu_status cgpu_render(cgpu_ctx* ctx, const cgpu_render_params* params) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    return cg_render_batches(ctx, params);
}

cgpu_status cgpu_film_clear(cgpu_ctx* ctx, int32_t scene) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "film_clear: unknown scene id");
    return cg_film_clear(ctx, scene);
}

cgpu_status cgpu_film_read(cgpu_ctx* ctx, int32_t scene, double* sum_rgb, double* sum_sq_rgb, double* count) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "film_read: unknown scene id");
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    const size_t npix = size_t(sl.width) * sl.height;
    cudaError_t e = cudaSuccess;
    if (sum_rgb) e = cudaMemcpyAsync(sum_rgb, sl.film.sum, npix * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && sum_sq_rgb)
        e = cudaMemcpyAsync(sum_sq_rgb, sl.film.sumsq, npix * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && count) e = cudaMemcpyAsync(count, sl.film.count, npix * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    const cgpu_status st = cg_cuda(ctx, e, "film_read");
    return st != CGPU_OK ? st : cg_check_status(ctx);
}

cgpu_status cgpu_path_radiance(cgpu_ctx* ctx, int32_t scene, int32_t mode, const double* film_xy, const uint64_t* keys,
                               uint32_t n, float* out_rgb) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "path_radiance: unknown scene id");
    if (n == 0) return CGPU_OK;
    if (!film_xy || !keys || !out_rgb) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "path_radiance: null buffer");
    cudaSetDevice(ctx->device);
    const cgpu_status st = cg_path_radiance(ctx, scene, mode, film_xy, keys, n, out_rgb);
    return st != CGPU_OK ? st : cg_check_status(ctx);
}

cgpu_status cgpu_render_paths(cgpu_ctx* ctx, int32_t scene, int32_t mode, uint32_t first_sample, uint32_t num_samples,
                              uint64_t seed, float* out_rgb) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "render_paths: unknown scene id");
    if (!out_rgb) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_paths: null buffer");
    if (mode != CGPU_MODE_MEGAKERNEL && mode != CGPU_MODE_WAVEFRONT)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_paths: unknown mode");
    cudaSetDevice(ctx->device);
    const cgpu_status st = cg_render_paths_raw(ctx, scene, mode, first_sample, num_samples, seed, out_rgb);
    return st != CGPU_OK ? st : cg_check_status(ctx);
}

cgpu_status cgpu_render_stats_get(cgpu_ctx* ctx, cgpu_render_stats* out) {
    if (!check_ctx(ctx) || !out) return CGPU_ERR_INVALID_ARGUMENT;
    *out = ctx->stats;
    return CGPU_OK;
}

cgpu_status cgpu_set_profiling(cgpu_ctx* ctx, int32_t enabled) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    ctx->profiling = enabled != 0;
    return CGPU_OK;
}

cgpu_status cgpu_kernel_times_get(cgpu_ctx* ctx, cgpu_kernel_times* out) {
    if (!check_ctx(ctx) || !out) return CGPU_ERR_INVALID_ARGUMENT;
    *out = ctx->times;
    return CGPU_OK;
}

cgpu_status cgpu_set_counting(cgpu_ctx* ctx, int32_t enabled) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    ctx->counting = enabled != 0;
    return CGPU_OK;
}

}  // extern "C"
