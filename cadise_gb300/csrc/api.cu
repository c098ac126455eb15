// C ABI entry points (include/cadise_gpu.h): context, scene upload, ray
// queries, camera rays, render, film.
#include "bvh_build.h"
#include "internal.h"

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

struct HostV3 {
    float x, y, z;
};
HostV3 v3(const float* p) { return {p[0], p[1], p[2]}; }
float3 f3h(HostV3 a) { return make_float3(a.x, a.y, a.z); }
HostV3 sub(HostV3 a, HostV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
HostV3 add(HostV3 a, HostV3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
HostV3 scale(HostV3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
HostV3 crossh(HostV3 a, HostV3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float len2h(HostV3 a) {
    float r = 0.0f;
    r += a.x * a.x;
    r += a.y * a.y;
    r += a.z * a.z;
    return r;
}
float lenh(HostV3 a) { return std::sqrt(len2h(a)); }
HostV3 normh(HostV3 a) { return scale(a, 1.0f / lenh(a)); }
bool zeroh(HostV3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }

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
    if (e != cudaSuccess) {
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
    return cg_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

cgpu_status cgpu_scene_upload(cgpu_ctx* ctx, const cgpu_scene_desc* d, int32_t* out_scene) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!d || !out_scene) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: null argument");
    if (d->num_primitives == 0 || !d->prim_vertices || !d->prim_material)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: no primitives");
    if (d->width <= 0 || d->height <= 0 || d->max_depth < 0)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: bad film size or depth");
    if ((d->num_lights == 0 || !d->lights) && d->environment_texture == 0)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: the estimator needs at least one light");
    if (d->num_materials == 0 || !d->materials || d->num_materials > 0xFFFFu)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: bad material table");
    if (d->num_lights > 0xFFFEu) return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "scene_upload: too many lights");
    if (size_t(d->width) * size_t(d->height) > (size_t(1) << 30))
        return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "scene_upload: film too large");
    cudaSetDevice(ctx->device);
    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t np = d->num_primitives;
    // ---- validate and count triangles
    std::vector<int> light_of(np, -1);
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const int p = d->lights[i].primitive;
        if (p < 0 || uint32_t(p) >= np) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: light primitive out of range");
        light_of[size_t(p)] = int(i);
    }
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const int t = d->materials[i].type;
        if (t < 0 || t >= kNumBsdfKinds) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: unknown BSDF type");
        const int tex = d->materials[i].albedo_texture;
        if (tex >= int(d->num_textures)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: texture index out of range");
    }
    uint32_t ntris = 0, nrects = 0;
    for (uint32_t i = 0; i < np; ++i) {
        const int k = d->prim_kind ? d->prim_kind[i] : CGPU_PRIM_TRIANGLE;
        if (k != CGPU_PRIM_TRIANGLE && k != CGPU_PRIM_RECTANGLE)
            return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: unknown primitive kind");
        if (d->prim_material[i] < 0 || uint32_t(d->prim_material[i]) >= d->num_materials)
            return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: material index out of range");
        ntris += k == CGPU_PRIM_RECTANGLE ? 2 : 1;
        nrects += k == CGPU_PRIM_RECTANGLE ? 1 : 0;
    }
    // ---- expand rectangles, keep per-triangle vertices for the build
    std::vector<float> tv(size_t(ntris) * 9);
    std::vector<uint32_t> tprim(ntris), tflags(ntris);
    std::vector<float> rect_frames(size_t(nrects) * 9);
    {
        uint32_t t = 0, r = 0;
        for (uint32_t i = 0; i < np; ++i) {
            const float* v = d->prim_vertices + 9 * size_t(i);
            const int k = d->prim_kind ? d->prim_kind[i] : CGPU_PRIM_TRIANGLE;
            if (k == CGPU_PRIM_TRIANGLE) {
                std::memcpy(&tv[9 * size_t(t)], v, 9 * sizeof(float));
                tprim[t] = i;
                tflags[t] = 0;
                ++t;
            } else {
                // rectangle v1 v2 v3 = vA vB vC; eA = vA - vB, eB = vC - vB, vD = vB + eA + eB
                const HostV3 vA = v3(v), vB = v3(v + 3), vC = v3(v + 6);
                const HostV3 eA = sub(vA, vB), eB = sub(vC, vB);
                const HostV3 vD = add(add(vB, eA), eB);
                const HostV3 h1[3] = {vB, vA, vC}, h2[3] = {vA, vD, vC};
                for (int h = 0; h < 2; ++h) {
                    const HostV3* hv = h == 0 ? h1 : h2;
                    for (int j = 0; j < 3; ++j) {
                        tv[9 * size_t(t) + 3 * j + 0] = hv[j].x;
                        tv[9 * size_t(t) + 3 * j + 1] = hv[j].y;
                        tv[9 * size_t(t) + 3 * j + 2] = hv[j].z;
                    }
                    tprim[t] = i;
                    tflags[t] = 1u | (r << 1);
                    ++t;
                }
                float* fr = &rect_frames[9 * size_t(r)];
                fr[0] = vB.x; fr[1] = vB.y; fr[2] = vB.z;
                fr[3] = eA.x; fr[4] = eA.y; fr[5] = eA.z;
                fr[6] = eB.x; fr[7] = eB.y; fr[8] = eB.z;
                ++r;
            }
        }
    }
    for (float f : tv) {
        if (!std::isfinite(f)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: non-finite vertex");
    }
    Bvh4Result bvh;
    std::string err;
    if (!build_bvh4(tv.data(), ntris, &bvh, &err)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: " + err);
    if (3 * bvh.wide_depth + 1 > kStackSize)
        return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "scene_upload: BVH too deep for the traversal stack");
    std::vector<TriRecord> recs(ntris);
    for (uint32_t s = 0; s < ntris; ++s) {
        const uint32_t t = bvh.order[s];
        const float* v = &tv[9 * size_t(t)];
        const uint32_t prim = tprim[t];
        const uint32_t mat = uint32_t(d->prim_material[prim]);
        const uint32_t packed = mat | (uint32_t(light_of[prim] + 1) << 16);
        TriRecord& R = recs[s];
        R.v0 = make_float4(v[0], v[1], v[2], 0.0f);
        R.v1 = make_float4(v[3], v[4], v[5], 0.0f);
        R.v2 = make_float4(v[6], v[7], v[8], 0.0f);
        std::memcpy(&R.v0.w, &prim, 4);
        std::memcpy(&R.v1.w, &packed, 4);
        std::memcpy(&R.v2.w, &tflags[t], 4);
    }
    // rect flags carry the rectangle index; the device reads frames by it
    // ---- materials
    std::vector<MaterialD> mats(d->num_materials);
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const cgpu_material& m = d->materials[i];
        MaterialD& M = mats[i];
        M.type = m.type;
        M.albedo_tex = m.albedo_texture;
        M.roughness = m.roughness;
        const float safe = std::max(m.roughness, 0.001f);  // tRoughnessMapper.h:18-40 (SQUARE)
        M.alpha = std::max(safe * safe, 0.001f);
        M.albedo = make_float3(m.albedo[0], m.albedo[1], m.albedo[2]);
        M.f0 = make_float3(m.f0[0], m.f0[1], m.f0[2]);
        M.ior_outer = m.ior_outer;
        M.ior_inner = m.ior_inner;
    }
    // ---- lights (singleAreaLight.cpp:20-37)
    std::vector<LightD> lights(d->num_lights);
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const cgpu_area_light& l = d->lights[i];
        LightD& L = lights[i];
        std::memset(&L, 0, sizeof(L));
        const uint32_t p = uint32_t(l.primitive);
        const float* v = d->prim_vertices + 9 * size_t(p);
        const int k = d->prim_kind ? d->prim_kind[p] : CGPU_PRIM_TRIANGLE;
        L.prim = int(p);
        L.kind = k == CGPU_PRIM_RECTANGLE ? 1 : 0;
        L.back_face = l.back_face_emit ? 1 : 0;
        float area;
        if (L.kind == 0) {
            const HostV3 A = v3(v), eAB = sub(v3(v + 3), A), eAC = sub(v3(v + 6), A);
            const HostV3 c = crossh(eAB, eAC);
            area = 0.5f * lenh(c);
            const HostV3 N = zeroh(c) ? HostV3{0.0f, 1.0f, 0.0f} : normh(c);
            L.p0 = f3h(A);
            L.e0 = f3h(eAB);
            L.e1 = f3h(eAC);
            L.n = f3h(N);
            L.nA = L.nB = L.nC = L.n;
            if (d->prim_normals) {
                const float* nn = d->prim_normals + 9 * size_t(p);
                const HostV3 na = v3(nn), nb = v3(nn + 3), nc = v3(nn + 6);
                if (!zeroh(na)) L.nA = f3h(na);
                if (!zeroh(nb)) L.nB = f3h(nb);
                if (!zeroh(nc)) L.nC = f3h(nc);
                L.has_normals = 1;
            }
        } else {
            const HostV3 vA = v3(v), vB = v3(v + 3), vC = v3(v + 6);
            const HostV3 eA = sub(vA, vB), eB = sub(vC, vB);
            area = lenh(eA) * lenh(eB);
            const HostV3 c = crossh(eA, eB);
            const HostV3 N = zeroh(c) ? HostV3{0.0f, 1.0f, 0.0f} : normh(c);
            L.p0 = f3h(vB);
            L.e0 = f3h(eA);
            L.e1 = f3h(eB);
            L.n = f3h(N);
            HostV3 le = eA, se = eB;
            if (lenh(eA) < lenh(eB)) std::swap(le, se);
            L.long_e = f3h(le);
            L.long_len = lenh(le);
            L.short_len = lenh(se);
            L.short_dir = f3h(normh(se));
        }
        if (!(area > 0.0f)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: light primitive has zero area");
        L.area = area;
        L.pdf_area = 1.0f / area;
        const HostV3 color = v3(l.color);
        const float csum = color.x + color.y + color.z;
        const HostV3 unit = scale(color, 1.0f / csum);
        const HostV3 total = scale(unit, l.watt);
        L.radiance = f3h(scale(scale(total, 1.0f / area), 0.3183098861837906f));
    }
    // ---- environment light (environmentLight.cpp:16-57): sampling weights
    // luminance x sin(theta) per texel, Rec. 709 luminance
    const int env_tex = d->environment_texture - 1;
    std::vector<float> env_marg, env_cond;
    if (d->environment_texture != 0) {
        if (env_tex < 0 || env_tex >= int(d->num_textures) || !d->textures[env_tex].texels)
            return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: environment texture index out of range");
        const cgpu_texture& et = d->textures[env_tex];
        const int W = et.width, H = et.height;
        if (W <= 0 || H <= 0) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: empty environment texture");
        env_marg.assign(size_t(H) + 1, 0.0f);
        env_cond.assign(size_t(H) * (W + 1), 0.0f);
        std::vector<double> rows(static_cast<size_t>(H), 0.0);
        double total = 0.0;
        for (int y = 0; y < H; ++y) {
            const double st = std::sin((1.0 - (y + 0.5) / H) * 3.14159265358979323846);
            double acc = 0.0;
            std::vector<double> wrow(static_cast<size_t>(W));
            for (int x = 0; x < W; ++x) {
                const float* t = et.texels + 3 * (size_t(y) * W + x);
                const double lum = 0.2126 * t[0] + 0.7152 * t[1] + 0.0722 * t[2];
                wrow[size_t(x)] = std::max(lum, 0.0) * st;
                acc += wrow[size_t(x)];
            }
            float* c = &env_cond[size_t(y) * (W + 1)];
            double run = 0.0;
            for (int x = 0; x < W; ++x) {
                run += acc > 0.0 ? wrow[size_t(x)] / acc : 1.0 / W;
                c[x + 1] = float(run);
            }
            c[W] = 1.0f;
            rows[size_t(y)] = acc;
            total += acc;
        }
        if (!(total > 0.0)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: environment map is black");
        double run = 0.0;
        for (int y = 0; y < H; ++y) {
            run += rows[size_t(y)] / total;
            env_marg[size_t(y) + 1] = float(run);
        }
        env_marg[size_t(H)] = 1.0f;
    }
    // ---- textures
    SceneSlot sl;
    std::vector<TextureD> texs(d->num_textures);
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        const cgpu_texture& t = d->textures[i];
        if (t.width <= 0 || t.height <= 0 || !t.texels) {
            free_slot(sl);
            return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "scene_upload: bad texture");
        }
        float* dev = nullptr;
        cgpu_status st = upload(ctx, sl, t.texels, size_t(t.width) * t.height * 3, &dev);
        if (st != CGPU_OK) { free_slot(sl); return st; }
        texs[i] = TextureD{t.width, t.height, dev};
    }
    cgpu_status st = CGPU_OK;
    Bvh4Node* dn = nullptr;
    TriRecord* dt = nullptr;
    MaterialD* dm = nullptr;
    LightD* dl = nullptr;
    TextureD* dtex = nullptr;
    float *dnorm = nullptr, *duvw = nullptr, *drect = nullptr;
    if (st == CGPU_OK) st = upload(ctx, sl, bvh.nodes.data(), bvh.nodes.size(), &dn);
    if (st == CGPU_OK) st = upload(ctx, sl, recs.data(), recs.size(), &dt);
    if (st == CGPU_OK) st = upload(ctx, sl, mats.data(), mats.size(), &dm);
    if (st == CGPU_OK) st = upload(ctx, sl, lights.data(), lights.size(), &dl);
    if (st == CGPU_OK) st = upload(ctx, sl, texs.data(), texs.size(), &dtex);
    if (st == CGPU_OK && d->prim_normals) st = upload(ctx, sl, d->prim_normals, size_t(np) * 9, &dnorm);
    if (st == CGPU_OK && d->prim_uvws) st = upload(ctx, sl, d->prim_uvws, size_t(np) * 9, &duvw);
    if (st == CGPU_OK) st = upload(ctx, sl, rect_frames.data(), rect_frames.size(), &drect);
    sl.num_area_lights = int(lights.size());
    if (st == CGPU_OK && env_tex >= 0) {
        float *dm_cdf = nullptr, *dc_cdf = nullptr;
        st = upload(ctx, sl, env_marg.data(), env_marg.size(), &dm_cdf);
        if (st == CGPU_OK) st = upload(ctx, sl, env_cond.data(), env_cond.size(), &dc_cdf);
        if (st == CGPU_OK) {
            LightD E;
            std::memset(&E, 0, sizeof(E));
            E.prim = -1;
            E.kind = 2;
            E.tex = env_tex;
            E.ew = d->textures[env_tex].width;
            E.eh = d->textures[env_tex].height;
            E.marg_cdf = dm_cdf;
            E.cond_cdf = dc_cdf;
            lights.push_back(E);
            // re-upload the light table with the environment appended
            st = upload(ctx, sl, lights.data(), lights.size(), &dl);
        }
    }
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
    sl.h_mats = mats;
    sl.h_lights = lights;
    sl.h_texs = texs;
    sl.d_mats = dm;
    sl.d_lights = dl;
    SceneD& S = sl.d;
    S.nodes = dn;
    S.tris = dt;
    S.materials = dm;
    S.lights = dl;
    S.textures = dtex;
    S.prim_normals = dnorm;
    S.prim_uvws = duvw;
    S.rect_frames = drect;
    S.num_lights = int(lights.size());
    S.env_light = env_tex >= 0 ? int(lights.size()) - 1 : -1;
    S.num_tris = int(ntris);
    S.width = d->width;
    S.height = d->height;
    S.max_depth = d->max_depth;
    S.spp = d->spp > 0 ? d->spp : 1;
    // camera (perspectivePinholeCamera.cpp:32-50, tMatrix4.ipp:47-60)
    {
        const HostV3 pos = v3(d->cam_position), dir = v3(d->cam_direction), up = v3(d->cam_up);
        const HostV3 z = normh(scale(dir, -1.0f));
        const HostV3 x = normh(crossh(up, z));
        const HostV3 y = crossh(z, x);
        CameraD& C = S.cam;
        C.pos = f3h(pos);
        C.ax = f3h(x);
        C.ay = f3h(y);
        C.az = f3h(z);
        const double sw = d->sensor_width_mm > 0.0f ? double(d->sensor_width_mm) : 36.0;
        const double aspect = double(d->width) / double(d->height);
        const double sh = sw / aspect;
        const float half_fov = float(double(d->fov_degrees) * 0.5) * 0.0174532925199432f;
        C.offset = float((sw * 0.5) / std::tan(half_fov));
        C.sx = float(sw / d->width);
        C.sy = float(-sh / d->height);
        C.tx = float(-(sw * 0.5));
        C.ty = float(sh * 0.5);
    }
    sl.width = d->width;
    sl.height = d->height;
    sl.spp = S.spp;
    sl.max_depth = d->max_depth;
    sl.live = true;
    cgpu_scene_info& I = sl.info;
    I.num_primitives = np;
    I.num_triangles = ntris;
    I.num_bvh_nodes = uint32_t(bvh.nodes.size());
    I.num_lights = uint32_t(lights.size());
    I.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t t = 0; t < ntris; ++t)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], tv[9 * size_t(t) + 3 * j + k]);
                    hi[k] = std::max(hi[k], tv[9 * size_t(t) + 3 * j + k]);
                }
        for (int k = 0; k < 3; ++k) { I.bounds_min[k] = lo[k]; I.bounds_max[k] = hi[k]; }
    }
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
    return st;
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
    return cg_cuda(ctx, e, "film_read");
}

cgpu_status cgpu_path_radiance(cgpu_ctx* ctx, int32_t scene, int32_t mode, const double* film_xy, const uint64_t* keys,
                               uint32_t n, float* out_rgb) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "path_radiance: unknown scene id");
    if (n == 0) return CGPU_OK;
    if (!film_xy || !keys || !out_rgb) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "path_radiance: null buffer");
    cudaSetDevice(ctx->device);
    return cg_path_radiance(ctx, scene, mode, film_xy, keys, n, out_rgb);
}

cgpu_status cgpu_render_paths(cgpu_ctx* ctx, int32_t scene, int32_t mode, uint32_t first_sample, uint32_t num_samples,
                              uint64_t seed, float* out_rgb) {
    if (!check_ctx(ctx)) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid_scene(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "render_paths: unknown scene id");
    if (!out_rgb) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_paths: null buffer");
    if (mode != CGPU_MODE_MEGAKERNEL && mode != CGPU_MODE_WAVEFRONT)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "render_paths: unknown mode");
    cudaSetDevice(ctx->device);
    return cg_render_paths_raw(ctx, scene, mode, first_sample, num_samples, seed, out_rgb);
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
