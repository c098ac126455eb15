// Host-side scene construction (see scene_build.h).
#include "scene_build.h"

#include "bvh_build.h"
#include "tie_order.h"

#include <algorithm>
#include <chrono>
#include <future>
#include <cmath>
#include <cstring>

namespace cg {
namespace {

cgpu_status fail(std::string* err, cgpu_status s, const std::string& m) {
    if (err) *err = m;
    return s;
}

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

}  // namespace

// The filter constants are computed here in FP32 with the C library's exp,
// as the reference's filter constructors compute them
// (gaussianFilter.cpp:9-25, filter.cpp:19-21).
cgpu_status resolve_filter(const cgpu_film_filter& f, FilterD* out, std::string* err) {
    FilterD F{};
    F.type = f.type;
    float w = f.width, h = f.height;
    if (f.type == CGPU_FILTER_BOX) {
        if (w == 0.0f) w = 1.0f;
        if (h == 0.0f) h = 1.0f;
    } else if (f.type != CGPU_FILTER_GAUSSIAN && f.type != CGPU_FILTER_MITCHELL && f.type != CGPU_FILTER_CONE) {
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "unknown film filter");
    }
    if (!(w > 0.0f) || !(h > 0.0f) || !std::isfinite(w) || !std::isfinite(h) || w > 64.0f || h > 64.0f)
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "film filter size must be in (0, 64]");
    F.tile_w = f.tile_width == 0 ? 16 : f.tile_width;
    F.tile_h = f.tile_height == 0 ? 16 : f.tile_height;
    if (F.tile_w <= 0 || F.tile_h <= 0) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "film tile size must be positive");
    F.hx = w / 2.0f;
    F.hy = h / 2.0f;
    F.pixel_only = (f.type == CGPU_FILTER_BOX && w == 1.0f && h == 1.0f) ? 1 : 0;
    if (f.type == CGPU_FILTER_GAUSSIAN) {
        if (!(f.sigma_x > 0.0f) || !(f.sigma_y > 0.0f))
            return fail(err, CGPU_ERR_INVALID_ARGUMENT, "gaussian filter sigma must be positive");
        F.p0 = -1.0f / (2.0f * f.sigma_x * f.sigma_x);
        F.p1 = -1.0f / (2.0f * f.sigma_y * f.sigma_y);
        F.p3 = f.amplitude;
        F.p2 = f.amplitude * std::exp(F.p0 * F.hx * F.hx + F.p1 * F.hy * F.hy);
    } else if (f.type == CGPU_FILTER_MITCHELL) {
        F.p0 = f.b;
        F.p1 = f.c;
    }
    *out = F;
    return CGPU_OK;
}

cgpu_status build_host_scene(const cgpu_scene_desc* d, HostScene* out, std::string* err, BvhBuildFn bvh_builder,
                             void* bvh_user, bool tie_ranks) {
    if (!d) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "null scene description");
    {
        const cgpu_status fs = resolve_filter(d->filter, &out->filter, err);
        if (fs != CGPU_OK) return fs;
    }
    if (d->num_primitives == 0 || !d->prim_vertices || !d->prim_material)
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "no primitives");
    if (d->width <= 0 || d->height <= 0 || d->max_depth < 0)
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "bad film size or depth");
    if ((d->num_lights == 0 || !d->lights) && d->environment_texture == 0)
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "the estimator needs at least one light");
    if (d->num_materials == 0 || !d->materials || d->num_materials > 0xFFFFu)
        return fail(err, CGPU_ERR_INVALID_ARGUMENT, "bad material table");
    if (d->num_lights > 0xFFFEu) return fail(err, CGPU_ERR_UNSUPPORTED, "too many lights");
    if (size_t(d->width) * size_t(d->height) > (size_t(1) << 30))
        return fail(err, CGPU_ERR_UNSUPPORTED, "film too large");
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        const cgpu_texture& t = d->textures[i];
        if (t.width <= 0 || t.height <= 0 || !t.texels) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "bad texture");
    }
    const uint32_t np = d->num_primitives;
    // ---- validate and count triangles
    std::vector<int> light_of(np, -1);
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const int p = d->lights[i].primitive;
        if (p < 0 || uint32_t(p) >= np) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "light primitive out of range");
        light_of[size_t(p)] = int(i);
    }
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const int t = d->materials[i].type;
        if (t < 0 || t >= kNumBsdfTypes) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "unknown BSDF type");
        const int tex = d->materials[i].albedo_texture;
        if (tex >= int(d->num_textures)) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "texture index out of range");
    }
    uint32_t ntris = 0, nrects = 0;
    for (uint32_t i = 0; i < np; ++i) {
        const int k = d->prim_kind ? d->prim_kind[i] : CGPU_PRIM_TRIANGLE;
        if (k != CGPU_PRIM_TRIANGLE && k != CGPU_PRIM_RECTANGLE && k != CGPU_PRIM_SPHERE)
            return fail(err, CGPU_ERR_INVALID_ARGUMENT, "unknown primitive kind");
        if (k == CGPU_PRIM_SPHERE && light_of[i] >= 0)
            return fail(err, CGPU_ERR_UNSUPPORTED, "sphere light (the reference cannot sample sphere positions)");
        if (k == CGPU_PRIM_SPHERE && !(d->prim_vertices[9 * size_t(i) + 3] > 0.0f))
            return fail(err, CGPU_ERR_INVALID_ARGUMENT, "sphere radius must be positive");
        if (d->prim_material[i] < 0 || uint32_t(d->prim_material[i]) >= d->num_materials)
            return fail(err, CGPU_ERR_INVALID_ARGUMENT, "material index out of range");
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
                tflags[t] = kRecTriangle;
                ++t;
            } else if (k == CGPU_PRIM_SPHERE) {
                // the build sees the sphere's box as a degenerate "triangle" (lo, hi, lo),
                // widened by a few ulps of its coordinates
                const float r = v[3];
                for (int a = 0; a < 3; ++a) {
                    const float pad = 1e-5f * (std::fabs(v[a]) + r);
                    tv[9 * size_t(t) + a] = tv[9 * size_t(t) + 6 + a] = v[a] - r - pad;
                    tv[9 * size_t(t) + 3 + a] = v[a] + r + pad;
                }
                tprim[t] = i;
                tflags[t] = kRecSphere;
                ++t;
                out->has_spheres = true;
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
                    tflags[t] = kRecRectHalf | (r << 2);
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
        if (!std::isfinite(f)) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "non-finite vertex");
    }
    // the reference's tie order, built on other threads while the BVH builds
    std::future<std::vector<uint32_t>> ranks;
    if (tie_ranks) ranks = std::async(std::launch::async, [d] { return reference_visit_ranks(d); });
    Bvh4Result bvh;
    std::string berr;
    const auto tb = std::chrono::steady_clock::now();
    const bool built = bvh_builder ? bvh_builder(tv.data(), ntris, &bvh, &berr, bvh_user)
                                   : build_bvh4(tv.data(), ntris, &bvh, &berr);
    out->info.bvh_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
    if (!built) return fail(err, CGPU_ERR_INVALID_ARGUMENT, berr);
    if (3 * bvh.wide_depth + 1 > kStackSize)
        return fail(err, CGPU_ERR_UNSUPPORTED, "BVH too deep for the traversal stack");
    std::vector<TriRecord> recs(ntris);
    for (uint32_t s = 0; s < ntris; ++s) {
        const uint32_t t = bvh.order[s];
        const float* v = &tv[9 * size_t(t)];
        const uint32_t prim = tprim[t];
        const uint32_t mat = uint32_t(d->prim_material[prim]);
        const uint32_t packed = mat | (uint32_t(light_of[prim] + 1) << 16);
        TriRecord& R = recs[s];
        if (tflags[t] == kRecSphere) {
            const float* c = d->prim_vertices + 9 * size_t(prim);
            R.v0 = make_float4(c[0], c[1], c[2], 0.0f);
            R.v1 = make_float4(c[3], 0.0f, 0.0f, 0.0f);
            R.v2 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            R.v0 = make_float4(v[0], v[1], v[2], 0.0f);
            R.v1 = make_float4(v[3], v[4], v[5], 0.0f);
            R.v2 = make_float4(v[6], v[7], v[8], 0.0f);
        }
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
        M.exponent = m.exponent;
        M.ratio = m.diffuse_ratio;
        M.fresnel = m.fresnel;
        M.pad = 0;
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
        if (!(area > 0.0f)) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "light primitive has zero area");
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
            return fail(err, CGPU_ERR_INVALID_ARGUMENT, "environment texture index out of range");
        const cgpu_texture& et = d->textures[env_tex];
        const int W = et.width, H = et.height;
        if (W <= 0 || H <= 0) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "empty environment texture");
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
        if (!(total > 0.0)) return fail(err, CGPU_ERR_INVALID_ARGUMENT, "environment map is black");
        double run = 0.0;
        for (int y = 0; y < H; ++y) {
            run += rows[size_t(y)] / total;
            env_marg[size_t(y) + 1] = float(run);
        }
        env_marg[size_t(H)] = 1.0f;
    }
    // each area light's primitive records, in leaf order
    for (LightD& L : lights) L.slot[0] = L.slot[1] = -1;
    for (uint32_t s = 0; s < ntris; ++s) {
        const int li = light_of[tprim[bvh.order[s]]];
        if (li < 0) continue;
        int* sl = lights[size_t(li)].slot;
        if (sl[0] < 0) sl[0] = int(s);
        else if (sl[1] < 0) sl[1] = int(s);
    }
    out->nodes = std::move(bvh.nodes);
    out->tris = std::move(recs);
    out->mats = std::move(mats);
    out->num_area_lights = int(lights.size());
    out->lights = std::move(lights);
    if (env_tex >= 0) {
        LightD E;
        std::memset(&E, 0, sizeof(E));
        E.prim = -1;
        E.kind = 2;
        E.slot[0] = E.slot[1] = -1;
        E.tex = env_tex;
        E.ew = d->textures[env_tex].width;
        E.eh = d->textures[env_tex].height;
        out->lights.push_back(E);
        out->env_light = int(out->lights.size()) - 1;
    }
    out->env_tex = env_tex;
    out->env_marg = std::move(env_marg);
    out->env_cond = std::move(env_cond);
    out->textures.resize(d->num_textures);
    for (uint32_t i = 0; i < d->num_textures; ++i)
        out->textures[i] = TextureD{d->textures[i].width, d->textures[i].height, d->textures[i].texels};
    out->rect_frames = std::move(rect_frames);
    out->wide_depth = bvh.wide_depth;
    // camera (perspectivePinholeCamera.cpp:32-50, tMatrix4.ipp:47-60)
    {
        const HostV3 pos = v3(d->cam_position), dir = v3(d->cam_direction), up = v3(d->cam_up);
        const HostV3 z = normh(scale(dir, -1.0f));
        const HostV3 x = normh(crossh(up, z));
        const HostV3 y = crossh(z, x);
        CameraD& C = out->cam;
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
    out->info.num_primitives = np;
    out->info.num_triangles = ntris;
    out->info.num_bvh_nodes = uint32_t(out->nodes.size());
    out->info.num_lights = uint32_t(out->lights.size());
    {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t t = 0; t < ntris; ++t)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], tv[9 * size_t(t) + 3 * j + k]);
                    hi[k] = std::max(hi[k], tv[9 * size_t(t) + 3 * j + k]);
                }
        for (int k = 0; k < 3; ++k) { out->info.bounds_min[k] = lo[k]; out->info.bounds_max[k] = hi[k]; }
    }
    // ---- power light cluster (powerLightCluster.cpp:9-27): pick distribution
    // over the lights' approximate fluxes, Distribution1D's CDF
    // (distribution1D.cpp:10-41), in the reference's FP32 order
    if (d->light_cluster == CGPU_LIGHT_CLUSTER_POWER) {
        // RgbSpectrum::luminance (rgbSpectrum.cpp:33-37), weights as the reference has them
        auto luminance = [](float3 c) { return 0.0126f * c.x + 0.7152f * c.y + 0.0722f * c.z; };
        const size_t n = out->lights.size();
        std::vector<float> flux(n);
        for (size_t i = 0; i < n; ++i) {
            const LightD& L = out->lights[i];
            if (L.kind == 2) {
                // EnvironmentLight::approximateFlux (environmentLight.cpp:32-50, 125-139):
                // sum of texel luminance x sin(theta) x 4 pi x R^2, R half the scene diagonal
                const cgpu_texture& et = d->textures[L.tex];
                float background = 0.0f;
                for (int y = 0; y < et.height; ++y) {
                    const float v = (float(y) + 0.5f) / float(et.height);
                    const float st = std::sin((1.0f - v) * 3.1415926535897932f);
                    for (int x = 0; x < et.width; ++x) {
                        const float* t = et.texels + 3 * (size_t(y) * et.width + x);
                        background += luminance(make_float3(t[0], t[1], t[2])) * st;
                    }
                }
                float e2 = 0.0f;
                for (int k = 0; k < 3; ++k) {
                    const float e = out->info.bounds_max[k] - out->info.bounds_min[k];
                    e2 += e * e;
                }
                const float R = std::sqrt(e2) * 0.5f;
                flux[i] = background * 12.566370614359172f * R * R;
            } else {
                // SingleAreaLight::approximateFlux (singleAreaLight.cpp:170-187)
                const float f = luminance(L.radiance) * L.area * 3.1415926535897932f;
                flux[i] = f > 0.0f ? f : 1.0f;  // AreaLight::_defaultFlux
            }
        }
        std::vector<float> cdf(n + 1);
        const float delta = 1.0f / float(n);
        cdf[0] = 0.0f;
        for (size_t i = 1; i <= n; ++i) cdf[i] = cdf[i - 1] + flux[i - 1] * delta;
        const float sum = cdf[n];
        if (sum > 0.0f) {
            const float inv = 1.0f / sum;
            for (size_t i = 1; i <= n; ++i) cdf[i] *= inv;
        } else {
            for (size_t i = 1; i <= n; ++i) cdf[i] = float(i) * delta;
        }
        cdf[n] = 1.0f;
        out->light_cdf = std::move(cdf);
    }
    if (tie_ranks) out->prim_rank = ranks.get();
    return CGPU_OK;
}

SceneD host_view(HostScene& hs, const cgpu_scene_desc* d) {
    SceneD S{};
    if (hs.env_light >= 0) {
        hs.lights[size_t(hs.env_light)].marg_cdf = hs.env_marg.data();
        hs.lights[size_t(hs.env_light)].cond_cdf = hs.env_cond.data();
    }
    S.nodes = hs.nodes.data();
    S.tris = hs.tris.data();
    S.materials = hs.mats.data();
    S.lights = hs.lights.data();
    S.textures = hs.textures.data();
    S.prim_normals = d->prim_normals;
    S.prim_uvws = d->prim_uvws;
    S.rect_frames = hs.rect_frames.data();
    S.prim_rank = hs.prim_rank.empty() ? nullptr : hs.prim_rank.data();
    S.light_cdf = hs.light_cdf.empty() ? nullptr : hs.light_cdf.data();
    S.num_lights = int(hs.lights.size());
    S.env_light = hs.env_light;
    S.num_tris = int(hs.tris.size());
    S.width = d->width;
    S.height = d->height;
    S.max_depth = d->max_depth;
    S.spp = d->spp > 0 ? d->spp : 1;
    S.cam = hs.cam;
    S.filter = hs.filter;
    S.bounds_lo = make_float3(hs.info.bounds_min[0], hs.info.bounds_min[1], hs.info.bounds_min[2]);
    {
        float inv[3];
        for (int k = 0; k < 3; ++k) {
            const float e = hs.info.bounds_max[k] - hs.info.bounds_min[k];
            inv[k] = e > 0.0f ? 1.0f / e : 0.0f;
        }
        S.bounds_inv = make_float3(inv[0], inv[1], inv[2]);
    }
    S.visit_budget = auto_visit_budget(hs.nodes.size());
    S.status = nullptr;
    {
        const float c[3] = {hs.cam.pos.x, hs.cam.pos.y, hs.cam.pos.z};
        S.tie_abs = tie_window_abs(hs.info.bounds_min, hs.info.bounds_max, c);
    }
    return S;
}

}  // namespace cg
