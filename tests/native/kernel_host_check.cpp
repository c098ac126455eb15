// CPU execution of the CUDA library's device code for testing (test
// infrastructure, never part of the library): the traversal
// (traverse.cuh), the per-path estimator (pathtrace.cuh / shading.cuh) and
// the per-path adjoint (adjoint.cuh) and
// the scene construction (scene_build.cpp, bvh_build.cpp) compiled as plain
// host C++, so their logic is checked against the golden vectors before any
// GPU time is spent.
#include "../../cadise_gb300/csrc/adjoint.cuh"
#include "../../cadise_gb300/csrc/film.cuh"
#include "../../cadise_gb300/csrc/scene_build.h"

#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace {
struct Check {
    cg::HostScene hs;
    cg::SceneD S;
};

struct HostSink {
    double* g_rough;
    double* g_rad;
    double* g_tex;
    const std::vector<int>& tex_offset;
    void rough(int m, double v) { g_rough[m] += v; }
    void rad(int i, double v) { g_rad[i] += v; }
    void tex(int t, int k, double v) { g_tex[tex_offset[size_t(t)] + k] += v; }
};
}  // namespace

extern "C" {

void* khc_create(const cgpu_scene_desc* d, char* err, int errlen) {
    auto c = std::make_unique<Check>();
    std::string e;
    if (cg::build_host_scene(d, &c->hs, &e) != CGPU_OK) {
        std::snprintf(err, size_t(errlen), "%s", e.c_str());
        return nullptr;
    }
    c->S = cg::host_view(c->hs, d);
    return c.release();
}

void khc_destroy(void* p) { delete static_cast<Check*>(p); }

// The kernels' texel lookup (texture_rgb: nearest, repeat wrap) of texture
// `tex` at n uvws (3 floats each); 3 floats out per uvw.
void khc_texel(void* p, int tex, const float* uvw, uint32_t n, float* rgb) {
    const Check& c = *static_cast<Check*>(p);
    for (uint32_t i = 0; i < n; ++i) {
        const float3 v = cg::texture_rgb(c.S.textures[tex], cg::mk(uvw[3 * i], uvw[3 * i + 1], uvw[3 * i + 2]));
        rgb[3 * i + 0] = v.x;
        rgb[3 * i + 1] = v.y;
        rgb[3 * i + 2] = v.z;
    }
}

// Device-side iteration budget of the traversals (0: the automatic one) and
// the word that counts the rays that ran out of it.
// the scene's exact-tie ranks (reference_visit_ranks), 8 per primitive
void khc_ranks(void* p, uint32_t* out) {
    const Check& c = *static_cast<Check*>(p);
    for (size_t i = 0; i < c.hs.prim_rank.size(); ++i) out[i] = c.hs.prim_rank[i];
}

void khc_set_budget(void* p, uint32_t visits, uint32_t* status) {
    Check& c = *static_cast<Check*>(p);
    c.S.visit_budget = visits ? visits : cg::auto_visit_budget(c.hs.nodes.size());
    c.S.status = status;
}

// rays: 8 floats (org, t_min, dir, t_max); dyn 1 uses the resumable stepper, 2 the warp traversal
void khc_trace(void* p, const float* rays, uint32_t n, int dyn, int32_t* prim, float* t, float* u, float* v,
               int32_t* occ) {
    const Check& c = *static_cast<Check*>(p);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 8 * size_t(i);
        const cg::RayPre pr = cg::ray_prep(cg::mk(r[0], r[1], r[2]), cg::normalize(cg::mk(r[4], r[5], r[6])), r[3], r[7]);
        cg::TraceCounters tc{0, 0};
        cg::HitD h;
        bool hit, any;
        if (dyn == 1) {
            std::unique_ptr<cg::TravState> st(new cg::TravState());
            cg::trav_begin(*st, pr, c.S.visit_budget);
            while (!st->done) cg::trav_step<false, false>(c.S, pr, *st, &tc);
            hit = st->hslot >= 0;
            h.slot = st->hslot;
            h.t = st->tcur;
            h.u = st->hu;
            h.v = st->hv;
            cg::trav_begin(*st, pr, c.S.visit_budget);
            while (!st->done) cg::trav_step<true, false>(c.S, pr, *st, &tc);
            any = st->hslot >= 0;
        } else if (dyn == 2) {
            hit = cg::traverse_warp<false>(c.S, pr, &h, &tc);
            cg::HitD h2;
            any = cg::traverse<true, false>(c.S, pr, &h2, &tc);
        } else {
            hit = cg::traverse<false, false>(c.S, pr, &h, &tc);
            cg::HitD h2;
            any = cg::traverse<true, false>(c.S, pr, &h2, &tc);
        }
        prim[i] = hit ? __float_as_int(c.S.tris[h.slot].v0.w) : -1;
        cg::HitPoint hp{};
        if (hit) hp = cg::hit_point(c.S, pr.o, pr.d, h);
        t[i] = hit ? hp.t : 0.0f;
        u[i] = hit ? (hp.rect >= 0 ? hp.p1 : hp.b1) : 0.0f;
        v[i] = hit ? (hp.rect >= 0 ? hp.p2 : hp.b2) : 0.0f;
        occ[i] = any ? 1 : 0;
    }
}

void khc_paths(void* p, const double* xy, const uint64_t* keys, uint32_t n, float* rgb) {
    const Check& c = *static_cast<Check*>(p);
    for (uint32_t i = 0; i < n; ++i) {
        cg::Rng rng;
        rng.key = keys[i];
        rng.ctr = 0;
        float3 o, d;
        cg::camera_ray(c.S.cam, float(xy[2 * i]), float(xy[2 * i + 1]), &o, &d);
        float3 L, Le, Ls;
        cg::TraceCounters tc{0, 0}, ta{0, 0};
        uint32_t nc = 0, na = 0;
        cg::mk_path<false>(c.S, o, d, rng, &L, &Le, &Ls, &tc, &ta, &nc, &na);
        const float3 v = cg::path_sample(L, Le, Ls);
        rgb[3 * i + 0] = v.x;
        rgb[3 * i + 1] = v.y;
        rgb[3 * i + 2] = v.z;
    }
}

// samples [first, first + count) of every pixel, sample-major, as cgpu_render_paths
void khc_render_paths(void* p, uint64_t seed, uint32_t scene_index, uint32_t first, uint32_t count, float* out) {
    const Check& c = *static_cast<Check*>(p);
    const uint32_t npix = uint32_t(c.S.width) * uint32_t(c.S.height);
    for (uint32_t k = 0; k < count; ++k)
        for (uint32_t px = 0; px < npix; ++px) {
            cg::PathId id;
            id.scene = int(scene_index);
            id.pixel = px;
            id.sample = first + k;
            id.width = uint32_t(c.S.width);
            cg::Rng rng;
            float3 o, d;
            cg::primary_ray(c.S, id, seed, rng, &o, &d);
            float3 L, Le, Ls;
            cg::TraceCounters tc{0, 0}, ta{0, 0};
            uint32_t nc = 0, na = 0;
            cg::mk_path<false>(c.S, o, d, rng, &L, &Le, &Ls, &tc, &ta, &nc, &na);
            const float3 v = cg::path_sample(L, Le, Ls);
            float* q = out + 3 * (size_t(k) * npix + px);
            q[0] = v.x;
            q[1] = v.y;
            q[2] = v.z;
        }
}

// Gradients of sum(dLdI * image) over samples [0, spp) of every pixel, as
// cgpu_adjoint_backward: texel floats (all textures back to back),
// roughness per material, radiance per area light and channel.
void khc_adjoint(void* p, uint64_t seed, uint32_t scene_index, uint32_t spp, const float* dLdI, double* g_tex,
                 double* g_rough, double* g_rad) {
    const Check& c = *static_cast<Check*>(p);
    std::vector<int> off;
    int acc = 0;
    for (const cg::TextureD& t : c.hs.textures) {
        off.push_back(acc);
        acc += t.width * t.height * 3;
    }
    HostSink sink{g_rough, g_rad, g_tex, off};
    const uint32_t npix = uint32_t(c.S.width) * uint32_t(c.S.height);
    const float inv_spp = 1.0f / float(spp);
    for (uint32_t k = 0; k < spp; ++k)
        for (uint32_t px = 0; px < npix; ++px) {
            const float3 delta = cg::mk(dLdI[3 * px] * inv_spp, dLdI[3 * px + 1] * inv_spp, dLdI[3 * px + 2] * inv_spp);
            if (cg::is_zero(delta)) continue;
            cg::PathId id;
            id.scene = int(scene_index);
            id.pixel = px;
            id.sample = k;
            id.width = uint32_t(c.S.width);
            cg::adjoint_path(c.S, id, seed, delta, c.hs.num_area_lights, sink);
        }
}

// The path-state layout of the wavefront (wf_layout) for `cap` paths and
// `rows` counter rows: 0 when every array lies inside the measured size,
// 256-byte aligned and disjoint from the others, else the failing array + 1.
// The splat kernel's filtered gather (film.cuh filter_gather) for every pixel
// of a W x H film over `count` samples per pixel (sample-major arrays:
// positions count x H x W x 2, radiance count x H x W x 3); film H x W x 7
// {sum w rgb, sum w rgb^2, sum w}.  Returns 0, or -1 if the filter is invalid.
int khc_filter_gather(const cgpu_film_filter* f, int W, int H, uint32_t count, const float* xy, const float* rgb,
                      double* film) {
    cg::FilterD F;
    std::string err;
    if (cg::resolve_filter(*f, &F, &err) != CGPU_OK) return -1;
    const size_t npix = size_t(W) * H;
    auto fetch = [&](uint32_t k, int sx, int sy, float3* v, float2* pos) {
        const size_t i = size_t(k) * npix + size_t(sy) * W + sx;
        *v = make_float3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
        *pos = make_float2(xy[2 * i], xy[2 * i + 1]);
        return std::isfinite(v->x) && std::isfinite(v->y) && std::isfinite(v->z);
    };
    for (int iy = 0; iy < H; ++iy)
        for (int ix = 0; ix < W; ++ix) {
            double* o = film + 7 * (size_t(iy) * W + ix);
            cg::filter_gather(F, W, H, ix, iy, count, fetch, o, o + 3, o + 6);
        }
    return 0;
}

// quantize_node on nk child boxes (lo / hi: nk x 3 floats each); out: the 64-byte node.
void khc_quantize(const float* lo, const float* hi, int nk, void* out) {
    float l[4][3] = {}, h[4][3] = {};
    uint32_t child[4] = {1, 2, 3, 4};
    for (int i = 0; i < nk; ++i)
        for (int a = 0; a < 3; ++a) {
            l[i][a] = lo[3 * i + a];
            h[i][a] = hi[3 * i + a];
        }
    cg::quantize_node(l, h, child, nk, static_cast<cg::Bvh4Node*>(out));
}

int khc_wf_layout_check(uint64_t cap, int rows) {
    cg::WfBuffers w{};
    const size_t total = cg::wf_layout(nullptr, size_t(cap), rows, &w);
    char* base = reinterpret_cast<char*>(size_t(1) << 40);  // carve from a fake, aligned base; nothing is touched
    cg::wf_layout(base, size_t(cap), rows, &w);
    struct Span { const void* p; size_t bytes; };
    std::vector<Span> v;
    const float4* f4s[] = {w.ray_o, w.ray_d, w.hit, w.thr, w.L, w.Le, w.Ls, w.mis_a, w.mis_b, w.mis_d, w.sh_d, w.sh_c};
    for (const float4* f : f4s) v.push_back({f, size_t(cap) * 16});
    v.push_back({w.meta, size_t(cap) * 16});
    for (int k = 0; k < 2; ++k) {
        v.push_back({w.q_cont[k], size_t(cap) * 4});
        v.push_back({w.q_mis[k], size_t(cap) * 4});
        v.push_back({w.q_shadow[k], size_t(cap) * 4});
    }
    for (int k = 0; k < cg::kNumBsdfKinds; ++k) v.push_back({w.q_mat[k], size_t(cap) * 4});
    v.push_back({w.cnt, size_t(rows) * cg::kCntStride * 4});
    for (size_t i = 0; i < v.size(); ++i) {
        const size_t a = size_t(static_cast<const char*>(v[i].p) - base);
        if (a % 256 != 0 || a + v[i].bytes > total) return int(i) + 1;
        for (size_t j = 0; j < i; ++j) {
            const size_t b = size_t(static_cast<const char*>(v[j].p) - base);
            if (a < b + v[j].bytes && b < a + v[i].bytes) return int(i) + 1;
        }
    }
    return w.cnt_depth == rows ? 0 : -1;
}

// Bytes the static scratch of cgpu_render_noalloc needs, and its size.
uint64_t khc_noalloc_layout_bytes() {
    cg::NoAllocView v;
    return cg::noalloc_layout(nullptr, &v);
}
uint64_t khc_noalloc_scratch_bytes() { return cg::kNoAllocScratchBytes; }

}  // extern "C"
