// CPU execution of the CUDA library's device code for testing (test
// infrastructure, never part of the library): the traversal
// (traverse.cuh), the per-path estimator (pathtrace.cuh / shading.cuh) and
// the scene construction (scene_build.cpp, bvh_build.cpp) compiled as plain
// host C++, so their logic is checked against the golden vectors before any
// GPU time is spent.
#include "../../cadise_gb300/csrc/pathtrace.cuh"
#include "../../cadise_gb300/csrc/scene_build.h"

#include <cstdio>
#include <memory>
#include <string>

namespace {
struct Check {
    cg::HostScene hs;
    cg::SceneD S;
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

// rays: 8 floats (org, t_min, dir, t_max); dyn != 0 uses the resumable stepper
void khc_trace(void* p, const float* rays, uint32_t n, int dyn, int32_t* prim, float* t, float* u, float* v,
               int32_t* occ) {
    const Check& c = *static_cast<Check*>(p);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 8 * size_t(i);
        const cg::RayPre pr = cg::ray_prep(cg::mk(r[0], r[1], r[2]), cg::mk(r[4], r[5], r[6]), r[3], r[7]);
        cg::TraceCounters tc{0, 0};
        cg::HitD h;
        bool hit, any;
        if (dyn) {
            std::unique_ptr<cg::TravState> st(new cg::TravState());
            cg::trav_begin(*st, pr);
            while (!st->done) cg::trav_step<false, false>(c.S, pr, *st, &tc);
            hit = st->hslot >= 0;
            h.slot = st->hslot;
            h.t = st->tcur;
            h.u = st->hu;
            h.v = st->hv;
            cg::trav_begin(*st, pr);
            while (!st->done) cg::trav_step<true, false>(c.S, pr, *st, &tc);
            any = st->hslot >= 0;
        } else {
            hit = cg::traverse<false, false>(c.S, pr, &h, &tc);
            cg::HitD h2;
            any = cg::traverse<true, false>(c.S, pr, &h2, &tc);
        }
        prim[i] = hit ? __float_as_int(c.S.tris[h.slot].v0.w) : -1;
        t[i] = hit ? h.t : 0.0f;
        u[i] = hit ? h.u : 0.0f;
        v[i] = hit ? h.v : 0.0f;
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
        float3 L, Ls;
        cg::TraceCounters tc{0, 0}, ta{0, 0};
        uint32_t nc = 0, na = 0;
        cg::mk_path<false>(c.S, o, d, rng, &L, &Ls, &tc, &ta, &nc, &na);
        rgb[3 * i + 0] = L.x + Ls.x;
        rgb[3 * i + 1] = L.y + Ls.y;
        rgb[3 * i + 2] = L.z + Ls.z;
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
            float3 L, Ls;
            cg::TraceCounters tc{0, 0}, ta{0, 0};
            uint32_t nc = 0, na = 0;
            cg::mk_path<false>(c.S, o, d, rng, &L, &Ls, &tc, &ta, &nc, &na);
            float* q = out + 3 * (size_t(k) * npix + px);
            q[0] = L.x + Ls.x;
            q[1] = L.y + Ls.y;
            q[2] = L.z + Ls.z;
        }
}

}  // extern "C"
