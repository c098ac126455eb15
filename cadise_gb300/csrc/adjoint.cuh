// Per-path body of the path-replay adjoint (see adjoint.cu for the method):
// both replays of one path sample and the gradient terms of its vertices,
// handed to a sink.  The kernel's sink reduces into shared / global FP64
// memory with atomics; the CPU check of the kernel logic sums directly.
#pragma once

#include "pathtrace.cuh"

namespace cg {

// Sink interface:
//   rough(material, value)           d loss / d roughness of a material
//   rad(3 * light + channel, value)  d loss / d radiance of an area light
//   tex(texture, texel float, value) d loss / d albedo texel float
template <class Sink>
CG_D void adjoint_path(const SceneD& S, const PathId& id, uint64_t seed, float3 delta, int nlight, Sink& sink) {
    // ---- replay 1: the path's radiance
    Rng rng;
    float3 o, d;
    primary_ray(S, id, seed, rng, &o, &d);
    float3 L1, Le1, Ls1;
    TraceCounters tc{0, 0}, ta{0, 0};
    uint32_t nc = 0, na = 0;
    mk_path<false>(S, o, d, rng, &L1, &Le1, &Ls1, &tc, &ta, &nc, &na);
    const float3 Ltot = path_sample(L1, Le1, Ls1);
    if (!finite3(Ltot)) return;  // the film drops this sample too
    // ---- replay 2: the same path with gradient bookkeeping
    primary_ray(S, id, seed, rng, &o, &d);
    float3 T = splat3(1.0f), acc = splat3(0.0f);
    bool ce = true;
    for (int b = 0; b < S.max_depth; ++b) {
        const RayPre r = ray_prep(o, d, kRayEps, kFloatMax);
        HitD hit;
        if (!traverse<false, false>(S, r, &hit, &tc)) break;  // the sky has no parameters here
        const SurfaceD si = surface_at(S, o, d, hit);
        const VertexPlan pl = plan_vertex(S, si, T, ce, b, rng);
        const MaterialD& m = S.materials[si.material];
        // emission term E_j = T * Le
        if (si.light >= 0 && ce && can_emit(S.lights[si.light], si.wi, si.Ns)) {
            const float3 gx = delta * T;
            sink.rad(3 * si.light + 0, gx.x);
            sink.rad(3 * si.light + 1, gx.y);
            sink.rad(3 * si.light + 2, gx.z);
        }
        acc += pl.emit;
        float3 A = splat3(0.0f), B = splat3(0.0f);
        if (pl.shadow) {
            const RayPre sr = ray_prep(si.P, pl.sdir, kRayEps, pl.stmax);
            HitD sh;
            if (!traverse<true, false>(S, sr, &sh, &ta)) {
                A = pl.scontrib;
                if (pl.slight < nlight) {
                    const float3 gx = delta * pl.sx;
                    sink.rad(3 * pl.slight + 0, gx.x);
                    sink.rad(3 * pl.slight + 1, gx.y);
                    sink.rad(3 * pl.slight + 2, gx.z);
                }
            }
        }
        if (pl.mis) {
            const RayPre mr = ray_prep(si.P, pl.mdir, kRayEps, kFloatMax);
            HitD mh;
            const bool hitp = traverse<false, false>(S, mr, &mh, &tc);
            if (hitp && light_of_slot(S, mh.slot) == pl.mlight) {
                const SurfaceD hs = surface_at(S, si.P, pl.mdir, mh);
                float3 X;
                B = mis_resolve(S, hs, si.P, T, pl.mfactor, pl.mpdf, &X);
                const float3 gx = delta * X;
                sink.rad(3 * pl.mlight + 0, gx.x);
                sink.rad(3 * pl.mlight + 1, gx.y);
                sink.rad(3 * pl.mlight + 2, gx.z);
            } else if (!hitp && pl.mlight == S.env_light) {
                B = mis_resolve_env(S, pl.mdir, T, pl.mfactor, pl.mpdf);
            }
        }
        const float3 after = Ltot - acc - A - B;  // radiance of the vertices after this one
        if (m.type == BSDF_LAMBERTIAN && m.albedo_tex >= 0) {
            const TextureD& tex = S.textures[m.albedo_tex];
            const float3 alb = texture_rgb(tex, si.uvw);
            const float3 num = delta * (A + B + after);
            const int k = 3 * texel_index(tex, si.uvw);
            if (alb.x > 0.0f && num.x != 0.0f) sink.tex(m.albedo_tex, k + 0, double(num.x / alb.x));
            if (alb.y > 0.0f && num.y != 0.0f) sink.tex(m.albedo_tex, k + 1, double(num.y / alb.y));
            if (alb.z > 0.0f && num.z != 0.0f) sink.tex(m.albedo_tex, k + 2, double(num.z / alb.z));
        } else if (m.type == BSDF_CONDUCTOR || m.type == BSDF_DIELECTRIC_GGX) {
            float gr = 0.0f;
            if (!is_zero(A)) gr += dot(delta, A) * dlogf_droughness(m, si.wi, pl.sdir, si.Ns);
            if (!is_zero(B)) gr += dot(delta, B) * dlogf_droughness(m, si.wi, pl.mdir, si.Ns);
            if (pl.cont) gr += dot(delta, after) * dlogf_droughness(m, si.wi, pl.cdir, si.Ns);
            sink.rough(si.material, double(gr));
        }
        acc += A + B;
        if (!pl.cont) break;
        T = pl.T;
        ce = pl.count_emission != 0;
        o = si.P;
        d = pl.cdir;
    }
}

}  // namespace cg
