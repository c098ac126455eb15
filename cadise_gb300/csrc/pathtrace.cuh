// Per-path pieces shared by the render kernels and the adjoint: batch path
// indexing, primary rays, and the whole-path estimator (megakernel body).
#pragma once

#include "internal.h"
#include "shading.cuh"

namespace cg {

struct PathId {
    int scene;
    uint32_t pixel, sample, width;
};

CG_D int find_chunk(const Chunk* ch, int n, uint32_t p) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ch[mid].path_begin <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

CG_D PathId path_id(const Chunk* chunks, int nchunks, uint32_t p) {
    const Chunk& c = chunks[find_chunk(chunks, nchunks, p)];
    const uint32_t local = p - c.path_begin;
    PathId id;
    id.scene = c.scene;
    id.sample = c.sample0 + local / c.npix;
    id.pixel = local % c.npix;
    id.width = c.width;
    return id;
}

// fxy (optional): the sample's film position, for the film filter.
CG_D void primary_ray(const SceneD& S, const PathId& id, uint64_t seed, Rng& rng, float3* o, float3* d,
                      float2* fxy = nullptr) {
    rng.key = path_key(seed, uint32_t(id.scene), id.pixel, id.sample);
    rng.ctr = 0;
    float jx, jy;
    stratum_jitter(S.spp, id.sample, rng, &jx, &jy);
    const float fx = float(id.pixel % id.width) + jx;
    const float fy = float(id.pixel / id.width) + jy;
    camera_ray(S.cam, fx, fy, o, d);
    if (fxy) *fxy = make_float2(fx, fy);
}

CG_D int light_of_slot(const SceneD& S, int slot) {
    const float4* tp = reinterpret_cast<const float4*>(S.tris + slot);
    return int(__float_as_uint(ldg4(tp + 1).w) >> 16) - 1;
}
CG_D int material_of_slot(const SceneD& S, int slot) {
    const float4* tp = reinterpret_cast<const float4*>(S.tris + slot);
    return int(__float_as_uint(ldg4(tp + 1).w) & 0xFFFFu);
}

// Counting replay: [0] closest rays, [1] any-hit rays, [2] / [3] 4-wide
// nodes / triangles fetched by closest-hit rays, [4] / [5] by any-hit rays,
// [6] closest-hit rays traced again by the tie rule (k_wf_ties).
template <bool COUNT>
CG_D void count_flush(unsigned long long* counters, const TraceCounters& cc, const TraceCounters& ca, uint32_t closest,
                      uint32_t any) {
    if (!COUNT) return;
    if (closest) atomicAdd(counters + 0, (unsigned long long)closest);
    if (any) atomicAdd(counters + 1, (unsigned long long)any);
    if (cc.nodes) atomicAdd(counters + 2, (unsigned long long)cc.nodes);
    if (cc.tris) atomicAdd(counters + 3, (unsigned long long)cc.tris);
    if (ca.nodes) atomicAdd(counters + 4, (unsigned long long)ca.nodes);
    if (ca.tris) atomicAdd(counters + 5, (unsigned long long)ca.tris);
}

// A MIS ray adds its light's term only when its closest hit is the sampled
// light (or, for the environment, when it hits nothing).  So the shade pass
// tests the ray against that light's own records first, as the closest-hit
// traversal tests them (the smaller t of a rectangle's two halves; a first
// hit must lie within the ray's tmax): a ray that misses the light adds
// nothing whatever else it meets and is not traced.  A ray that meets it is
// left to k_wf_mis_occl, which asks only whether a primitive comes before
// that hit in closest-hit order - the same answer as the closest-hit pass,
// bit for bit, with an any-hit query bounded by the light's distance.
// Writes (t, slot, u, v) of the light's hit; slot -1 for the environment.
CG_D bool mis_light_hit(const SceneD& S, const RayPre& r, int mlight, float4* mh) {
    if (mlight == S.env_light) {
        *mh = make_float4(r.tmax, __int_as_float(-1), 0.0f, 0.0f);
        return true;
    }
    const LightD& L = S.lights[mlight];
    int best = -1;
    float bt = 0.0f, bu = 0.0f, bv = 0.0f;
    for (int k = 0; k < 2; ++k) {
        const int slot = L.slot[k];
        if (slot < 0) continue;
        const float4* tp = reinterpret_cast<const float4*>(S.tris + slot);
        const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
        float t, u, v;
        // the closest-hit pass's rule between the halves (closer_hit): the
        // smaller t, on a tie (the diagonal) the lower record slot
        if (tri_test(r, f3(a), f3(b), f3(c), r.tmax * 1.00000036f, &t, &u, &v) && t <= r.tmax &&
            (best < 0 || t < bt || (t == bt && slot < best))) {
            best = slot;
            bt = t;
            bu = u;
            bv = v;
        }
    }
    *mh = make_float4(bt, __int_as_float(best), bu, bv);
    return best >= 0;
}

// One whole path sample (PtEstimator::estimate): the megakernel body.
// Three accumulators, as the wavefront keeps them: L (emission and the
// BSDF-sampled half of NEE), Le (the sky seen by an escaping continuation
// ray) and Ls (the light-sampled half of NEE); the sample is (L + Le) + Ls.
// The same rays as the wavefront schedule: a shadow ray whose contribution
// is zero in every channel is not traced, and a MIS ray is resolved against
// its sampled light at the vertex (mis_light_hit) and, when it meets it,
// traced as an any-hit query bounded by the light's hit (occluded_before)
// instead of a closest-hit ray - the closest-hit answer bit for bit.
template <bool COUNT, bool SPH = true>
CG_D void mk_path(const SceneD& S, float3 o, float3 d, Rng& rng, float3* Lout, float3* Leout, float3* Lsout,
                  TraceCounters* tc, TraceCounters* ta, uint32_t* nclosest, uint32_t* nany) {
    float3 L = splat3(0.0f), Le = splat3(0.0f), Ls = splat3(0.0f), T = splat3(1.0f);
    bool ce = true;
    for (int b = 0; b < S.max_depth; ++b) {
        const RayPre r = ray_prep(o, d, kRayEps, kFloatMax);
        HitD hit;
        if (COUNT) ++*nclosest;
        if (!traverse<false, COUNT, SPH>(S, r, &hit, tc)) {
            if (S.env_light >= 0 && ce) Le = T * env_radiance(S, d);
            break;
        }
        const SurfaceD si = surface_at(S, o, d, hit);
        const VertexPlan pl = plan_vertex(S, si, T, ce, b, rng);
        L += pl.emit;
        if (pl.shadow && !is_zero(pl.scontrib)) {
            const RayPre sr = ray_prep(si.P, pl.sdir, kRayEps, pl.stmax);
            HitD sh;
            if (COUNT) ++*nany;
            if (!traverse<true, COUNT, SPH>(S, sr, &sh, ta)) Ls += pl.scontrib;
        }
        if (pl.mis) {
            const RayPre mr = ray_prep(si.P, pl.mdir, kRayEps, kFloatMax);
            float4 mh;
            if (mis_light_hit(S, mr, pl.mlight, &mh)) {
                const int slot = __float_as_int(mh.y);
                const int prim_l =
                    slot >= 0 ? __float_as_int(ldg4(reinterpret_cast<const float4*>(S.tris + slot)).w) : 0x7FFFFFFF;
                if (COUNT) ++*nany;
                if (!occluded_before<COUNT, SPH>(S, mr, mh.x, prim_l, slot, ta)) {
                    if (slot >= 0) {
                        HitD hit;
                        hit.t = mh.x;
                        hit.slot = slot;
                        hit.u = mh.z;
                        hit.v = mh.w;
                        const SurfaceD hs = surface_at(S, si.P, pl.mdir, hit);
                        L += mis_resolve(S, hs, si.P, T, pl.mfactor, pl.mpdf);
                    } else {
                        L += mis_resolve_env(S, pl.mdir, T, pl.mfactor, pl.mpdf);
                    }
                }
            }
        }
        if (!pl.cont) break;
        T = pl.T;
        ce = pl.count_emission != 0;
        o = si.P;
        d = pl.cdir;
    }
    *Lout = L;
    *Leout = Le;
    *Lsout = Ls;
}

CG_HD float3 path_sample(float3 L, float3 Le, float3 Ls) { return (L + Le) + Ls; }

}  // namespace cg
