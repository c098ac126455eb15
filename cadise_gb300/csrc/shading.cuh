// Camera, surface reconstruction, BSDFs, area lights and the per-vertex
// plan of the NEE + MIS path estimator.
//
// Behaviour follows the reference estimator PtEstimator::estimate
// (source/core/estimator/ptEstimator.cpp:25-123) and its callees; each device
// function names the reference routine it stands for.  One vertex is split
// into `plan_vertex` (draws every random number the reference draws at that
// vertex, in the reference's order, and emits up to three rays: the shadow
// ray, the MIS BSDF ray and the continuation ray) and the resolve functions
// that turn trace results into radiance.  The megakernel and the wavefront
// scheduler both run exactly these functions, so they produce the same
// per-path result.
#pragma once

#include "traverse.cuh"

namespace cg {

// ------------------------------------------------------------------ camera --
// PerspectivePinholeCamera::spawnPrimaryRay (perspectivePinholeCamera.cpp:52-73)
CG_D void camera_ray(const CameraD& c, float fx, float fy, float3* o, float3* d) {
    const float cx = c.sx * fx + c.tx;
    const float cy = c.sy * fy + c.ty;
    const float cz = -c.offset;
    const float3 v = mk(c.ax.x * cx + c.ay.x * cy + c.az.x * cz,
                        c.ax.y * cx + c.ay.y * cy + c.az.y * cz,
                        c.ax.z * cx + c.ay.z * cy + c.az.z * cz);
    *o = c.pos;
    *d = normalize(v);
}

// Sample `s` of a pixel: stratum s of the floor(sqrt(spp))^2 grid (uniform
// beyond it), jittered by the first two draws of the path stream - the set
// StratifiedSampler::requestSample2D builds (stratifiedSampler.cpp:38-73)
// minus its in-pixel shuffle.
CG_D void stratum_jitter(int spp, uint32_t s, Rng& rng, float* jx, float* jy) {
    const int base = int(floorf(sqrtf(float(spp))));
    const float u0 = rng.next(), u1 = rng.next();
    if (int(s) < base * base) {
        const float inv = 1.0f / float(base);
        *jx = (float(s % uint32_t(base)) + u0) * inv;
        *jy = (float(s / uint32_t(base)) + u1) * inv;
    } else {
        *jx = u0;
        *jy = u1;
    }
}

// SphericalMapper::mappingToUvw (sphericalMapper.cpp:14-28): y up,
// phi = atan2(x, z), u = phi / 2 pi, v = (pi - theta) / pi.
CG_D float3 env_uvw(float3 d) {
    const float3 n = normalize(d);
    const float theta = acosf(fminf(fmaxf(n.y, -1.0f), 1.0f));
    float phi = atan2f(n.x, n.z);
    if (phi < 0.0f) phi += 2.0f * kPi;
    return mk(phi * 0.1591549430918953f, (kPi - theta) * kInvPi, 0.0f);
}

// ----------------------------------------------------------------- surface --
struct SurfaceD {
    float3 P, Ng, Ns, uvw, wi;
    int prim, material, light;
};

// The distance the reference reports for the primitive a ray hit: the
// Moller-Trumbore distance of a triangle (triangle.cpp:54-89, edges swapped
// to face the ray) or the plane distance of a rectangle (rectangle.cpp:49-75).
// The traversal's watertight distance `t_wt` decides which primitive is hit;
// this one places the hit point, so that o + d t is the reference's point to
// the bit (the next ray starts there: one ulp decides self-shadowing at
// grazing angles).  Falls back to t_wt where the formula degenerates.
CG_D float ref_tri_t(float3 o, float3 d, float3 A, float3 B, float3 C, float t_wt) {
    float3 eAB = B - A, eAC = C - A;
    if (dot(d, cross(eAB, eAC)) > 0.0f) {
        const float3 t = eAB;
        eAB = eAC;
        eAC = t;
    }
    const float3 T = o - A;
    const float3 Q = cross(T, eAB);
    const float3 P = cross(d, eAC);
    const float den = dot(P, eAB);
    if (den == 0.0f) return t_wt;
    const float inv = 1.0f / den;
    const float t = dot(Q, eAC) * inv;
    return isfinite(t) ? t : t_wt;
}
CG_D float ref_rect_t(float3 o, float3 d, float3 vB, float3 eA, float3 eB, float t_wt) {
    if (dot(d, cross(eA, eB)) > 0.0f) {
        const float3 t = eA;
        eA = eB;
        eB = t;
    }
    const float3 n = normalize(cross(eA, eB));
    const float t = dot(n, vB - o) / dot(n, d);
    return isfinite(t) ? t : t_wt;
}

// Hit point, reference distance and surface coordinates of a closest hit:
// for a triangle the barycentrics of its vertices recomputed from the hit
// point (Triangle::barycentric, triangle.cpp:233-262); for a rectangle the
// edge coordinates (p1, p2), both divided by |eA| as rectangle.cpp:122-129
// does.
struct HitPoint {
    float t;
    float3 P;
    float b0, b1, b2;  // triangle barycentrics (b1 of B, b2 of C)
    float p1, p2;      // rectangle coordinates
    int rect;          // rectangle index, -1 for a triangle or a sphere
    int sphere;        // 1 for a sphere (its t is the traversal's, already the reference's)
};

CG_D void rect_frame(const SceneD& S, int rect, float3* vB, float3* eA, float3* eB) {
    const float* fr = S.rect_frames + 9 * size_t(rect);
    *vB = mk(fr[0], fr[1], fr[2]);
    *eA = mk(fr[3], fr[4], fr[5]);
    *eB = mk(fr[6], fr[7], fr[8]);
}

CG_D HitPoint hit_point(const SceneD& S, float3 o, float3 d, const HitD& h) {
    HitPoint hp;
    const float4* tp = reinterpret_cast<const float4*>(S.tris + h.slot);
    const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
    const uint32_t flags = __float_as_uint(c.w);
    hp.sphere = (flags & 3u) == kRecSphere;
    if (hp.sphere) {
        hp.rect = -1;
        hp.t = h.t;
        hp.P = o + d * hp.t;
        hp.b0 = hp.b1 = hp.b2 = hp.p1 = hp.p2 = 0.0f;
        return hp;
    }
    if ((flags & 3u) == kRecRectHalf) {
        hp.rect = int(flags >> 2);
        float3 vB, eA, eB;
        rect_frame(S, hp.rect, &vB, &eA, &eB);
        hp.t = ref_rect_t(o, d, vB, eA, eB, h.t);
        hp.P = o + d * hp.t;
        const float3 onp = hp.P - vB;
        const float la = len(eA);
        hp.p1 = dot(onp, normalize(eA)) / la;
        hp.p2 = dot(onp, normalize(eB)) / la;
        hp.b0 = hp.b1 = hp.b2 = 0.0f;
        return hp;
    }
    hp.rect = -1;
    const float3 A = f3(a), B = f3(b), C = f3(c);
    hp.t = ref_tri_t(o, d, A, B, C, h.t);
    hp.P = o + d * hp.t;
    const float3 v0 = B - A, v1 = C - A, v2 = hp.P - A;
    const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    const float den = d00 * d11 - d01 * d01;
    if (den == 0.0f) {
        hp.b0 = hp.b1 = hp.b2 = 0.0f;
    } else {
        const float inv = 1.0f / den;
        hp.b1 = (d11 * d20 - d01 * d21) * inv;
        hp.b2 = (d00 * d21 - d01 * d20) * inv;
        hp.b0 = 1.0f - hp.b1 - hp.b2;
    }
    hp.p1 = hp.p2 = 0.0f;
    return hp;
}

// Scene::isIntersecting surface detail (scene.cpp:30-65, triangle.cpp:125-160,
// rectangle.cpp:102-132).
CG_D SurfaceD surface_at(const SceneD& S, float3 o, float3 d, const HitD& h) {
    SurfaceD si;
    const float4* tp = reinterpret_cast<const float4*>(S.tris + h.slot);
    const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
    si.prim = __float_as_int(a.w);
    const uint32_t packed = __float_as_uint(b.w);
    si.material = int(packed & 0xFFFFu);
    si.light = int(packed >> 16) - 1;
    const HitPoint hp = hit_point(S, o, d, h);
    si.P = hp.P;
    si.wi = -d;
    if (hp.sphere) {
        // Sphere::evaluateSurfaceDetail (sphere.cpp:106-135): the normal from
        // the centre, uvw from SphericalMapper (sphericalMapper.cpp:14-28)
        const float3 N = normalize(hp.P - f3(a));
        si.Ng = N;
        si.Ns = N;
        si.uvw = env_uvw(N);
        return si;
    }
    if (hp.rect >= 0) {
        // normal and uvw from the rectangle's own frame; the uvw is the
        // bilinear blend of the corner uvws (1,0) (0,0) (0,1) (1,1) as the
        // reference evaluates it, which rounds like this
        float3 vB, eA, eB;
        rect_frame(S, hp.rect, &vB, &eA, &eB);
        float3 N = cross(eA, eB);
        N = is_zero(N) ? mk(0.0f, 1.0f, 0.0f) : normalize(N);
        si.Ng = N;
        si.Ns = N;
        const float p1 = hp.p1, p2 = hp.p2;
        si.uvw = mk(p1 * ((1.0f - p2) + p2), (1.0f - p1) * p2 + p1 * p2, 0.0f);
        return si;
    }
    const float b0 = hp.b0, b1 = hp.b1, b2 = hp.b2;
    const float3 A = f3(a), B = f3(b), C = f3(c);
    float3 Ng = cross(B - A, C - A);
    Ng = is_zero(Ng) ? mk(0.0f, 1.0f, 0.0f) : normalize(Ng);
    si.Ng = Ng;
    // the vertex normals start as the face normal and a mesh's own replace
    // them where non-zero (triangle.cpp:15-41, triangleMesh.cpp:24-28); the
    // shading normal always interpolates them, which rounds differently from
    // the face normal itself even on a flat mesh (triangle.cpp:125-160)
    float3 nA = Ng, nB = Ng, nC = Ng;
    if (S.prim_normals) {
        const float* n = S.prim_normals + 9 * size_t(si.prim);
        const float3 a3 = mk(n[0], n[1], n[2]), b3 = mk(n[3], n[4], n[5]), c3 = mk(n[6], n[7], n[8]);
        if (!is_zero(a3)) nA = a3;
        if (!is_zero(b3)) nB = b3;
        if (!is_zero(c3)) nC = c3;
    }
    const float3 Ns = nA * b0 + nB * b1 + nC * b2;
    si.Ns = is_zero(Ns) ? Ng : normalize(Ns);
    if (S.prim_uvws) {
        const float* u = S.prim_uvws + 9 * size_t(si.prim);
        si.uvw = mk(u[0], u[1], u[2]) * b0 + mk(u[3], u[4], u[5]) * b1 + mk(u[6], u[7], u[8]) * b2;
    } else {
        si.uvw = mk(b1, b2, 0.0f);
    }
    return si;
}

// ------------------------------------------------------------------ texture --
// RgbImageTexture + TNearestPixelSampler + RepeatUvwWrapper
// (rgbImageTexture.cpp:8-15, tNearestPixelSampler.ipp:14-31, repeatUvwWrapper.cpp:9-15)
CG_D float3 texture_rgb(const TextureD& t, float3 uvw) {
    const float u = uvw.x - floorf(uvw.x), v = uvw.y - floorf(uvw.y);
    int x = int(u * float(t.width)), y = int(v * float(t.height));
    x = x < t.width ? x : x - 1;
    y = y < t.height ? y : y - 1;
    const float* p = t.texels + 3 * (size_t(y) * size_t(t.width) + size_t(x));
    return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

CG_D float3 albedo_of(const SceneD& S, const MaterialD& m, float3 uvw) {
    return m.albedo_tex >= 0 ? texture_rgb(S.textures[m.albedo_tex], uvw) : m.albedo;
}

// --------------------------------------------------------------------- GGX --
// IsotropicGgx (isotropicGgx.cpp:11-100), Microfacet::_isShadowingMaskingValid
// (microfacet.cpp:11-23)
CG_D float ggx_D(float alpha, float NdotH) {
    if (NdotH <= 0.0f) return 0.0f;
    const float a2 = alpha * alpha, c2 = NdotH * NdotH, c4 = c2 * c2;
    const float tan2 = (1.0f - c2) / c2;
    return a2 / (kPi * c4 * (a2 + tan2) * (a2 + tan2));
}
CG_D float ggx_G1(float alpha, float cosv) {
    const float c2 = cosv * cosv;
    return 2.0f / (1.0f + sqrtf(1.0f + alpha * alpha * ((1.0f - c2) / c2)));
}
CG_D float ggx_G(float alpha, float3 V, float3 L, float3 N, float3 H) {
    const float VdotH = dot(V, H), VdotN = dot(V, N), LdotH = dot(L, H), LdotN = dot(L, N);
    if (!((VdotH * VdotN > 0.0f) && (LdotH * LdotN > 0.0f))) return 0.0f;
    return ggx_G1(alpha, VdotN) * ggx_G1(alpha, LdotN);
}
// D(h) cos(theta_h) sampling: tan(theta) = alpha sqrt(u / (1 - u)), u clamped to
// [0, 0.9999]; cos(theta) = sqrt((1 - u) / (1 - u + alpha^2 u)).
CG_D float3 ggx_sample_h(float alpha, float u0, float u1) {
    const float s0 = fminf(fmaxf(u0, 0.0f), 0.9999f);
    const float s1 = fminf(fmaxf(u1, 0.0f), 0.9999f);
    float sp, cp;
    sincospif(2.0f * s0, &sp, &cp);
    const float a2 = alpha * alpha;
    const float c = sqrtf((1.0f - s1) / (1.0f - s1 + a2 * s1));
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    return mk(sp * s, c, cp * s);
}
// SchlickConductorFresnel::evaluateReflectance (schlickConductorFresnel.cpp:28-41)
CG_D float3 schlick(float3 f0, float cosI) {
    const float c = 1.0f - fabsf(cosI);
    return f0 + (splat3(1.0f) - f0) * (c * (c * c) * (c * c));
}
// VanillaDielectricFresnel::evaluateReflectance (vanillaDielectricFresnel.cpp:17-48)
CG_D float fresnel_dielectric(float etaI, float etaT, float cosI) {
    if (cosI < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; cosI = -cosI; }
    const float ratio = etaI / etaT;
    const float sinT2 = ratio * ratio * (1.0f - cosI * cosI);
    if (sinT2 >= 1.0f) return 1.0f;
    const float cosT = sqrtf(1.0f - sinT2);
    const float rPar = (etaT * cosI - etaI * cosT) / (etaT * cosI + etaI * cosT);
    const float rPer = (etaI * cosI - etaT * cosT) / (etaI * cosI + etaT * cosT);
    return 0.5f * (rPar * rPar + rPer * rPer);
}
// TVector::canRefract (tVector.ipp:468-503)
CG_D bool refract_dir(float3 v, float3 n, float etaI, float etaT, float3* out) {
    float sgn = 1.0f;
    const float cosI = dot(v, n);
    if (cosI < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; sgn = -1.0f; }
    const float ratio = etaI / etaT;
    const float sinT2 = ratio * ratio * (1.0f - cosI * cosI);
    if (sinT2 >= 1.0f) return false;
    const float cosT = sqrtf(1.0f - sinT2);
    *out = normalize(v * (-ratio) + n * ((ratio * sgn * cosI - cosT) * sgn));
    return true;
}

// -------------------------------------------------------------------- BSDF --
// A BSDF with a specular lobe: no next-event estimation at its vertices
// (ptEstimator.cpp:64-72 tests the lobes for SPECULAR_REFLECTION / _TRANSMISSION).
CG_HD bool bsdf_is_specular(int type) { return type == BSDF_GLASS || type == BSDF_MIRROR; }

// PhongBsdf (phongBsdf.cpp:14-98): pow(max(R.V, 0), e) with R = L.reflect(Ns),
// value factor (e + 2) / 2 pi, pdf factor (e + 1) / 2 pi.  Zero when V and L
// are on different sides.
CG_D float phong_power(const MaterialD& m, float3 V, float3 L, float3 N) {
    if (dot(V, N) * dot(L, N) <= 0.0f) return -1.0f;
    const float3 R = reflect(L, N);
    const float RdotV = fmaxf(dot(R, V), 0.0f);
    return powf(RdotV, m.exponent);
}
CG_D float phong_value_factor(const MaterialD& m) { return (m.exponent + 2.0f) * 0.1591549430918953f; }
CG_D float phong_pdf_factor(const MaterialD& m) { return (m.exponent + 1.0f) * 0.1591549430918953f; }

// LambertianDiffuse::evaluate / evaluatePdfW (lambertianDiffuse.cpp:27-44, 83-96)
CG_D float3 lambert_eval(const SceneD& S, const MaterialD& m, const SurfaceD& si, float3 L) {
    if (dot(si.wi, si.Ns) * dot(L, si.Ns) <= 0.0f) return splat3(0.0f);
    return albedo_of(S, m, si.uvw) * kInvPi;
}
CG_D float lambert_pdf(const SurfaceD& si, float3 L) {
    if (dot(si.wi, si.Ns) * dot(L, si.Ns) <= 0.0f) return 0.0f;
    return absdot(L, si.Ns) * kInvPi;
}
CG_D float3 phong_eval(const MaterialD& m, const SurfaceD& si, float3 L) {
    const float p = phong_power(m, si.wi, L, si.Ns);
    return splat3(p < 0.0f ? 0.0f : p * phong_value_factor(m));
}
CG_D float phong_pdf(const MaterialD& m, const SurfaceD& si, float3 L) {
    const float p = phong_power(m, si.wi, L, si.Ns);
    return p < 0.0f ? 0.0f : p * phong_pdf_factor(m);
}

// Rough dielectric (no reference counterpart): GGX BRDF + BTDF of Walter,
// Marschner, Li & Torrance, "Microfacet Models for Refraction through Rough
// Surfaces" (EGSR 2007), radiance form, Fresnel-weighted lobe choice.
// Everything is expressed with the normal turned to V's side.
CG_D void rough_dielectric_eval(const MaterialD& m, float3 albedo, float3 V, float3 L, float3 N, float3* f, float* pdf) {
    *f = splat3(0.0f);
    *pdf = 0.0f;
    const float cv = dot(V, N), cl = dot(L, N);
    if (cv == 0.0f || cl == 0.0f) return;
    const float3 Nv = cv > 0.0f ? N : -N;
    const float etaV = cv > 0.0f ? m.ior_outer : m.ior_inner;
    const float etaL = cv > 0.0f ? m.ior_inner : m.ior_outer;
    const float acv = fabsf(cv), acl = fabsf(cl);
    const float alpha = m.alpha;
    if (cv * cl > 0.0f) {
        float3 H = V + L;
        if (is_zero(H)) return;
        H = normalize(H);
        const float VH = dot(V, H);
        if (VH <= 0.0f) return;
        const float F = fresnel_dielectric(etaV, etaL, VH);
        const float NH = dot(Nv, H);
        const float D = ggx_D(alpha, NH);
        const float G = ggx_G(alpha, V, L, Nv, H);
        *f = albedo * (F * D * G / (4.0f * acv * acl));
        *pdf = F * D * NH / (4.0f * VH);
    } else {
        const float eta = etaL / etaV;
        float3 H = V + L * eta;
        if (is_zero(H)) return;
        H = normalize(H);
        if (dot(H, Nv) < 0.0f) H = -H;
        const float VH = dot(V, H), LH = dot(L, H);
        if (!(VH > 0.0f && LH < 0.0f)) return;
        const float F = fresnel_dielectric(etaV, etaL, VH);
        const float NH = dot(Nv, H);
        const float D = ggx_D(alpha, NH);
        const float G = ggx_G(alpha, V, L, Nv, H);
        const float den = VH + eta * LH;
        const float den2 = den * den;
        *f = albedo * ((1.0f - F) * D * G * fabsf(VH * LH) / (acv * acl * den2));
        *pdf = (1.0f - F) * D * NH * eta * eta * fabsf(LH) / den2;
    }
    if (!isfinite(*pdf)) { *pdf = 0.0f; *f = splat3(0.0f); }
}

// Bsdf::evaluate (lambertianDiffuse.cpp:27-44, conductorMicrofacet.cpp:32-66)
template <int Q = -1>
CG_D float3 bsdf_eval(const SceneD& S, const MaterialD& m, const SurfaceD& si, float3 L) {
    const float3 N = si.Ns, V = si.wi;
    if (queue_has<Q>(BSDF_LAMBERTIAN) && m.type == BSDF_LAMBERTIAN) {
        if (dot(V, N) * dot(L, N) <= 0.0f) return splat3(0.0f);
        return albedo_of(S, m, si.uvw) * kInvPi;
    }
    if (queue_has<Q>(BSDF_CONDUCTOR) && m.type == BSDF_CONDUCTOR) {
        const float VdotN = dot(V, N), LdotN = dot(L, N);
        if (VdotN * LdotN <= 0.0f) return splat3(0.0f);
        float3 H = (V + L) * (VdotN > 0.0f ? 1.0f : -1.0f);
        if (is_zero(H)) return splat3(0.0f);
        H = normalize(H);
        const float3 F = schlick(m.f0, dot(L, H));
        const float D = ggx_D(m.alpha, dot(N, H));
        const float G = ggx_G(m.alpha, V, L, N, H);
        return F * G * D * (1.0f / (4.0f * fabsf(VdotN * LdotN)));
    }
    if (queue_has<Q>(BSDF_DIELECTRIC_GGX) && m.type == BSDF_DIELECTRIC_GGX) {
        float3 f;
        float pdf;
        rough_dielectric_eval(m, albedo_of(S, m, si.uvw), V, L, N, &f, &pdf);
        return f;
    }
    if (queue_has<Q>(BSDF_PHONG) && m.type == BSDF_PHONG) return phong_eval(m, si, L);
    if (queue_has<Q>(BSDF_PLASTIC) && m.type == BSDF_PLASTIC) {  // MixedBsdf::evaluate (mixedBsdf.cpp:33-57), A Lambert, B Phong
        return lambert_eval(S, m, si, L) * m.ratio + phong_eval(m, si, L) * (1.0f - m.ratio);
    }
    return splat3(0.0f);  // glass, mirror, absorber: no non-delta part
}

// Bsdf::evaluatePdfW (lambertianDiffuse.cpp:83-96, conductorMicrofacet.cpp:126-163)
template <int Q = -1>
CG_D float bsdf_pdf(const SceneD& S, const MaterialD& m, const SurfaceD& si, float3 L) {
    const float3 N = si.Ns, V = si.wi;
    if (queue_has<Q>(BSDF_LAMBERTIAN) && m.type == BSDF_LAMBERTIAN) {
        if (dot(V, N) * dot(L, N) <= 0.0f) return 0.0f;
        return absdot(L, N) * kInvPi;
    }
    if (queue_has<Q>(BSDF_CONDUCTOR) && m.type == BSDF_CONDUCTOR) {
        const float VdotN = dot(V, N), LdotN = dot(L, N);
        if (VdotN * LdotN <= 0.0f) return 0.0f;
        float3 H = (V + L) * (VdotN > 0.0f ? 1.0f : -1.0f);
        if (is_zero(H)) return 0.0f;
        H = normalize(H);
        const float D = ggx_D(m.alpha, dot(N, H));
        const float pdfL = fabsf(fabsf(D * dot(N, H)) / (4.0f * dot(L, H)));
        return isfinite(pdfL) ? pdfL : 0.0f;
    }
    if (queue_has<Q>(BSDF_DIELECTRIC_GGX) && m.type == BSDF_DIELECTRIC_GGX) {
        float3 f;
        float pdf;
        rough_dielectric_eval(m, splat3(1.0f), V, L, N, &f, &pdf);
        return pdf;
    }
    if (queue_has<Q>(BSDF_PHONG) && m.type == BSDF_PHONG) return phong_pdf(m, si, L);
    if (queue_has<Q>(BSDF_PLASTIC) && m.type == BSDF_PLASTIC) {  // MixedBsdf::evaluatePdfW (mixedBsdf.cpp:157-185)
        const float avg = (m.ratio + m.ratio + m.ratio) / 3.0f;
        return lambert_pdf(si, L) * avg + phong_pdf(m, si, L) * (1.0f - avg);
    }
    return 0.0f;
}

struct BsdfS {
    float3 f, L;
    float pdf;
    CG_D bool valid() const { return !is_zero(f) && pdf > 0.0f; }  // bsdfSample.cpp:39-41
};

// LambertianDiffuse::evaluateSample (lambertianDiffuse.cpp:46-81) with
// Hemisphere::cosineWeightedSampling (hemisphere.cpp:30-48):
// theta = acos(1 - 2 u1) / 2, i.e. cos(theta) = sqrt(1 - u1)
CG_D BsdfS lambert_sample(const SceneD& S, const MaterialD& m, const SurfaceD& si, Rng& rng) {
    BsdfS out;
    const float3 N = si.Ns, V = si.wi;
    float3 z, x;
    frame_from_y(N, &z, &x);
    float u0, u1;
    rng.next2(&u0, &u1);
    float sp, cp;
    sincospif(2.0f * u0, &sp, &cp);
    const float c = sqrtf(1.0f - u1);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    float3 L = x * (sp * s) + N * c + z * (cp * s);
    L = normalize(L);
    if (dot(V, N) <= 0.0f) L = -L;
    out.f = albedo_of(S, m, si.uvw) * kInvPi;
    out.L = L;
    out.pdf = c * kInvPi;
    return out;
}

// PhongBsdf::evaluateSample (phongBsdf.cpp:38-81) with
// Hemisphere::cosineExpWeightedSampling (hemisphere.cpp:50-69): the lobe
// sampled around the shading normal, its value and pdf evaluated around the
// mirror direction, as the reference does.
CG_D BsdfS phong_sample(const MaterialD& m, const SurfaceD& si, Rng& rng) {
    BsdfS out;
    out.f = splat3(0.0f);
    out.L = mk(0.0f, 1.0f, 0.0f);
    out.pdf = 0.0f;
    const float3 N = si.Ns, V = si.wi;
    float3 z, x;
    frame_from_y(N, &z, &x);
    float u0, u1;
    rng.next2(&u0, &u1);
    float sp, cp;
    sincospif(2.0f * u0, &sp, &cp);
    const float c = powf(u1, 1.0f / (m.exponent + 1.0f));
    const float s = sqrtf(1.0f - c * c);
    const float3 L = normalize(x * (sp * s) + N * c + z * (cp * s));
    const float p = phong_power(m, V, L, N);
    if (p < 0.0f) return out;
    out.f = splat3(p * phong_value_factor(m));
    out.L = L;
    out.pdf = p * phong_pdf_factor(m);
    return out;
}

// MixedBsdf::evaluateSample (mixedBsdf.cpp:59-155) of plastic: one draw picks
// the lobe by the average ratio; the other lobe is evaluated at the sampled
// direction.  When Phong (B) is sampled the reference weights its value by
// the ratio and Lambert's by its complement, as written there
// (mixedBsdf.cpp:123-128); so does this.
CG_D BsdfS plastic_sample(const SceneD& S, const MaterialD& m, const SurfaceD& si, Rng& rng) {
    BsdfS out;
    out.f = splat3(0.0f);
    out.L = mk(0.0f, 1.0f, 0.0f);
    out.pdf = 0.0f;
    const float avg = (m.ratio + m.ratio + m.ratio) / 3.0f;
    const float u = rng.next();
    if (u < avg) {
        const BsdfS a = lambert_sample(S, m, si, rng);
        if (!a.valid()) return out;
        out.L = a.L;
        out.f = a.f * m.ratio + phong_eval(m, si, a.L) * (1.0f - m.ratio);
        out.pdf = avg * a.pdf + (1.0f - avg) * phong_pdf(m, si, a.L);
    } else {
        const BsdfS b = phong_sample(m, si, rng);
        if (!b.valid()) return out;
        out.L = b.L;
        out.f = b.f * m.ratio + lambert_eval(S, m, si, b.L) * (1.0f - m.ratio);
        out.pdf = avg * b.pdf + (1.0f - avg) * lambert_pdf(si, b.L);
    }
    return out;
}

// SpecularReflection::evaluateSample (specularReflection.cpp:32-57), pdf 1
CG_D BsdfS mirror_sample(const SceneD& S, const MaterialD& m, const SurfaceD& si) {
    BsdfS out;
    const float3 N = si.Ns, V = si.wi;
    const float VdotN = dot(V, N);
    const float3 L = reflect(V, N * (VdotN > 0.0f ? 1.0f : -1.0f));
    const float LdotN = dot(L, N);
    const float3 R = m.fresnel == 0 ? schlick(m.f0, LdotN)
                                    : splat3(fresnel_dielectric(m.ior_outer, m.ior_inner, LdotN));
    out.f = divs(R * albedo_of(S, m, si.uvw), fabsf(LdotN));
    out.L = L;
    out.pdf = 1.0f;
    return out;
}

// Bsdf::evaluateSample (lambertianDiffuse.cpp:46-81, conductorMicrofacet.cpp:68-124,
// specularDielectric.cpp:35-127)
template <int Q = -1>
CG_D BsdfS bsdf_sample(const SceneD& S, const MaterialD& m, const SurfaceD& si, Rng& rng) {
    BsdfS out;
    out.f = splat3(0.0f);
    out.L = mk(0.0f, 1.0f, 0.0f);
    out.pdf = 0.0f;
    const float3 N = si.Ns, V = si.wi;
    if (queue_has<Q>(BSDF_LAMBERTIAN) && m.type == BSDF_LAMBERTIAN) return lambert_sample(S, m, si, rng);
    if (queue_has<Q>(BSDF_PHONG) && m.type == BSDF_PHONG) return phong_sample(m, si, rng);
    if (queue_has<Q>(BSDF_PLASTIC) && m.type == BSDF_PLASTIC) return plastic_sample(S, m, si, rng);
    if (queue_has<Q>(BSDF_MIRROR) && m.type == BSDF_MIRROR) return mirror_sample(S, m, si);
    if (queue_has<Q>(BSDF_CONDUCTOR) && m.type == BSDF_CONDUCTOR) {
        const float nf = dot(V, N) > 0.0f ? 1.0f : -1.0f;
        float3 z, x;
        frame_from_y(N, &z, &x);
        float u0, u1;
        rng.next2(&u0, &u1);
        const float3 hl = ggx_sample_h(m.alpha, u0, u1);
        const float3 H = normalize(x * hl.x + N * hl.y + z * hl.z);
        const float3 L = reflect(V, H * nf);
        const float VdotN = dot(V, N), LdotN = dot(L, N), LdotH = dot(L, H), NdotH = dot(N, H);
        if (VdotN * LdotN <= 0.0f) return out;
        const float3 F = schlick(m.f0, LdotH);
        const float D = ggx_D(m.alpha, NdotH);
        const float G = ggx_G(m.alpha, V, L, N, H);
        const float pdfL = fabsf(fabsf(D * NdotH) / (4.0f * LdotH));
        if (!isfinite(pdfL)) return out;
        out.f = F * G * D * (1.0f / (4.0f * fabsf(VdotN * LdotN)));
        out.L = L;
        out.pdf = pdfL;
        return out;
    }
    if (queue_has<Q>(BSDF_GLASS) && m.type == BSDF_GLASS) {
        const float VdotN = dot(V, N);
        const float R = fresnel_dielectric(m.ior_outer, m.ior_inner, VdotN);
        const float pr = (R + R + R) / 3.0f;  // Spectrum::average of a grey reflectance
        const float u = rng.next();
        const float3 alb = albedo_of(S, m, si.uvw);
        if (u < pr) {
            const float3 L = reflect(V, N * (VdotN > 0.0f ? 1.0f : -1.0f));
            out.f = alb * R * (1.0f / absdot(L, N));
            out.L = L;
            out.pdf = pr;
        } else {
            float3 L;
            if (!refract_dir(V, N, m.ior_outer, m.ior_inner, &L)) return out;
            const float cosI = dot(L, N);
            const float Rt = fresnel_dielectric(m.ior_outer, m.ior_inner, cosI);
            float etaI = m.ior_outer, etaT = m.ior_inner;
            if (cosI < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
            const float btdf = (etaT * etaT) / (etaI * etaI);
            out.f = alb * (1.0f - Rt) * btdf * (1.0f / fabsf(cosI));
            out.L = L;
            out.pdf = 1.0f - pr;
        }
        return out;
    }
    if (queue_has<Q>(BSDF_DIELECTRIC_GGX) && m.type == BSDF_DIELECTRIC_GGX) {
        const float cv = dot(V, N);
        if (cv == 0.0f) return out;
        const float3 Nv = cv > 0.0f ? N : -N;
        const float etaV = cv > 0.0f ? m.ior_outer : m.ior_inner;
        const float etaL = cv > 0.0f ? m.ior_inner : m.ior_outer;
        float3 z, x;
        frame_from_y(Nv, &z, &x);
        float u0, u1;
        rng.next2(&u0, &u1);
        const float3 hl = ggx_sample_h(m.alpha, u0, u1);
        const float3 H = normalize(x * hl.x + Nv * hl.y + z * hl.z);
        const float VH = dot(V, H);
        const float u = rng.next();
        if (VH <= 0.0f) return out;
        const float F = fresnel_dielectric(etaV, etaL, VH);
        float3 L;
        if (u < F) {
            L = H * (2.0f * VH) - V;
        } else {
            const float ratio = etaV / etaL;
            const float sinT2 = ratio * ratio * (1.0f - VH * VH);
            if (sinT2 >= 1.0f) return out;
            const float cosT = sqrtf(1.0f - sinT2);
            L = normalize(V * (-ratio) + H * (ratio * VH - cosT));
        }
        float3 f;
        float pdf;
        rough_dielectric_eval(m, albedo_of(S, m, si.uvw), V, L, N, &f, &pdf);
        out.f = f;
        out.L = L;
        out.pdf = pdf;
        return out;
    }
    return out;  // absorber: never valid (absorberBsdf.cpp)
}

// ------------------------------------------------------------------ lights --
CG_D bool can_emit(const LightD& l, float3 dir, float3 N) { return (dot(dir, N) >= 0.0f) != (l.back_face != 0); }

struct LightS {
    float3 pos, radiance;
    float pdfW;
    CG_D bool valid() const { return !is_zero(radiance) && pdfW > 0.0f; }  // directLightSample.cpp:53-55
};

// ------------------------------------------------------------- environment --
// One direction <-> (u, v) mapping for both lookup and sampling: the one of
// SphericalMapper::mappingToUvw (sphericalMapper.cpp:14-28), y up,
// phi = atan2(x, z), v = (pi - theta) / pi.  (The reference samples with a
// z-up inverse, infiniteSphere.cpp:62-78, which does not invert its lookup;
// this library keeps one mapping so NEE and BSDF sampling see the same sky.)
CG_D float3 env_dir(float u, float v) {
    const float theta = (1.0f - v) * kPi;
    float sp, cp, st, ct;
    sincospif(2.0f * u, &sp, &cp);
    sincospif(1.0f - v, &st, &ct);
    (void)theta;
    return mk(st * sp, ct, st * cp);
}
CG_D int cdf_find(const float* cdf, int n, float u) {
    int lo = 0, hi = n - 1;  // largest i with cdf[i] <= u, in [0, n-1]
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(cdf + mid) <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// pdf over (u, v) in [0, 1]^2 (Distribution2D::pdfContinuous, distribution2D.cpp:42-50)
CG_D float env_pdf_uv(const LightD& l, float u, float v) {
    int iy = min(int(v * float(l.eh)), l.eh - 1);
    int ix = min(int(u * float(l.ew)), l.ew - 1);
    iy = max(iy, 0);
    ix = max(ix, 0);
    const float* c = l.cond_cdf + size_t(iy) * (l.ew + 1);
    return (__ldg(l.marg_cdf + iy + 1) - __ldg(l.marg_cdf + iy)) * float(l.eh) * (__ldg(c + ix + 1) - __ldg(c + ix)) * float(l.ew);
}
CG_D float env_pdfW(const LightD& l, float3 dir) {
    const float3 uvw = env_uvw(dir);
    const float s = sinf((1.0f - uvw.y) * kPi);
    if (s <= 0.0f) return 0.0f;
    return env_pdf_uv(l, uvw.x, uvw.y) / (2.0f * kPi * kPi * s);
}

// SingleAreaLight::evaluateDirectSample (singleAreaLight.cpp:54-85) with
// Triangle / Rectangle::evaluatePositionSample (triangle.cpp:162-193,
// sampleWarp.cpp:10-19; rectangle.cpp:134-169 rejection sampler).
// EnvironmentLight::evaluateDirectSample (environmentLight.cpp:67-92) with
// Distribution2D::sampleContinuous (distribution2D.cpp:27-40): the row from
// the .y draw, the column from the .x draw.
CG_D LightS env_sample(const SceneD& S, const LightD& l, float3 target, Rng& rng) {
    LightS out;
    out.radiance = splat3(0.0f);
    out.pdfW = 0.0f;
    out.pos = splat3(0.0f);
    float sx, sy;
    rng.next2(&sx, &sy);
    const int iy = cdf_find(l.marg_cdf, l.eh, sy);
    const float* c = l.cond_cdf + size_t(iy) * (l.ew + 1);
    const int ix = cdf_find(c, l.ew, sx);
    const float m0 = __ldg(l.marg_cdf + iy), m1 = __ldg(l.marg_cdf + iy + 1);
    const float c0 = __ldg(c + ix), c1 = __ldg(c + ix + 1);
    float dy = sy - m0, dx = sx - c0;
    if (m1 > m0) dy /= m1 - m0;
    if (c1 > c0) dx /= c1 - c0;
    const float v = fminf(fmaxf((float(iy) + dy) / float(l.eh), 0.0f), 1.0f);
    const float u = fminf(fmaxf((float(ix) + dx) / float(l.ew), 0.0f), 1.0f);
    const float pdf_uv = (m1 - m0) * float(l.eh) * (c1 - c0) * float(l.ew);
    const float s = sinf((1.0f - v) * kPi);
    if (s <= 0.0f || !(pdf_uv > 0.0f)) return out;
    const float3 dir = env_dir(u, v);
    out.pos = target + dir * 1.0e6f;  // the reference's sky sphere radius (infiniteSphere.cpp:17-20)
    out.pdfW = pdf_uv / (2.0f * kPi * kPi * s);
    out.radiance = texture_rgb(S.textures[l.tex], mk(u, v, 0.0f));
    return out;
}

CG_D LightS light_sample(const SceneD& S, const LightD& l, float3 target, Rng& rng) {
    if (l.kind == 2) return env_sample(S, l, target, rng);
    LightS out;
    out.radiance = splat3(0.0f);
    out.pdfW = 0.0f;
    out.pos = splat3(0.0f);
    float3 P, Ns;
    if (l.kind == 0) {
        float u0, u1;
        rng.next2(&u0, &u1);
        const float sa = sqrtf(u0);
        const float s = 1.0f - sa, t = sa * u1;
        P = l.p0 + l.e0 * s + l.e1 * t;
        if (l.has_normals) {
            const float3 n = l.nA * (1.0f - s - t) + l.nB * s + l.nC * t;
            Ns = is_zero(n) ? l.n : n;
        } else {
            Ns = l.n;
        }
    } else {
        const float ratio = l.short_len / l.long_len;
        float a = 0.0f, b = 2.0f;
        for (int it = 0; it < 4096 && b > ratio; ++it) {
            a = rng.next();
            b = rng.next();
        }
        if (b > ratio) return out;  // bounded rejection loop gave up
        P = l.p0 + l.long_e * a + l.short_dir * (b * l.long_len);
        Ns = l.n;
    }
    const float3 ev = target - P;
    if (!can_emit(l, ev, Ns)) return out;
    const float d2 = len2(ev);
    const float cosE = absdot(ev * (1.0f / sqrtf(d2)), Ns);
    if (cosE <= 0.0f) return out;
    out.pos = P;
    out.pdfW = l.pdf_area * d2 / cosE;
    out.radiance = l.radiance;
    return out;
}

// SingleAreaLight::emittance (singleAreaLight.cpp:39-52)
CG_D float3 light_emittance(const LightD& l, const SurfaceD& si) {
    return can_emit(l, si.wi, si.Ns) ? l.radiance : splat3(0.0f);
}
// SingleAreaLight::evaluateDirectPdfW (singleAreaLight.cpp:87-109)
CG_D float light_pdfW(const LightD& l, const SurfaceD& si, float3 target) {
    if (!can_emit(l, si.wi, si.Ns)) return 0.0f;
    const float c = absdot(si.wi, si.Ns);
    if (c <= 0.0f) return 0.0f;
    return l.pdf_area * len2(target - si.P) / c;
}

// LightCluster::sampleOneLight: uniform (uniformLightCluster.cpp:15-24,
// Random::nextIndex) or by flux (powerLightCluster.cpp:29-36: one draw,
// Distribution1D::sampleDiscrete, distribution1D.cpp:83-94 / 115-125 - the
// largest index whose CDF value is <= the draw, found here by bisection).
CG_D int pick_light(const SceneD& S, Rng& rng, float* pdf) {
    if (!S.light_cdf) {
        *pdf = 1.0f / float(S.num_lights);
        return rng.index(S.num_lights);
    }
    const float u = rng.next();
    int lo = 0, hi = S.num_lights - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(S.light_cdf + mid) <= u) lo = mid; else hi = mid - 1;
    }
    *pdf = __ldg(S.light_cdf + lo + 1) - __ldg(S.light_cdf + lo);
    return lo;
}
// LightCluster::evaluatePickLightPdf of light `li`
CG_D float light_pick_pdf(const SceneD& S, int li) {
    if (!S.light_cdf) return 1.0f / float(S.num_lights);
    return __ldg(S.light_cdf + li + 1) - __ldg(S.light_cdf + li);
}

CG_D float mis_power(float a, float b) {  // TMis<POWER>::weight (tMis.h:21-47)
    const float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}

// ------------------------------------------------------------ vertex plan --
struct VertexPlan {
    float3 emit;          // T * Le, added to L now
    int shadow;           // shadow ray (P, sdir, stmax) unoccluded => Ls += scontrib
    float3 sdir, scontrib;
    float3 sx;            // scontrib without the light's radiance factor (adjoint)
    int slight;
    float stmax;
    int mis;              // MIS ray (P, mdir): hitting light `mlight` => L += mis_resolve(...)
    float3 mdir, mfactor;
    float mpdf;
    int mlight;
    int cont;             // continuation (P, cdir) with throughput T
    float3 cdir, T;
    int count_emission;
};

// One vertex of PtEstimator::estimate (ptEstimator.cpp:43-119) and the
// light-sampling half of DirectLightEvaluator::evaluate
// (directLightEvaluator.cpp:36-76); random numbers in the reference's order:
// light pick, light position, MIS BSDF sample, continuation sample, roulette.
// Q: the shade queue the caller handles (-1: any material) - only that
// queue's BSDFs are compiled in.
template <int Q = -1>
CG_D VertexPlan plan_vertex(const SceneD& S, const SurfaceD& si, float3 T, bool count_emission, int bounce, Rng& rng) {
    VertexPlan p;
    p.emit = splat3(0.0f);
    p.shadow = 0;
    p.mis = 0;
    p.cont = 0;
    p.mlight = -1;
    const MaterialD m = S.materials[si.material];
    if (si.light >= 0 && count_emission) p.emit = T * light_emittance(S.lights[si.light], si);
    if (!bsdf_is_specular(m.type)) {
        p.count_emission = 0;
        float pick;
        const int li = pick_light(S, rng, &pick);
        if (m.type != BSDF_ABSORBER) {
            const LightD& l = S.lights[li];
            const LightS ls = light_sample(S, l, si.P, rng);
            if (ls.valid()) {
                const float3 Lv = ls.pos - si.P;
                const float dist = len(Lv);
                const float3 L = divs(Lv, dist);
                const float3 f = bsdf_eval<Q>(S, m, si, L);
                const float3 factor = f * absdot(L, si.Ns);
                const float bp = bsdf_pdf<Q>(S, m, si, L);
                const float w = mis_power(ls.pdfW, bp);
                const float3 part = divs(divs(ls.radiance * w * factor, ls.pdfW), pick);
                p.shadow = 1;
                p.sdir = normalize(L);
                p.stmax = dist - kRayEps;
                p.scontrib = T * part;
                p.sx = T * divs(divs(factor * w, ls.pdfW), pick);
                p.slight = li;
            }
            const BsdfS bs = bsdf_sample<Q>(S, m, si, rng);
            if (bs.valid()) {
                p.mis = 1;
                p.mdir = normalize(bs.L);
                p.mfactor = bs.f * absdot(bs.L, si.Ns);
                p.mpdf = bs.pdf;
                p.mlight = li;
            }
        }
    } else {
        p.count_emission = 1;
    }
    const BsdfS bs = bsdf_sample<Q>(S, m, si, rng);
    if (!bs.valid()) return p;
    T *= divs(bs.f * absdot(bs.L, si.Ns), bs.pdf);
    if (bounce > 2) {  // RussianRoulette::isSurvivedOnNextRound (russianRoulette.cpp:9-28)
        const float q = fminf(fmaxf(1.0f - max_comp(T), 0.05f), 1.0f);
        const float u = rng.next();
        if (!(u > q)) return p;
        T = T * (1.0f / (1.0f - q));
    }
    if (is_zero(T)) return p;
    p.cont = 1;
    p.cdir = normalize(bs.L);
    p.T = T;
    return p;
}

// The BSDF-sampling half of DirectLightEvaluator::evaluate
// (directLightEvaluator.cpp:79-106), divided by the pick pdf and weighted by
// the throughput at the vertex (ptEstimator.cpp:80-83).
CG_D float3 mis_resolve(const SceneD& S, const SurfaceD& hit, float3 origin, float3 T, float3 factor, float pdf,
                        float3* x_out = nullptr) {
    const LightD& l = S.lights[hit.light];
    const float3 rad = light_emittance(l, hit);
    const float lp = light_pdfW(l, hit, origin);
    const float w = mis_power(pdf, lp);
    const float pick = light_pick_pdf(S, hit.light);
    if (x_out) *x_out = can_emit(l, hit.wi, hit.Ns) ? T * divs(divs(factor * w, pdf), pick) : splat3(0.0f);
    return T * divs(divs(rad * w * factor, pdf), pick);
}

// A ray that leaves the scene sees the environment: the emission counted at
// a background "hit" (scene.cpp:47-62, environmentLight.cpp:59-65).
CG_D float3 env_radiance(const SceneD& S, float3 dir) {
    const LightD& l = S.lights[S.env_light];
    return texture_rgb(S.textures[l.tex], env_uvw(dir));
}
// The BSDF-sampling half of DirectLightEvaluator for a sampled direction
// that escapes while the environment is the picked light.
CG_D float3 mis_resolve_env(const SceneD& S, float3 dir, float3 T, float3 factor, float pdf, float3* x_out = nullptr) {
    const LightD& l = S.lights[S.env_light];
    const float3 rad = env_radiance(S, dir);
    const float w = mis_power(pdf, env_pdfW(l, dir));
    const float pick = light_pick_pdf(S, S.env_light);
    if (x_out) *x_out = T * divs(divs(factor * w, pdf), pick);
    return T * divs(divs(rad * w * factor, pdf), pick);
}

// d ln(D G) / d alpha of the isotropic GGX terms above (D of isotropicGgx.cpp:11-34,
// separable Smith G of :36-69) at microfacet normal cosine NH and the two
// direction cosines: ln D = 2 ln a - 4 ln c - 2 ln(a^2 + tan^2) + const,
// ln G1 = ln 2 - ln(1 + s), s = sqrt(1 + a^2 tan^2(theta_v)).
CG_D float ggx_dlogDG_dalpha(float a, float NH, float cv, float cl) {
    const float c2 = NH * NH;
    const float t2 = (1.0f - c2) / c2;
    float g = 2.0f / a - 4.0f * a / (a * a + t2);
    const float tv = (1.0f - cv * cv) / (cv * cv), tl = (1.0f - cl * cl) / (cl * cl);
    const float sv = sqrtf(1.0f + a * a * tv), sl = sqrtf(1.0f + a * a * tl);
    g -= a * tv / (sv * (1.0f + sv));
    g -= a * tl / (sl * (1.0f + sl));
    return g;
}

// d ln f / d roughness of a GGX BSDF for the pair (V, L) (0 where f does not
// depend on roughness or the roughness floor clamps it), with
// alpha = max(max(r, 1e-3)^2, 1e-3) (tRoughnessMapper.h:18-40).
CG_D float dlogf_droughness(const MaterialD& m, float3 V, float3 L, float3 N) {
    if (m.type != BSDF_CONDUCTOR && m.type != BSDF_DIELECTRIC_GGX) return 0.0f;
    const float r = m.roughness;
    if (!(r > 1e-3f) || !(r * r > 1e-3f)) return 0.0f;
    const float cv = dot(V, N), cl = dot(L, N);
    if (cv == 0.0f || cl == 0.0f) return 0.0f;
    float3 H;
    if (cv * cl > 0.0f) {
        H = V + L;
    } else {
        const float etaV = cv > 0.0f ? m.ior_outer : m.ior_inner;
        const float etaL = cv > 0.0f ? m.ior_inner : m.ior_outer;
        H = V + L * (etaL / etaV);
    }
    if (is_zero(H)) return 0.0f;
    H = normalize(H);
    const float NH = fabsf(dot(N, H));
    const float g = ggx_dlogDG_dalpha(m.alpha, NH, fabsf(cv), fabsf(cl)) * (2.0f * r);
    return isfinite(g) ? g : 0.0f;
}

CG_D int texel_index(const TextureD& t, float3 uvw) {
    const float u = uvw.x - floorf(uvw.x), v = uvw.y - floorf(uvw.y);
    int x = int(u * float(t.width)), y = int(v * float(t.height));
    x = x < t.width ? x : x - 1;
    y = y < t.height ? y : y - 1;
    return y * t.width + x;
}

}  // namespace cg
