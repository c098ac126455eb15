// Closest-hit and any-hit traversal of the 4-wide BVH with a watertight
// FP32 ray/triangle test.
//
// Replaces BvhAccelerator::isIntersecting / isOccluded
// (source/core/intersector/accelerator/bvh/bvhAccelerator.cpp:40-156) and
// Triangle::isIntersecting (source/core/intersector/primitive/triangle.cpp:54-123):
// same contract - closest hit with t in [t_min, t_max] (inclusive), or any
// hit in that range - but every ray/triangle decision is watertight
// (Woop, Benthin & Wald, "Watertight Ray/Triangle Intersection", JCGT 2013):
// the three edge functions are evaluated in a ray-aligned sheared space with
// exactly rounded products (no contraction), falling back to FP64 when one of
// them is exactly zero, so no ray slips between adjoining triangles.  Two
// primitives met within a few roundings of each other (a ray through an edge
// two triangles share, coplanar overlapping quads) are ordered by the
// reference's own test and tie order (tie_prefers), so the closest hit is the
// reference's there too.  Box tests widen t_max by 1 + 2 gamma(3) (and by the
// tie window for closest hits) to stay conservative.
#pragma once

#include "scene_device.cuh"

namespace cg {

struct RayPre {
    float3 o, d, inv;
    float tmin, tmax;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

CG_D RayPre ray_prep(float3 o, float3 d, float tmin, float tmax) {
    RayPre r;
    r.o = o;
    r.d = d;
    r.tmin = tmin;
    r.tmax = tmax;
    // zero components would make (lo - o) * inf = NaN on a box face plane
    const float e = 1e-30f;
    const float dx = fabsf(d.x) < e ? copysignf(e, d.x) : d.x;
    const float dy = fabsf(d.y) < e ? copysignf(e, d.y) : d.y;
    const float dz = fabsf(d.z) < e ? copysignf(e, d.z) : d.z;
    r.inv = mk(1.0f / dx, 1.0f / dy, 1.0f / dz);
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > fmaxf(ax, ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) { const int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    const float dkz = comp(d, kz);
    r.Sx = comp(d, kx) / dkz;
    r.Sy = comp(d, ky) / dkz;
    r.Sz = 1.0f / dkz;
    return r;
}

// Watertight test.  On a hit inside [tmin, tcur] writes t and the
// barycentrics of vertices B (u) and C (v).
CG_D bool tri_test(const RayPre& r, float3 A3, float3 B3, float3 C3, float tcur, float* tout, float* uout, float* vout) {
    const float3 A = A3 - r.o, B = B3 - r.o, C = C3 - r.o;
    const float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    const float Ax = comp(A, r.kx) - r.Sx * Akz;
    const float Ay = comp(A, r.ky) - r.Sy * Akz;
    const float Bx = comp(B, r.kx) - r.Sx * Bkz;
    const float By = comp(B, r.ky) - r.Sy * Bkz;
    const float Cx = comp(C, r.kx) - r.Sx * Ckz;
    const float Cy = comp(C, r.ky) - r.Sy * Ckz;
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
        V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
        W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    if (det < 0.0f) { T = -T; det = -det; U = -U; V = -V; W = -W; }
    if (T < r.tmin * det || T > tcur * det) return false;
    const float inv = 1.0f / det;
    *tout = T * inv;
    *uout = V * inv;
    *vout = W * inv;
    return true;
}

struct HitD {
    float t;
    int slot;  // triangle slot in leaf order, -1 on a miss
    float u, v;
};

struct TraceCounters {
    uint32_t nodes;
    uint32_t tris;
};

CG_D float4 ldg4(const float4* p) { return __ldg(p); }

// Loads node `idx`: q[0] the frame origin and step exponents, q[1] the four
// child entries, q[2] / q[3] the quantized planes (lo / hi x, lo / hi y,
// lo / hi z).
CG_D void load_node(const Bvh4Node* nodes, uint32_t idx, const RayPre& r, float4 (&q)[4]) {
    const float4* p = reinterpret_cast<const float4*>(nodes + idx);
    q[0] = __ldg(p + 0);
    q[1] = __ldg(p + 1);
    q[2] = __ldg(p + 2);
    q[3] = __ldg(p + 3);
}

// Closest-hit tie window (tie_prefers): candidates whose distances lie within
// tie_hi of each other are ordered by the reference's rule, so closest-hit
// bounds are widened to tie_hi, and box distances by a further 1 + 2 gamma(3).
// The window is relative (kTieSlack) plus absolute (SceneD::tie_abs, 2^-16 of
// the scene's coordinate scale): the watertight distance of a short ray
// carries the rounding of vertex coordinates of the scene's magnitude, up to
// 3e-6 of the scale on the reference's test scenes.
constexpr float kTieSlack = 1.000004f;
CG_D float tie_hi(const SceneD& S, float t) { return t * kTieSlack + S.tie_abs; }

// Child box distances; tnear = +inf marks a miss.  Empty child slots hold
// entry 0 (the root, never anyone's child) and are always a miss.  Per axis
// the slab distances are a + q * b with a = (origin - o) / d and b = step / d
// (exact: the step is a power of two), the near plane picked by the sign of d.
CG_D void child_hits(const RayPre& r, const float4 (&q)[4], float tcur, float (&tn)[4]) {
    const uint32_t ce[4] = {__float_as_uint(q[1].x), __float_as_uint(q[1].y), __float_as_uint(q[1].z),
                            __float_as_uint(q[1].w)};
    const uint32_t exps = __float_as_uint(q[0].w);
    const float bx = __uint_as_float((exps & 255u) << 23) * r.inv.x;
    const float by = __uint_as_float(((exps >> 8) & 255u) << 23) * r.inv.y;
    const float bz = __uint_as_float(((exps >> 16) & 255u) << 23) * r.inv.z;
    const float ax = (q[0].x - r.o.x) * r.inv.x;
    const float ay = (q[0].y - r.o.y) * r.inv.y;
    const float az = (q[0].z - r.o.z) * r.inv.z;
    // 1 where the ray runs towards -axis: the near plane is the upper one
    const bool sx = (__float_as_uint(r.inv.x) >> 31) != 0u, sy = (__float_as_uint(r.inv.y) >> 31) != 0u,
               sz = (__float_as_uint(r.inv.z) >> 31) != 0u;
    const uint32_t lox = __float_as_uint(q[2].x), hix = __float_as_uint(q[2].y);
    const uint32_t loy = __float_as_uint(q[2].z), hiy = __float_as_uint(q[2].w);
    const uint32_t loz = __float_as_uint(q[3].x), hiz = __float_as_uint(q[3].y);
    const uint32_t nx = sx ? hix : lox, fx = sx ? lox : hix;
    const uint32_t ny = sy ? hiy : loy, fy = sy ? loy : hiy;
    const uint32_t nz = sz ? hiz : loz, fz = sz ? loz : hiz;
    const float tlim = tcur * 1.00000036f;  // 1 + 2 gamma(3)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int sh = 8 * i;
        const float tnx = fmaf(float((nx >> sh) & 255u), bx, ax), tfx = fmaf(float((fx >> sh) & 255u), bx, ax);
        const float tny = fmaf(float((ny >> sh) & 255u), by, ay), tfy = fmaf(float((fy >> sh) & 255u), by, ay);
        const float tnz = fmaf(float((nz >> sh) & 255u), bz, az), tfz = fmaf(float((fz >> sh) & 255u), bz, az);
        const float tnear = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
        const float tfar = fminf(fminf(tfx, tfy), fminf(tfz, tlim));
        tn[i] = (ce[i] != 0u && tnear <= tfar * 1.00000036f) ? tnear : __int_as_float(0x7f800000);
    }
}

constexpr uint32_t kNoEntry = 0xFFFFFFFFu;  // never a node or leaf entry (28-bit triangle range)

// Device-side iteration budget of one ray: `left` starts at its scene's
// SceneD::visit_budget and counts its node and leaf visits down; at the
// visit past the budget the traversal stops, reports the hit it holds so
// far (or none) and counts the ray in S.status.  The host reads that count
// at its next synchronising call and returns CGPU_ERR_TIMEOUT, so a
// corrupted tree ends in an error status instead of a kernel that never
// returns.
CG_D bool over_budget(const SceneD& S, uint32_t& left) {
    if (left != 0) {
        --left;
        return false;
    }
    if (S.status) atomicAdd(S.status, 1u);
    return true;
}

// Traversal stacks: kStackSize entries of (child entry, entry distance),
// enough for any tree the upload accepts (3 x depth + 1 entries).
// LocalStack keeps them in per-thread arrays (local memory on the GPU): the
// megakernel, the per-ray loops and the host build of these headers.
struct LocalStack {
    uint32_t e[kStackSize];
    float t[kStackSize];
    CG_HD void push(int sp, uint32_t ee, float tt) { e[sp] = ee; t[sp] = tt; }
    CG_HD uint32_t entry(int sp) const { return e[sp]; }
    CG_HD float dist(int sp) const { return t[sp]; }
};

#ifdef __CUDACC__
// The persistent traversal passes keep the bottom kSmemStack entries of each
// lane in shared memory and only deeper ones in local memory: on the 1 M-
// triangle field a closest-hit ray's stack reaches 4 entries at the median,
// 10 at the 99th percentile and more than 16 for 2 rays in 100,000.  Each
// warp owns kSmemStack rows of 32 words (64 with distances: the 32 entries,
// then their 32 distances); entry k of lane l sits at word
// row_base + k * row + l, so the lanes of a warp always hit 32 different
// banks whatever depth each one is at, and one register (the lane's base)
// addresses the whole stack.  WITH_T = false (any-hit) keeps no distances:
// an any-hit pass pops without the distance test.
constexpr int kSmemStack = 16;
// the dynamic shared memory of a persistent traversal launch
extern __shared__ uint32_t trav_stack_smem[];

template <bool WITH_T>
struct SharedStack {
    static constexpr int kRow = WITH_T ? 64 : 32;  // words per stack level of a warp
    uint32_t base;   // this lane's word of level 0
    uint32_t oe[kStackSize - kSmemStack];
    float ot[WITH_T ? kStackSize - kSmemStack : 1];

    // Shared memory per block for `threads` threads (a multiple of 32).
    static constexpr size_t bytes(int threads) { return size_t(threads) * kSmemStack * (WITH_T ? 8u : 4u); }
    CG_D void bind() { base = (threadIdx.x >> 5) * uint32_t(kSmemStack * kRow) + (threadIdx.x & 31u); }
    CG_D void push(int sp, uint32_t ee, float tt) {
        if (sp < kSmemStack) {
            trav_stack_smem[base + sp * kRow] = ee;
            if (WITH_T) trav_stack_smem[base + sp * kRow + 32] = __float_as_uint(tt);
        } else {
            oe[sp - kSmemStack] = ee;
            if (WITH_T) ot[sp - kSmemStack] = tt;
        }
    }
    CG_D uint32_t entry(int sp) const {
        return sp < kSmemStack ? trav_stack_smem[base + sp * kRow] : oe[sp - kSmemStack];
    }
    CG_D float dist(int sp) const {
        if (!WITH_T) return 0.0f;
        return sp < kSmemStack ? __uint_as_float(trav_stack_smem[base + sp * kRow + 32]) : ot[sp - kSmemStack];
    }
};
#endif

// Visits inner node `e`: pushes the children the ray enters, farthest first,
// except the nearest, which it returns (kNoEntry when the ray misses all four).
// WIDE = false (the persistent closest-hit pass, which leaves ties to
// k_wf_ties): children culled by tcur itself, not by the tie window.
template <bool ANY, bool COUNT, bool WIDE = true, typename Stack>
CG_D uint32_t visit_node(const SceneD& S, const RayPre& r, uint32_t e, float tcur, Stack& stack, int& sp,
                         TraceCounters* cnt) {
    const float kInf = __int_as_float(0x7f800000);
    float4 q[4];
    load_node(S.nodes, e, r, q);
    if (COUNT) cnt->nodes++;
    float tn[4];
    child_hits(r, q, (ANY || !WIDE) ? tcur : tie_hi(S, tcur), tn);
    uint32_t ce[4] = {__float_as_uint(q[1].x), __float_as_uint(q[1].y), __float_as_uint(q[1].z),
                      __float_as_uint(q[1].w)};
    if (!ANY) {
        // ascending by distance (misses sort last)
#define CG_CSWAP(i, j)                                                      \
    if (tn[j] < tn[i]) {                                                    \
        const float tt = tn[i]; tn[i] = tn[j]; tn[j] = tt;                  \
        const uint32_t ee = ce[i]; ce[i] = ce[j]; ce[j] = ee;               \
    }
        CG_CSWAP(0, 1) CG_CSWAP(2, 3) CG_CSWAP(0, 2) CG_CSWAP(1, 3) CG_CSWAP(1, 2)
#undef CG_CSWAP
    }
    uint32_t nearest = kNoEntry;
    float nearest_t = kInf;
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        if (tn[i] < kInf) {
            if (nearest != kNoEntry && sp < kStackSize) {
                stack.push(sp, nearest, nearest_t);
                ++sp;
            }
            nearest = ce[i];
            nearest_t = tn[i];
        }
    }
    return nearest;
}

// Sphere::isIntersecting / isOccluded (sphere.cpp:43-104): the root pair of
// Haines et al., "Precision Improvements for Ray/Sphere Intersection" (Ray
// Tracing Gems 2019) - t0 = c / q, t1 = q - and _isSolutionValid's choice
// (sphere.cpp:150-170), in the reference's FP32 order; the traversal's t is
// the reference's t.
CG_D bool sphere_test(const RayPre& r, float3 G, float rad, float tmax, float* tout) {
    const float3 f = r.o - G;
    const float b = -dot(f, r.d);
    const float3 l = f + r.d * b;
    const float disc = rad * rad - absdot(l, l);
    if (disc < 0.0f) return false;
    const float signB = b > 0.0f ? 1.0f : -1.0f;
    const float q = b + signB * sqrtf(disc);
    const float c = absdot(f, f) - rad * rad;
    const float t0 = c / q, t1 = q;
    if (t0 > tmax || t1 < r.tmin) return false;
    float t = t0;
    if (t < r.tmin) {
        t = t1;
        if (t > tmax) return false;
    }
    *tout = t;
    return true;
}

// ---- exact ties --------------------------------------------------------
// Two candidates of a closest-hit query whose traversal (watertight)
// distances lie within the tie window (tie_hi, defined with the box test) of
// each other are ordered by the reference's own rule instead: its hit test of
// each primitive (ref_hit), the smaller of its distances, and on an exact tie
// the primitive its BVH traversal reaches last - the higher rank of the ray's
// direction octant (tie_order.h).  The traversal widens its closest-hit
// bounds by the same window, so every candidate inside it reaches the
// comparison.  Outside the window the watertight distances decide.

// Octant of a ray direction: bit k set when component k is negative (-0
// included), the reference's directionIsNegative (bvhAccelerator.cpp:44-48).
CG_D int ray_octant(const RayPre& r) {
    return int(__float_as_uint(r.d.x) >> 31) | int(__float_as_uint(r.d.y) >> 31) << 1 |
           int(__float_as_uint(r.d.z) >> 31) << 2;
}

// The reference's hit test of the primitive of record `slot` on the ray's
// [tmin, tmax], in its FP32 order: Triangle::isIntersecting (Moller-Trumbore,
// triangle.cpp:54-89), Rectangle::isIntersecting (plane distance and edge
// coordinates, rectangle.cpp:49-75), Sphere::isIntersecting (sphere_test is
// already the reference's).  Its distance in *tout.
CG_D bool ref_hit(const SceneD& S, const RayPre& r, int slot, float* tout) {
    const float4* tp = reinterpret_cast<const float4*>(S.tris + slot);
    const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
    const uint32_t flags = __float_as_uint(c.w);
    if ((flags & 3u) == kRecSphere) return sphere_test(r, f3(a), b.x, r.tmax, tout);
    if ((flags & 3u) == kRecRectHalf) {
        const float* fr = S.rect_frames + 9 * size_t(flags >> 2);
        const float3 vB = mk(fr[0], fr[1], fr[2]), eA0 = mk(fr[3], fr[4], fr[5]), eB0 = mk(fr[6], fr[7], fr[8]);
        float3 eA = eA0, eB = eB0;
        if (dot(r.d, cross(eA, eB)) > 0.0f) {
            eA = eB0;
            eB = eA0;
        }
        const float3 n = normalize(cross(eA, eB));
        const float t = dot(n, vB - r.o) / dot(n, r.d);
        if (t < r.tmin || t > r.tmax) return false;
        const float3 onp = (r.o + r.d * t) - vB;
        const float p1 = dot(onp, normalize(eA0)), p2 = dot(onp, normalize(eB0));
        if (p1 < 0.0f || p1 > len(eA0) || p2 < 0.0f || p2 > len(eB0)) return false;
        *tout = t;
        return true;
    }
    const float3 A = f3(a);
    float3 eAB = f3(b) - A, eAC = f3(c) - A;
    if (dot(r.d, cross(eAB, eAC)) > 0.0f) {
        const float3 e = eAB;
        eAB = eAC;
        eAC = e;
    }
    const float3 T = r.o - A;
    const float3 Q = cross(T, eAB), P = cross(r.d, eAC);
    const float den = dot(P, eAB);
    if (den == 0.0f) return false;
    const float inv = 1.0f / den;
    const float t = dot(Q, eAC) * inv, u = dot(P, T) * inv, v = dot(Q, r.d) * inv;
    if (u < 0.0f || v < 0.0f || u + v > 1.0f) return false;
    if (t < r.tmin || t > r.tmax) return false;
    *tout = t;
    return true;
}

// Whether the candidate (slot, prim, watertight t) comes before the kept hit
// (kslot, kprim, kt) of another primitive, the two within the tie window: a
// primitive the reference's test accepts comes before one it rejects; of two
// it accepts the smaller reference distance, and on equal distances the one
// the reference's traversal reaches last (no ranks uploaded: the lower
// primitive index).  Where the reference accepts neither, the watertight
// distance, then the lower primitive index.
CG_D bool tie_prefers(const SceneD& S, const RayPre& r, int slot, int prim, float t, int kslot, int kprim, float kt) {
    float rt = 0.0f, rk = 0.0f;
    const bool a = ref_hit(S, r, slot, &rt), ak = ref_hit(S, r, kslot, &rk);
    if (a != ak) return a;
    if (!a) return t < kt || (t == kt && prim < kprim);
    if (rt != rk) return rt < rk;
    if (!S.prim_rank) return prim < kprim;
    const int o = ray_octant(r);
    return S.prim_rank[8 * size_t(prim) + size_t(o)] > S.prim_rank[8 * size_t(kprim) + size_t(o)];
}

// Which of two hits a closest-hit query keeps: the smaller distance, within
// the tie window tie_prefers.  The two halves of a rectangle share a
// primitive; between them (a ray through the diagonal) the smaller t, then
// the lower record slot, the rule mis_light_hit applies to a light's halves
// too.  Either half gives the same hit point (hit_point recomputes t and the
// edge coordinates from the rectangle's own frame).  `prim` / `slot` are the
// candidate's; the kept hit's primitive is loaded only inside the window.
CG_D bool closer_hit(const SceneD& S, const RayPre& r, float t, int prim, int slot, float tcur, int hslot) {
    if (hslot < 0) return t <= tcur;
    if (tie_hi(S, t) < tcur) return true;
    if (t > tie_hi(S, tcur)) return false;
    const int kept = __float_as_int(ldg4(reinterpret_cast<const float4*>(S.tris + hslot)).w);
    if (prim == kept) return t < tcur || (t == tcur && slot < hslot);
    return tie_prefers(S, r, slot, prim, t, hslot, kept, tcur);
}

// Tests the primitives of leaf `e`; returns true when an any-hit query is
// answered (the hit is in slot / tcur).
// SPH = false: the scene holds no spheres, and the sphere test is compiled out
// of the hot kernels (a sphere record would then be misread as a triangle, so
// the host picks SPH from the scenes it renders).
// DEFER (the persistent closest-hit pass): the watertight rule alone, and hu
// set to 1 when a candidate lies within the tie window of the kept hit - the
// ray is then traced again by k_wf_ties with tie_prefers - so that the rare
// tie code stays out of that register-capped kernel.  hu / hv are not the
// hit's coordinates there.
template <bool ANY, bool COUNT, bool SPH = true, bool DEFER = false>
CG_D bool visit_leaf(const SceneD& S, const RayPre& r, uint32_t e, float& tcur, int& hslot, float& hu, float& hv,
                     TraceCounters* cnt) {
    const uint32_t first = leaf_first(e), n = leaf_count(e);
    for (uint32_t k = 0; k < n; ++k) {
        const float4* tp = reinterpret_cast<const float4*>(S.tris + first + k);
        const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
        if (COUNT) cnt->tris++;
        float t, u = 0.0f, v = 0.0f;
        // closest hit: a bound as wide as the tie window, so that every
        // primitive within it reaches closer_hit
        const bool sphere = SPH && (__float_as_uint(c.w) & 3u) == kRecSphere;
        const float bound = ANY ? tcur : tie_hi(S, tcur);
        if (sphere ? sphere_test(r, f3(a), b.x, bound, &t) : tri_test(r, f3(a), f3(b), f3(c), bound, &t, &u, &v)) {
            const int slot = int(first + k);
            if (ANY) {
                hslot = slot;
                tcur = t;
                return true;
            }
            if (DEFER) {
                if (hslot >= 0 && tie_hi(S, t) >= tcur) hu = 1.0f;
                if (hslot < 0 ? t <= tcur : (t < tcur || (t == tcur && slot < hslot))) {
                    hslot = slot;
                    tcur = t;
                }
            } else if (closer_hit(S, r, t, __float_as_int(a.w), slot, tcur, hslot)) {
                hslot = slot;
                tcur = t;
                hu = u;
                hv = v;
            }
        }
    }
    return false;
}

// One ray per thread, one node or one leaf per loop iteration: the
// megakernel's traversal (its threads are at different bounces anyway) and
// every any-hit query (the first hit ends the walk, so there is nothing to
// gain from holding leaves back).
template <bool ANY, bool COUNT, bool SPH = true>
CG_D bool traverse(const SceneD& S, const RayPre& r, HitD* hit, TraceCounters* cnt) {
    LocalStack stack;
    int sp = 0;
    float tcur = r.tmax;
    int hslot = -1;
    float hu = 0.0f, hv = 0.0f;
    uint32_t cur = 0;  // root first (always an inner node)
    uint32_t left = S.visit_budget;
    for (;;) {
        if (over_budget(S, left)) break;
        uint32_t next = kNoEntry;
        if (entry_is_leaf(cur)) {
            if (visit_leaf<ANY, COUNT, SPH>(S, r, cur, tcur, hslot, hu, hv, cnt)) {
                hit->slot = hslot;
                hit->t = tcur;
                return true;
            }
        } else {
            next = visit_node<ANY, COUNT>(S, r, cur, tcur, stack, sp, cnt);
        }
        // else the next stack entry that can still hold a closer hit
        while (next == kNoEntry && sp > 0) {
            --sp;
            if (ANY || stack.dist(sp) <= tie_hi(S, tcur) * 1.00000036f) next = stack.entry(sp);
        }
        if (next == kNoEntry) break;
        cur = next;
    }
    hit->slot = hslot;
    hit->t = tcur;
    hit->u = hu;
    hit->v = hv;
    return hslot >= 0;
}

// Whether a primitive other than `prim_l` comes before the hit (t_l, prim_l,
// record slot_l) in closest-hit order (closer_hit: a smaller t, within the
// tie window tie_prefers), so that the closest hit of the ray is not prim_l.
// Each primitive is tested as visit_leaf<false> tests it while its bound is
// t_l, with the same window; the nodes are culled by t_l with the
// closest-hit slack.  slot_l < 0, t_l = the ray's tmax: whether the ray hits
// anything at all (the environment is its light).
template <bool COUNT, bool SPH = true>
CG_D bool visit_leaf_before(const SceneD& S, const RayPre& r, uint32_t e, float t_l, int prim_l, int slot_l,
                            TraceCounters* cnt) {
    const uint32_t first = leaf_first(e), n = leaf_count(e);
    const float bound = tie_hi(S, t_l);
    for (uint32_t k = 0; k < n; ++k) {
        const float4* tp = reinterpret_cast<const float4*>(S.tris + first + k);
        const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
        if (COUNT) cnt->tris++;
        float t, u, v;
        const bool sphere = SPH && (__float_as_uint(c.w) & 3u) == kRecSphere;
        if (sphere ? sphere_test(r, f3(a), b.x, bound, &t) : tri_test(r, f3(a), f3(b), f3(c), bound, &t, &u, &v)) {
            const int prim = __float_as_int(a.w);
            if (prim == prim_l) continue;
            if (slot_l < 0) {
                if (t <= t_l) return true;
                continue;
            }
            if (tie_hi(S, t) < t_l) return true;
            if (tie_prefers(S, r, int(first + k), prim, t, slot_l, prim_l, t_l)) return true;
        }
    }
    return false;
}

template <bool COUNT, bool SPH = true>
CG_D bool occluded_before(const SceneD& S, const RayPre& r, float t_l, int prim_l, int slot_l, TraceCounters* cnt) {
    LocalStack stack;
    int sp = 0;
    uint32_t cur = 0;
    uint32_t left = S.visit_budget;
    const float tb = tie_hi(S, t_l);
    for (;;) {
        if (over_budget(S, left)) return false;
        uint32_t next = kNoEntry;
        if (entry_is_leaf(cur)) {
            if (visit_leaf_before<COUNT, SPH>(S, r, cur, t_l, prim_l, slot_l, cnt)) return true;
        } else {
            next = visit_node<true, COUNT>(S, r, cur, tb, stack, sp, cnt);
        }
        if (next == kNoEntry && sp > 0) next = stack.entry(--sp);
        if (next == kNoEntry) return false;
        cur = next;
    }
}

// Closest hit for a warp of independent rays (the wavefront's extend pass and
// the ray queries): while-while traversal with postponed leaves (Aila &
// Laine, "Understanding the efficiency of ray traversal on GPUs", HPG 2009).
// A lane that reaches a leaf keeps it and walks on through inner nodes until
// every active lane of the warp holds a leaf; then the warp tests its leaves
// together, so inner-node and triangle work run with more lanes in step.
// Finds the same hit as traverse<false> (closer_hit does not depend on the
// visiting order).
template <bool COUNT, bool SPH = true>
CG_D bool traverse_warp(const SceneD& S, const RayPre& r, HitD* hit, TraceCounters* cnt) {
    LocalStack stack;
    int sp = 0;
    float tcur = r.tmax;
    int hslot = -1;
    float hu = 0.0f, hv = 0.0f;
    uint32_t cur = 0;          // root first (always an inner node)
    uint32_t leaf = kNoEntry;  // postponed leaf
    uint32_t left = S.visit_budget;
    // next stack entry that can still hold a closer hit
    auto pop = [&]() -> uint32_t {
        while (sp > 0) {
            --sp;
            if (stack.dist(sp) <= tie_hi(S, tcur) * 1.00000036f) return stack.entry(sp);
        }
        return kNoEntry;
    };
    while (cur != kNoEntry || leaf != kNoEntry) {
        while (cur != kNoEntry && !entry_is_leaf(cur)) {
            if (over_budget(S, left)) {
                cur = leaf = kNoEntry;
                break;
            }
            cur = visit_node<false, COUNT>(S, r, cur, tcur, stack, sp, cnt);
            if (cur == kNoEntry) cur = pop();
            if (leaf == kNoEntry && cur != kNoEntry && entry_is_leaf(cur)) {
                leaf = cur;
                cur = pop();
            }
            if (!__any_sync(__activemask(), leaf == kNoEntry)) break;
        }
        if (leaf == kNoEntry) {
            if (cur == kNoEntry) break;
            leaf = cur;  // the walk stopped on a leaf
            cur = pop();
        }
        while (leaf != kNoEntry) {
            if (over_budget(S, left)) {
                cur = leaf = kNoEntry;
                break;
            }
            visit_leaf<false, COUNT, SPH>(S, r, leaf, tcur, hslot, hu, hv, cnt);
            leaf = kNoEntry;
            if (cur != kNoEntry && entry_is_leaf(cur)) {
                leaf = cur;
                cur = pop();
            }
        }
    }
    hit->slot = hslot;
    hit->t = tcur;
    hit->u = hu;
    hit->v = hv;
    return hslot >= 0;
}

// Resumable form of the same traversal for persistent kernels that replace
// finished rays (a warp keeps all lanes busy by giving a lane whose ray is
// done the next ray from a global counter; Aila & Laine, "Understanding the
// efficiency of ray traversal on GPUs", HPG 2009).  trav_step performs one
// node visit or one leaf test and finds the same hit as traverse() (the
// closest-hit rule does not depend on the visiting order).
struct TravState {
    LocalStack stack;
    int sp;
    uint32_t cur;
    float tcur;
    int hslot;
    float hu, hv;
    bool done;
    uint32_t left;  // node and leaf visits left (over_budget)
};

CG_D void trav_begin(TravState& st, const RayPre& r, uint32_t budget) {
    st.left = budget;
    st.sp = 0;
    st.cur = 0;
    st.tcur = r.tmax;
    st.hslot = -1;
    st.hu = st.hv = 0.0f;
    st.done = false;
}

template <bool ANY, bool COUNT, bool SPH = true>
CG_D void trav_step(const SceneD& S, const RayPre& r, TravState& st, TraceCounters* cnt) {
    if (over_budget(S, st.left)) {
        st.done = true;
        return;
    }
    if (entry_is_leaf(st.cur)) {
        if (visit_leaf<ANY, COUNT, SPH>(S, r, st.cur, st.tcur, st.hslot, st.hu, st.hv, cnt)) {
            st.done = true;
            return;
        }
    } else {
        const uint32_t next = visit_node<ANY, COUNT>(S, r, st.cur, st.tcur, st.stack, st.sp, cnt);
        if (next != kNoEntry) {
            st.cur = next;
            return;
        }
    }
    while (st.sp > 0) {
        --st.sp;
        if (ANY || st.stack.dist(st.sp) <= tie_hi(S, st.tcur) * 1.00000036f) {
            st.cur = st.stack.entry(st.sp);
            return;
        }
    }
    st.done = true;
}

}  // namespace cg
