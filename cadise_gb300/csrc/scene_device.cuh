// Device-resident scene layout (one per uploaded scene, all in HBM).
//
//  * Bvh4Node, 64 B, half an L2 line: the four child boxes quantized to 8
//    bits per plane in the node's own frame (see quantize_node) + four 32-bit
//    child entries.  A child entry is either an inner node index (bit 31
//    clear) or a leaf: bit 31 set, (count - 1) in bits 28..30, first triangle
//    slot in bits 0..27.  Empty slots hold entry 0 (the root can be no node's
//    child); the traversal tests the entry, not the box.
//  * TriRecord, 48 B per triangle in leaf order: the three vertices in the
//    primitive's own vertex order (so the geometric normal is the reference's
//    eAB x eAC) with the primitive index, the packed material / light id and
//    flags in the .w lanes.  A rectangle is stored as two TriRecords
//    (vB, vA, vC) and (vA, vD, vC), both carrying the rectangle's index.
//  * Material / Light tables and optional per-primitive shading attributes
//    (vertex normals, vertex uvws) read only at a hit.
#pragma once

#include "common.cuh"

namespace cg {

struct __align__(16) Bvh4Node {
    float ox, oy, oz;   // frame origin
    uint32_t exps;      // bytes 0..2: biased exponents e of the x, y, z steps 2^(e - 127)
    uint32_t child[4];
    uint32_t lox, hix, loy, hiy;  // byte i: child i's plane in steps from the origin
    uint32_t loz, hiz, pad0, pad1;
};
static_assert(sizeof(Bvh4Node) == 64, "Bvh4Node is 64 bytes");

// Encodes up to four child boxes (nk of them) conservatively: per axis a step
// 2^e with the union of the boxes inside 254 steps (and no finer than two
// float spacings of its coordinates), the origin at the union's lower plane,
// every lower plane rounded down and every upper plane rounded up to a step.
// The slab test computes (origin - o) / d + q * 2^e / d; its rounding error
// is a few ulps of t, inside the traversal's 1 + 2 gamma(3) slack.  FP64
// arithmetic, so host and device encode alike.
CG_HD void quantize_node(const float (&lo)[4][3], const float (&hi)[4][3], const uint32_t (&child)[4], int nk,
                         Bvh4Node* out) {
    float org[3] = {0.0f, 0.0f, 0.0f};
    uint32_t ebits[3] = {127u, 127u, 127u};
    uint32_t qlo[3] = {0u, 0u, 0u}, qhi[3] = {0u, 0u, 0u};
    for (int a = 0; a < 3 && nk > 0; ++a) {
        double ulo = lo[0][a], uhi = hi[0][a];
        for (int i = 1; i < nk; ++i) {
            ulo = ulo < lo[i][a] ? ulo : double(lo[i][a]);
            uhi = uhi > hi[i][a] ? uhi : double(hi[i][a]);
        }
        const double mag = fabs(ulo) > fabs(uhi) ? fabs(ulo) : fabs(uhi);
        double want = (uhi - ulo) / 254.0;
        if (want < mag * 0x1p-22) want = mag * 0x1p-22;
        if (want < 0x1p-120) want = 0x1p-120;
        int e = 0;
        frexp(want, &e);  // 2^e > want
        for (;; ++e) {
            const double step = ldexp(1.0, e);
            const float o = float(ulo);  // a float already
            uint32_t l4 = 0, h4 = 0;
            bool fits = true;
            for (int i = 0; i < nk; ++i) {
                double ql = floor((double(lo[i][a]) - double(o)) / step);
                double qh = ceil((double(hi[i][a]) - double(o)) / step);
                if (ql < 0.0) ql = 0.0;
                if (qh > 255.0 || qh < ql) fits = false;
                l4 |= uint32_t(ql) << (8 * i);
                h4 |= uint32_t(fits ? qh : 0.0) << (8 * i);
            }
            if (!fits && e < 126) continue;
            org[a] = o;
            ebits[a] = uint32_t(e + 127);
            qlo[a] = l4;
            qhi[a] = h4;
            break;
        }
    }
    out->ox = org[0];
    out->oy = org[1];
    out->oz = org[2];
    out->exps = ebits[0] | (ebits[1] << 8) | (ebits[2] << 16);
    for (int i = 0; i < 4; ++i) out->child[i] = i < nk ? child[i] : 0u;
    out->lox = qlo[0];
    out->hix = qhi[0];
    out->loy = qlo[1];
    out->hiy = qhi[1];
    out->loz = qlo[2];
    out->hiz = qhi[2];
    out->pad0 = out->pad1 = 0u;
}

constexpr uint32_t kLeafBit = 0x80000000u;
CG_HD bool entry_is_leaf(uint32_t e) { return (e & kLeafBit) != 0; }
CG_HD uint32_t leaf_first(uint32_t e) { return e & 0x0FFFFFFFu; }
CG_HD uint32_t leaf_count(uint32_t e) { return ((e >> 28) & 7u) + 1u; }
CG_HD uint32_t make_leaf(uint32_t first, uint32_t count) { return kLeafBit | ((count - 1u) << 28) | first; }
constexpr uint32_t kMaxLeafTris = 8;
constexpr uint32_t kMaxTriSlots = 0x0FFFFFFFu;
// traversal stack entries per ray; a 4-wide tree of depth D needs at most 3 D + 1
constexpr int kStackSize = 96;

struct __align__(16) TriRecord {
    float4 v0;  // xyz = vertex A, w = primitive index (int bits)
    float4 v1;  // xyz = vertex B, w = (material index) | ((light index + 1) << 16)
    float4 v2;  // xyz = vertex C, w = flags (kRec* kind in bits 0-1, rectangle index in bits 2-31)
    // a sphere: v0.xyz = centre, v1.x = radius
};
static_assert(sizeof(TriRecord) == 48, "TriRecord is 48 bytes");

enum : int {
    BSDF_LAMBERTIAN = 0,
    BSDF_CONDUCTOR = 1,
    BSDF_GLASS = 2,
    BSDF_ABSORBER = 3,
    BSDF_DIELECTRIC_GGX = 4,
    BSDF_MIRROR = 5,
    BSDF_PHONG = 6,
    BSDF_PLASTIC = 7
};
constexpr int kNumBsdfTypes = 8;
// Shade queues (one shade kernel each): materials that cost alike share one.
constexpr int kNumBsdfKinds = 5;
constexpr CG_HD int shade_queue(int type) {
    return type == BSDF_MIRROR ? BSDF_GLASS : (type == BSDF_PHONG || type == BSDF_PLASTIC) ? BSDF_LAMBERTIAN : type;
}
// Whether the shading code compiled for shade queue Q (-1: every queue, the
// megakernel and the adjoint) includes BSDF `type`.
template <int Q>
constexpr CG_HD bool queue_has(int type) { return Q < 0 || shade_queue(type) == Q; }

// Record flags (TriRecord::v2.w): bits 0-1 the kind, bits 2-31 the
// rectangle index of a rectangle half.
constexpr uint32_t kRecTriangle = 0u, kRecRectHalf = 1u, kRecSphere = 2u;

struct __align__(16) MaterialD {
    int type;
    int albedo_tex;   // -1 constant
    float roughness;  // raw CRSD roughness
    float alpha;      // max(max(r, 1e-3)^2, 1e-3)
    float3 albedo;
    float ior_outer;
    float3 f0;
    float ior_inner;
    float exponent;   // phong / plastic specular exponent
    float ratio;      // plastic diffuse ratio
    int fresnel;      // mirror: 0 conductor (f0), 1 dielectric (iors)
    int pad;
};

struct __align__(16) LightD {
    int prim;
    int kind;        // 0 triangle, 1 rectangle, 2 environment
    int slot[2];     // its primitive records (leaf order): the triangle, or the two rectangle halves; -1 none
    int back_face;
    float pdf_area;  // 1 / area
    float3 radiance; // color / sum(color) * watt / (area * pi)
    float area;
    // triangle: p0 = vA, e0 = eAB, e1 = eAC, n = Ng, nA..nC vertex normals
    // rectangle: p0 = vB, e0 = eA (vA - vB), e1 = eB (vC - vB), n = normalize(eA x eB)
    float3 p0, e0, e1, n;
    float3 nA, nB, nC;
    int has_normals;
    float long_len, short_len;  // rectangle rejection sampler
    float3 long_e, short_dir;    // rectangle: longer edge, unit shorter edge
    // environment: radiance texture and its piecewise-constant 2-D sampling
    // distribution (luminance x sin(theta) per texel): row CDF (eh + 1) and
    // per-row column CDFs (eh x (ew + 1))
    int tex, ew, eh;
    const float* marg_cdf;
    const float* cond_cdf;
};

struct TextureD {
    int width, height;
    const float* texels;  // RGB float
};

// Camera in the reference's film->camera->world form (perspectivePinholeCamera.cpp:32-73).
struct CameraD {
    float3 pos, ax, ay, az;
    float sx, sy, tx, ty, offset;
};

// Film filter of a scene (cgpu_film_filter resolved at upload).  pixel_only:
// the default box of size 1, whose footprint is the sample's own pixel.
// Gaussian: p0 / p1 = -1 / (2 sigma^2) in x / y, p2 = the value at the corner
// of the footprint, p3 = amplitude.  Mitchell: p0 = b, p1 = c.
struct FilterD {
    int type;
    int pixel_only;
    float hx, hy;  // half the filter's size
    float p0, p1, p2, p3;
    int tile_w, tile_h;
};

struct SceneD {
    const Bvh4Node* nodes;
    const TriRecord* tris;
    const MaterialD* materials;
    const LightD* lights;
    const TextureD* textures;
    const float* prim_normals;  // 9 per primitive or null
    const float* prim_uvws;     // 9 per primitive or null
    const float* rect_frames;   // 9 per rectangle (vB, eA, eB), indexed by the rectangle index
    const uint32_t* prim_rank;  // 8 per primitive: the reference's tie order per direction octant, or null
    const float* light_cdf;     // power light cluster: num_lights + 1 CDF values; null: uniform pick
    int num_lights;  // area lights + environment
    int env_light;   // index of the environment light, -1 if none
    int num_tris;
    int width, height;
    int max_depth;
    int spp;
    CameraD cam;
    FilterD filter;
    float3 bounds_lo, bounds_inv;  // scene bounds: lower corner, 1 / extent (0 for a flat axis)
    // Device-side iteration budget: node and leaf visits one traversal of
    // this scene may make before it stops (over_budget, traverse.cuh), and
    // the context's status word that counts the rays that ran out.
    uint32_t visit_budget;
    uint32_t* status;
    // absolute part of the closest-hit tie window (tie_hi, traverse.cuh):
    // 2^-16 of the largest coordinate magnitude of the scene and camera
    float tie_abs;
};

// SceneD::tie_abs of a scene with bounds [lo, hi] seen from camera position c.
inline float tie_window_abs(const float* lo, const float* hi, const float* c) {
    float m = 0.0f;
    for (int k = 0; k < 3; ++k) {
        m = fmaxf(m, fabsf(lo[k]));
        m = fmaxf(m, fabsf(hi[k]));
        m = fmaxf(m, fabsf(c[k]));
    }
    return ldexpf(m, -16);
}

// The automatic visit budget of a tree of `nodes` 4-wide nodes.  A stack
// traversal reaches every inner node and every leaf at most once (each is
// pushed by its parent, once), and a node holds at most four leaves, so a
// correct traversal makes fewer than 5 x nodes + 1 visits: only a corrupted
// tree, or a budget the caller set lower, runs out.
inline uint32_t auto_visit_budget(uint64_t nodes) {
    const uint64_t b = 5 * nodes + 64;
    return b > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(b);
}

}  // namespace cg
