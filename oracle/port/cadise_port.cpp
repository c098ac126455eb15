// CPU restatement of the reference's unidirectional path tracer.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle: only tests/, the smoke check
// and bench.py's CPU-baseline leg load it, and only as the checker / the timed
// CPU baseline.  The product library never links it.
//
// It restates, function by function and in the reference's floating-point
// evaluation order, the path the reference takes for one path sample, so
// that with the same per-path random stream (oracle_rng.h) it reproduces the
// reference harness's radiance bit-for-bit on x86 (pinned by
// tests/test_oracle_pin.py against tests/golden/).  Citations are to the
// reference project's files.
//
// Scene input is the C-ABI scene description (include/cadise_gpu.h), so the
// CUDA library and this oracle consume the very same arrays.

#include "../../include/cadise_gpu.h"
#include "../oracle_rng.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

namespace port {

// ---------------------------------------------------------------- math ----
// source/math/tVector.ipp: dot/lengthSquared accumulate left to right,
// normalize multiplies by 1/length, scalar division multiplies by 1/s.
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit V3(float s) : x(s), y(s), z(s) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator*(float s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(float s) const { const float inv = 1.0f / s; return V3(x * inv, y * inv, z * inv); }
    V3 operator+(float s) const { return V3(x + s, y + s, z + s); }
    V3 operator-(float s) const { return V3(x - s, y - s, z - s); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator*=(const V3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    V3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    float dot(const V3& o) const { float r = 0; r += x * o.x; r += y * o.y; r += z * o.z; return r; }
    float absDot(const V3& o) const { return std::abs(dot(o)); }
    float lengthSquared() const { float r = 0; r += x * x; r += y * y; r += z * z; return r; }
    float length() const { return std::sqrt(lengthSquared()); }
    V3 normalize() const { const float inv = 1.0f / length(); return *this * inv; }
    V3 cross(const V3& v) const { return V3(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x); }
    bool isZero() const { return x == 0.0f && y == 0.0f && z == 0.0f; }
    float sum() const { float r = 0; r += x; r += y; r += z; return r; }
    float average() const { return sum() / 3.0f; }
    float maxComponent() const { float m = x; if (y > m) m = y; if (z > m) m = z; return m; }
    V3 complement() const { return V3(1.0f) - *this; }
    V3 reciprocal() const { return V3(1.0f / x, 1.0f / y, 1.0f / z); }
    // tVector.ipp:462-465
    V3 reflect(const V3& n) const { const V3 r = n * (2.0f * absDot(n)); return r - *this; }
    bool finite() const { return std::isfinite(x) && std::isfinite(y) && std::isfinite(z); }
};
inline V3 operator*(float s, const V3& v) { return v * s; }

constexpr float kPi = 3.1415926535897932f;
constexpr float kTwoPi = 6.2831853071795864f;
constexpr float kInvPi = 0.3183098861837906f;
constexpr float kRayEps = 0.001f;  // constant::ray_epsilon (math/constant.h:9-11)

// math.cpp:36-58
void buildCoordinateSystem(const V3& y, V3* z, V3* x) {
    if (std::abs(y.x) > std::abs(y.y)) {
        V3 zz(-y.z, 0.0f, y.x);
        const float inv = 1.0f / std::sqrt(y.x * y.x + y.z * y.z);
        zz *= inv;
        *z = zz;
    } else {
        V3 zz(0.0f, y.z, -y.y);
        const float inv = 1.0f / std::sqrt(y.y * y.y + y.z * y.z);
        zz *= inv;
        *z = zz;
    }
    *x = y.cross(*z);
}

struct Rng {
    oracle_rng::Stream s;
    float next() { return s.next(); }
    // The reference builds 2-D samples as Vector2R(Random::nextReal(),
    // Random::nextReal()) (lambertianDiffuse.cpp:62, conductorMicrofacet.cpp:88,
    // triangle.cpp:165).  C++ leaves the order of argument evaluation
    // unspecified; GCC evaluates right to left, so the first draw becomes .y
    // and the second .x.  Kept so paths replay exactly.
    void next2(float* x, float* y) { *y = next(); *x = next(); }
    // random.cpp:21-26
    std::size_t index(std::size_t lo, std::size_t hi) {
        const std::size_t interval = hi - lo;
        const std::size_t idx = static_cast<std::size_t>(lo + next() * interval);
        return std::min(std::max(idx, lo), hi - 1);
    }
};

// ---------------------------------------------------------------- scene ---
struct Ray {
    V3 o, d;
    float minT = kRayEps, maxT = std::numeric_limits<float>::max();
};

struct Triangle {  // triangle.cpp:14-42
    V3 a, b, c, eAB, eAC, nA, nB, nC, uA, uB, uC;
};
struct Rectangle {  // rectangle.cpp:14-35
    V3 vA, vB, vC, vD, eA, eB;
};
struct Texture {
    int w = 0, h = 0;
    std::vector<float> texels;
};
struct Material {
    int type;
    V3 albedo, f0;
    float roughness, iorOuter, iorInner;
    int tex;
    float exponent = 32.0f, ratio = 0.7f;  // phong / plastic
    int fresnel = CGPU_FRESNEL_CONDUCTOR;  // mirror
};
struct Sphere {  // sphere.cpp:18-31
    V3 c;
    float r;
};
struct Light {
    int prim;
    V3 radiance;
    bool backFace;
};
struct Prim {
    int kind, material, light, slot;  // slot: index into tris or rects
};

struct Scene {
    std::vector<Prim> prims;
    std::vector<Triangle> tris;
    std::vector<Rectangle> rects;
    std::vector<Sphere> spheres;
    std::vector<Material> mats;
    std::vector<Texture> textures;
    std::vector<Light> lights;
    // reference BVH (bvhBuilder.cpp / bvhLinearNode.h): binary, 1-primitive leaves
    struct Node { V3 lo, hi; int second; int prim; int count; int axis; };
    std::vector<Node> nodes;
    std::vector<int> order;
    // camera (perspectivePinholeCamera.cpp:32-50)
    int W = 0, H = 0, maxDepth = 0, spp = 1;
    // environment light (no reference parity: see env* below)
    int envLight = -1, envTex = -1;
    std::vector<float> envMarg, envCond;
    // power light cluster: Distribution1D CDF over the lights' approximate
    // fluxes (powerLightCluster.cpp:9-27); empty for the uniform cluster
    std::vector<float> lightCdf;
    V3 camPos, camX, camY, camZ;
    float sx = 0, sy = 0, tx = 0, ty = 0, offset = 0;
};

// ------------------------------------------------------------ primitives --
V3 triNormal(const Triangle& t) {
    V3 n = t.eAB.cross(t.eAC);
    return n.isZero() ? V3(0.0f, 1.0f, 0.0f) : n.normalize();
}
V3 rectNormal(const Rectangle& r) {
    V3 n = r.eA.cross(r.eB);
    return n.isZero() ? V3(0.0f, 1.0f, 0.0f) : n.normalize();
}
float triArea(const Triangle& t) { return 0.5f * t.eAB.cross(t.eAC).length(); }  // triangle.cpp:199-201
float rectArea(const Rectangle& r) { return r.eA.length() * r.eB.length(); }      // rectangle.cpp:175-177

// triangle.cpp:54-89 (and :91-123 for the occlusion variant)
bool triHit(const Triangle& tr, const Ray& ray, float* tOut) {
    V3 eAB = tr.eAB, eAC = tr.eAC;
    const V3& D = ray.d;
    if (D.dot(eAB.cross(eAC)) > 0.0f) std::swap(eAB, eAC);
    const V3 T = ray.o - tr.a;
    const V3 Q = T.cross(eAB);
    const V3 P = D.cross(eAC);
    const float den = P.dot(eAB);
    if (den == 0.0f) return false;
    const float inv = 1.0f / den;
    const float t = Q.dot(eAC) * inv;
    const float u = P.dot(T) * inv;
    const float v = Q.dot(D) * inv;
    if (u < 0.0f || v < 0.0f || u + v > 1.0f) return false;
    if (t < ray.minT || t > ray.maxT) return false;
    *tOut = t;
    return true;
}

// rectangle.cpp:49-75
bool rectHit(const Rectangle& r, const Ray& ray, float* tOut) {
    V3 eA = r.eA, eB = r.eB;
    if (ray.d.dot(eA.cross(eB)) > 0.0f) std::swap(eA, eB);
    const V3 n = eA.cross(eB).normalize();
    const float t = n.dot(r.vB - ray.o) / n.dot(ray.d);
    if (t < ray.minT || t > ray.maxT) return false;
    const V3 onPlane = (ray.o + ray.d * t) - r.vB;
    const float p1 = onPlane.dot(r.eA.normalize());
    const float p2 = onPlane.dot(r.eB.normalize());
    if (p1 < 0.0f || p1 > r.eA.length() || p2 < 0.0f || p2 > r.eB.length()) return false;
    *tOut = t;
    return true;
}

// sphere.cpp:43-78 (Haines et al., Ray Tracing Gems 2019) and _isSolutionValid :150-170
bool sphereHit(const Sphere& sp, const Ray& ray, float* tOut) {
    const V3& O = ray.o;
    const V3 G = sp.c;
    const V3 f = O - G;
    const V3& d = ray.d;
    const float b = -f.dot(d);
    const float r = sp.r;
    const V3 l = f + b * d;
    const float discriminant = r * r - l.absDot(l);
    if (discriminant < 0.0f) return false;
    const float signB = (b > 0.0f) ? 1.0f : -1.0f;
    const float q = b + signB * std::sqrt(discriminant);
    const float c = f.absDot(f) - r * r;
    const float t0 = c / q;
    const float t1 = q;
    if (t0 > ray.maxT || t1 < ray.minT) return false;
    float t = t0;
    if (t < ray.minT) {
        t = t1;
        if (t > ray.maxT) return false;
    }
    *tOut = t;
    return true;
}

bool primHit(const Scene& s, int p, const Ray& ray, float* t) {
    const Prim& pr = s.prims[p];
    if (pr.kind == CGPU_PRIM_SPHERE) return sphereHit(s.spheres[pr.slot], ray, t);
    return pr.kind == CGPU_PRIM_TRIANGLE ? triHit(s.tris[pr.slot], ray, t) : rectHit(s.rects[pr.slot], ray, t);
}

void primBound(const Scene& s, int p, V3* lo, V3* hi) {
    const Prim& pr = s.prims[p];
    V3 vs[4];
    int n = 3;
    if (pr.kind == CGPU_PRIM_SPHERE) {  // sphere.cpp:33-40: (c - r, c + r) expanded by 0.0001
        const Sphere& sp = s.spheres[pr.slot];
        *lo = sp.c - sp.r - 0.0001f;
        *hi = sp.c + sp.r + 0.0001f;
        return;
    }
    if (pr.kind == CGPU_PRIM_TRIANGLE) {
        const Triangle& t = s.tris[pr.slot];
        vs[0] = t.a; vs[1] = t.b; vs[2] = t.c;
    } else {
        const Rectangle& r = s.rects[pr.slot];
        vs[0] = r.vA; vs[1] = r.vB; vs[2] = r.vC; vs[3] = r.vD; n = 4;
    }
    *lo = vs[0]; *hi = vs[0];
    for (int i = 1; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            (*lo)[k] = std::min((*lo)[k], vs[i][k]);
            (*hi)[k] = std::max((*hi)[k], vs[i][k]);
        }
    *lo = *lo - 0.0001f;  // expand(0.0001) triangle.cpp:45-52, rectangle.cpp:37-44
    *hi = *hi + 0.0001f;
}

// ------------------------------------------------------------------ BVH ---
// bvhBuilder.cpp:59-169 + :251-358: SAH over 12 buckets along the largest
// centroid extent (traversal 0.125, intersection 1), equal split for <= 2
// primitives, leaf of 1 primitive, depth-first layout with the first child
// adjacent.
struct BuildItem { V3 lo, hi, c; int idx; };

void boxUnion(V3& lo, V3& hi, const V3& l2, const V3& h2) {
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], l2[k]); hi[k] = std::max(hi[k], h2[k]); }
}
float halfArea(const V3& lo, const V3& hi) {
    const V3 e = hi - lo;
    return e.x * e.y + e.y * e.z + e.z * e.x;
}

int buildRec(Scene& s, std::vector<BuildItem>& items, int begin, int end) {
    const int nodeIndex = static_cast<int>(s.nodes.size());
    s.nodes.push_back({});
    // An empty TAABB starts at (FLT_MAX, FLT_MIN) with FLT_MIN the smallest
    // positive float (tAabb.ipp:13-17), so every bound the reference unions
    // up reaches at least 0 on its upper side; kept for the same tree.
    V3 lo(std::numeric_limits<float>::max()), hi(std::numeric_limits<float>::min());
    V3 clo = lo, chi = hi;
    for (int i = begin; i < end; ++i) {
        boxUnion(lo, hi, items[i].lo, items[i].hi);
        boxUnion(clo, chi, items[i].c, items[i].c);
    }
    auto makeLeaf = [&]() {
        Scene::Node& n = s.nodes[nodeIndex];
        n.lo = lo; n.hi = hi; n.second = -1; n.prim = static_cast<int>(s.order.size()); n.count = end - begin; n.axis = 0;
        for (int i = begin; i < end; ++i) s.order.push_back(items[i].idx);
        return nodeIndex;
    };
    const int count = end - begin;
    if (count <= 1) return makeLeaf();
    const V3 ext = chi - clo;
    int axis = 0;
    if (ext.y > ext[axis]) axis = 1;
    if (ext.z > ext[axis]) axis = 2;
    if (clo[axis] == chi[axis]) return makeLeaf();
    int mid;
    if (count <= 2) {  // bvhBuilder.cpp:212-249
        mid = begin + (count + 1) / 2;
        std::nth_element(items.begin() + begin, items.begin() + mid, items.begin() + end,
                         [axis](const BuildItem& a, const BuildItem& b) { return a.c[axis] < b.c[axis]; });
    } else {
        constexpr int NB = 12;
        const float invExt = 1.0f / ext[axis];
        int bc[NB] = {0};
        V3 blo[NB], bhi[NB];
        for (int b = 0; b < NB; ++b) { blo[b] = V3(std::numeric_limits<float>::max()); bhi[b] = V3(std::numeric_limits<float>::min()); }
        auto bucketOf = [&](const BuildItem& it) {
            int b = static_cast<int>((it.c[axis] - clo[axis]) * invExt * NB);
            return b >= NB ? NB - 1 : b;
        };
        for (int i = begin; i < end; ++i) {
            const int b = bucketOf(items[i]);
            bc[b]++;
            boxUnion(blo[b], bhi[b], items[i].lo, items[i].hi);
        }
        const float invArea = 1.0f / halfArea(lo, hi);
        float best = std::numeric_limits<float>::max();
        int bestSplit = -1;
        for (int split = 0; split < NB - 1; ++split) {
            V3 alo(std::numeric_limits<float>::max()), ahi(std::numeric_limits<float>::min()), b2lo = alo, b2hi = ahi;
            int ca = 0, cb = 0;
            for (int i = 0; i <= split; ++i) if (bc[i]) { boxUnion(alo, ahi, blo[i], bhi[i]); ca += bc[i]; }
            for (int i = split + 1; i < NB; ++i) if (bc[i]) { boxUnion(b2lo, b2hi, blo[i], bhi[i]); cb += bc[i]; }
            const float pa = ca ? halfArea(alo, ahi) * invArea : 0.0f;
            const float pb = cb ? halfArea(b2lo, b2hi) * invArea : 0.0f;
            const float cost = 0.125f + (pa * ca + pb * cb);
            if (cost < best) { best = cost; bestSplit = split; }
        }
        if (best >= static_cast<float>(count)) return makeLeaf();
        auto midIt = std::partition(items.begin() + begin, items.begin() + end,
                                    [&](const BuildItem& it) { return bucketOf(it) <= bestSplit; });
        mid = static_cast<int>(midIt - items.begin());
        if (mid == begin || mid == end) return makeLeaf();
    }
    buildRec(s, items, begin, mid);
    const int second = buildRec(s, items, mid, end);
    Scene::Node& n = s.nodes[nodeIndex];
    n.lo = lo; n.hi = hi; n.second = second; n.prim = -1; n.count = 0; n.axis = axis;
    return nodeIndex;
}

// tAabb.ipp:68-127
bool slab(const Scene::Node& n, const V3& o, const V3& inv, float minT, float maxT) {
    const V3 nearT = (n.lo - o) * inv;
    const V3 farT = (n.hi - o) * inv;
    for (int k = 0; k < 3; ++k) {
        if (inv[k] > 0.0f) { minT = std::max(minT, nearT[k]); maxT = std::min(maxT, farT[k]); }
        else { minT = std::max(minT, farT[k]); maxT = std::min(maxT, nearT[k]); }
    }
    return !(minT > maxT);
}

// bvhAccelerator.cpp:40-97 (closest) and :99-156 (any)
int traverse(const Scene& s, Ray& ray, bool anyHit) {
    const V3 inv = ray.d.reciprocal();
    const int neg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
    int stack[64];
    int sp = 0, cur = 0, hit = -1;
    for (;;) {
        const Scene::Node& n = s.nodes[cur];
        if (slab(n, ray.o, inv, ray.minT, ray.maxT)) {
            if (n.second < 0) {
                for (int i = 0; i < n.count; ++i) {
                    const int p = s.order[n.prim + i];
                    float t;
                    if (primHit(s, p, ray, &t)) {
                        if (anyHit) return p;
                        ray.maxT = t;
                        hit = p;
                    }
                }
                if (sp == 0) break;
                cur = stack[--sp];
            } else if (neg[n.axis]) {
                stack[sp++] = cur + 1;
                cur = n.second;
            } else {
                stack[sp++] = n.second;
                cur = cur + 1;
            }
        } else {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
    return hit;
}

// ----------------------------------------------------- surface details ---
struct Surface {
    int prim = -1;
    V3 P, Ng, Ns, uvw, wi;
};

// triangle.cpp:233-262
V3 barycentric(const Triangle& t, const V3& p) {
    const V3 v0 = t.b - t.a, v1 = t.c - t.a, v2 = p - t.a;
    const float d00 = v0.dot(v0), d01 = v0.dot(v1), d11 = v1.dot(v1), d20 = v2.dot(v0), d21 = v2.dot(v1);
    const float den = d00 * d11 - d01 * d01;
    if (den == 0.0f) return V3(0.0f);
    const float inv = 1.0f / den;
    const float u = (d11 * d20 - d01 * d21) * inv;
    const float v = (d00 * d21 - d01 * d20) * inv;
    return V3(1.0f - u - v, u, v);
}

V3 envUvw(const V3& d);

// scene.cpp:30-65 + triangle.cpp:125-160 + rectangle.cpp:102-132 + sphere.cpp:106-135
bool intersect(const Scene& s, Ray& ray, Surface* si) {
    const int p = traverse(s, ray, false);
    if (p < 0) return false;
    si->prim = p;
    si->wi = -ray.d;
    si->P = ray.o + ray.d * ray.maxT;
    const Prim& pr = s.prims[p];
    if (pr.kind == CGPU_PRIM_SPHERE) {
        const V3 N = (si->P - s.spheres[pr.slot].c).normalize();
        si->Ng = N;
        si->Ns = N;
        si->uvw = envUvw(N);  // SphericalMapper::mappingToUvw of the shading normal
        return true;
    }
    if (pr.kind == CGPU_PRIM_TRIANGLE) {
        const Triangle& t = s.tris[pr.slot];
        const V3 Ng = triNormal(t);
        const V3 b = barycentric(t, si->P);
        si->uvw = b.x * t.uA + b.y * t.uB + b.z * t.uC;
        V3 Ns = b.x * t.nA + b.y * t.nB + b.z * t.nC;
        Ns = Ns.isZero() ? Ng : Ns.normalize();
        si->Ng = Ng;
        si->Ns = Ns;
    } else {
        const Rectangle& r = s.rects[pr.slot];
        const V3 N = rectNormal(r);
        si->Ng = N;
        si->Ns = N;
        const V3 onPlane = si->P - r.vB;
        // rectangle.cpp:122-129 (both projections divide by |eA|, as there)
        const float p1 = onPlane.dot(r.eA.normalize()) / r.eA.length();
        const float p2 = onPlane.dot(r.eB.normalize()) / r.eA.length();
        auto lerp = [](const V3& a, const V3& b, float t) {
            const float c = 1.0f - t;
            return V3(c * a.x + t * b.x, c * a.y + t * b.y, c * a.z + t * b.z);
        };
        const V3 uA(1, 0, 0), uB(0, 0, 0), uC(0, 1, 0), uD(1, 1, 0);
        si->uvw = lerp(lerp(uB, uC, p2), lerp(uA, uD, p2), p1);
    }
    return true;
}

bool occluded(const Scene& s, Ray ray) { return traverse(s, ray, true) >= 0; }

// ----------------------------------------------------------------- BSDF ---
struct BsdfSample { V3 f, L; float pdf = 0.0f; bool valid() const { return !f.isZero() && pdf > 0.0f; } };

// ptEstimator.cpp:64-72: no NEE at a BSDF with a specular lobe
bool isSpecular(int type) { return type == CGPU_BSDF_GLASS || type == CGPU_BSDF_MIRROR; }

// tRoughnessMapper.h:18-40 (SQUARE)
float roughnessToAlpha(float r) {
    const float safe = std::max(r, 0.001f);
    return std::max(safe * safe, 0.001f);
}
// isotropicGgx.cpp:11-34
float ggxD(float alpha, const V3& N, const V3& H) {
    const float NdotH = N.dot(H);
    if (NdotH <= 0.0f) return 0.0f;
    const float a2 = alpha * alpha, c2 = NdotH * NdotH, c4 = c2 * c2;
    const float tan2 = (1.0f - c2) / c2;
    return a2 / (kPi * c4 * (a2 + tan2) * (a2 + tan2));
}
// microfacet.cpp:11-23 + isotropicGgx.cpp:36-69
float ggxG(float alpha, const V3& V, const V3& L, const V3& N, const V3& H) {
    const float VdotH = V.dot(H), VdotN = V.dot(N), LdotH = L.dot(H), LdotN = L.dot(N);
    if (!((VdotH * VdotN > 0.0f) && (LdotH * LdotN > 0.0f))) return 0.0f;
    const float a2 = alpha * alpha;
    const float v2 = VdotN * VdotN;
    const float g1v = 2.0f / (1.0f + std::sqrt(1.0f + a2 * ((1.0f - v2) / v2)));
    const float l2 = LdotN * LdotN;
    const float g1l = 2.0f / (1.0f + std::sqrt(1.0f + a2 * ((1.0f - l2) / l2)));
    return g1v * g1l;
}
// isotropicGgx.cpp:71-100
V3 ggxSampleH(float alpha, float u0, float u1) {
    const float s0 = std::min(std::max(u0, 0.0f), 0.9999f);
    const float s1 = std::min(std::max(u1, 0.0f), 0.9999f);
    const float phi = kTwoPi * s0;
    const float theta = std::atan(alpha * std::sqrt(s1 / (1.0f - s1)));
    if (!std::isfinite(theta)) return V3(0.0f, 1.0f, 0.0f);
    const float c = std::cos(theta);
    const float sn = std::sqrt(1.0f - c * c);
    return V3(std::sin(phi) * sn, c, std::cos(phi) * sn);
}
// schlickConductorFresnel.cpp:28-41
V3 schlick(const V3& f0, float cosI) {
    const float c = 1.0f - std::abs(cosI);
    const V3 comp = f0.complement();
    return f0 + comp * c * (c * c) * (c * c);
}
// vanillaDielectricFresnel.cpp:17-48
float dielectricFresnel(float etaI, float etaT, float cosI) {
    if (cosI < 0.0f) { std::swap(etaI, etaT); cosI *= -1.0f; }
    const float ratio = etaI / etaT;
    const float sinT2 = ratio * ratio * (1.0f - cosI * cosI);
    if (sinT2 >= 1.0f) return 1.0f;
    const float cosT = std::sqrt(1.0f - sinT2);
    const float rPar = (etaT * cosI - etaI * cosT) / (etaT * cosI + etaI * cosT);
    const float rPer = (etaI * cosI - etaT * cosT) / (etaI * cosI + etaT * cosT);
    return 0.5f * (rPar * rPar + rPer * rPer);
}
// tVector.ipp:468-503
bool canRefract(const V3& v, const V3& n, float etaI, float etaT, V3* out) {
    float sign = 1.0f;
    const float cosI = v.dot(n);
    if (cosI < 0.0f) { std::swap(etaI, etaT); sign = -1.0f; }
    const float ratio = etaI / etaT;
    const float sinT2 = ratio * ratio * (1.0f - cosI * cosI);
    if (sinT2 >= 1.0f) return false;
    const float cosT = std::sqrt(1.0f - sinT2);
    V3 r = v * (-ratio);
    r += n * ((ratio * sign * cosI - cosT) * sign);
    *out = r.normalize();
    return true;
}

// RgbImageTexture::evaluate with the nearest sampler and repeat wrap
// (rgbImageTexture.cpp:8-15, tNearestPixelSampler.ipp:14-31, repeatUvwWrapper.cpp:9-15)
const Scene* g_scene = nullptr;
V3 albedoAt(const Material& m, const V3& uvw) {
    if (m.tex < 0) return m.albedo;
    const Texture& t = g_scene->textures[size_t(m.tex)];
    const float u = uvw.x - std::floor(uvw.x), v = uvw.y - std::floor(uvw.y);
    int x = static_cast<int>(u * t.w), y = static_cast<int>(v * t.h);
    x = x < t.w ? x : x - 1;
    y = y < t.h ? y : y - 1;
    const float* p = &t.texels[3 * (size_t(y) * t.w + x)];
    return V3(p[0], p[1], p[2]);
}

// Rough GGX dielectric: no reference counterpart (the reference only has the
// smooth SpecularDielectric).  Walter, Marschner, Li & Torrance 2007 BRDF +
// BTDF in radiance form with a Fresnel-weighted lobe choice, normal turned to
// V's side; the same definition as the CUDA library's.  Parity for this
// material is unpinned against the reference.
void roughDielectric(const Material& m, const V3& alb, const V3& V, const V3& L, const V3& N, V3* f, float* pdf) {
    *f = V3(0.0f);
    *pdf = 0.0f;
    const float cv = V.dot(N), cl = L.dot(N);
    if (cv == 0.0f || cl == 0.0f) return;
    const V3 Nv = cv > 0.0f ? N : -N;
    const float etaV = cv > 0.0f ? m.iorOuter : m.iorInner;
    const float etaL = cv > 0.0f ? m.iorInner : m.iorOuter;
    const float acv = std::abs(cv), acl = std::abs(cl);
    const float alpha = roughnessToAlpha(m.roughness);
    if (cv * cl > 0.0f) {
        V3 H = V + L;
        if (H.isZero()) return;
        H = H.normalize();
        const float VH = V.dot(H);
        if (VH <= 0.0f) return;
        const float F = dielectricFresnel(etaV, etaL, VH);
        const float NH = Nv.dot(H);
        const float D = ggxD(alpha, Nv, H);
        const float G = ggxG(alpha, V, L, Nv, H);
        *f = alb * (F * D * G / (4.0f * acv * acl));
        *pdf = F * D * NH / (4.0f * VH);
    } else {
        const float eta = etaL / etaV;
        V3 H = V + L * eta;
        if (H.isZero()) return;
        H = H.normalize();
        if (H.dot(Nv) < 0.0f) H = -H;
        const float VH = V.dot(H), LH = L.dot(H);
        if (!(VH > 0.0f && LH < 0.0f)) return;
        const float F = dielectricFresnel(etaV, etaL, VH);
        const float NH = Nv.dot(H);
        const float D = ggxD(alpha, Nv, H);
        const float G = ggxG(alpha, V, L, Nv, H);
        const float den = VH + eta * LH;
        const float den2 = den * den;
        *f = alb * ((1.0f - F) * D * G * std::abs(VH * LH) / (acv * acl * den2));
        *pdf = (1.0f - F) * D * NH * eta * eta * std::abs(LH) / den2;
    }
    if (!std::isfinite(*pdf)) { *pdf = 0.0f; *f = V3(0.0f); }
}

// PhongBsdf (phongBsdf.cpp:14-98)
float phongPdfFactor(const Material& m) { return (m.exponent + 1.0f) * 0.1591549430918953f; }
float phongBrdfFactor(const Material& m) { return (m.exponent + 2.0f) * 0.1591549430918953f; }
V3 phongEval(const Material& m, const Surface& si, const V3& L) {
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    const V3 R = L.reflect(Ns);
    if (V.dot(Ns) * L.dot(Ns) <= 0.0f) return V3(0.0f);
    const float RdotV = std::max(R.dot(V), 0.0f);
    return V3(std::pow(RdotV, m.exponent) * phongBrdfFactor(m));
}
float phongPdf(const Material& m, const Surface& si, const V3& L) {
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    const V3 R = L.reflect(Ns);
    if (V.dot(Ns) * L.dot(Ns) <= 0.0f) return 0.0f;
    const float RdotV = std::max(R.dot(V), 0.0f);
    return std::pow(RdotV, m.exponent) * phongPdfFactor(m);
}
V3 lambertEval(const Material& m, const Surface& si, const V3& L);
float lambertPdf(const Surface& si, const V3& L);

// lambertianDiffuse.cpp:27-44 / conductorMicrofacet.cpp:32-66 / phongBsdf.cpp /
// mixedBsdf.cpp:33-57 (plastic = Mixed(Lambertian, Phong, ratio))
V3 bsdfEval(const Material& m, const Surface& si, const V3& L) {
    if (m.type == CGPU_BSDF_PHONG) return phongEval(m, si, L);
    if (m.type == CGPU_BSDF_PLASTIC) {
        const V3 ratio(m.ratio);
        return lambertEval(m, si, L) * ratio + phongEval(m, si, L) * ratio.complement();
    }
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    if (m.type == CGPU_BSDF_LAMBERTIAN) {
        if (V.dot(Ns) * L.dot(Ns) <= 0.0f) return V3(0.0f);
        return albedoAt(m, si.uvw) * kInvPi;
    }
    if (m.type == CGPU_BSDF_CONDUCTOR_GGX) {
        const float VdotN = V.dot(Ns), LdotN = L.dot(Ns);
        if (VdotN * LdotN <= 0.0f) return V3(0.0f);
        const float sgn = static_cast<float>((0.0f < VdotN) - (VdotN < 0.0f));
        V3 H = (V + L) * sgn;
        if (H.isZero()) return V3(0.0f);
        H = H.normalize();
        const float alpha = roughnessToAlpha(m.roughness);
        const V3 F = schlick(m.f0, L.dot(H));
        const float D = ggxD(alpha, Ns, H);
        const float G = ggxG(alpha, V, L, Ns, H);
        return F * G * D / (4.0f * std::abs(VdotN * LdotN));
    }
    if (m.type == CGPU_BSDF_DIELECTRIC_GGX) {
        V3 f;
        float pdf;
        roughDielectric(m, albedoAt(m, si.uvw), si.wi, L, si.Ns, &f, &pdf);
        return f;
    }
    return V3(0.0f);
}

// lambertianDiffuse.cpp:83-96 / conductorMicrofacet.cpp:126-163 / mixedBsdf.cpp:157-185
float bsdfPdf(const Material& m, const Surface& si, const V3& L) {
    if (m.type == CGPU_BSDF_PHONG) return phongPdf(m, si, L);
    if (m.type == CGPU_BSDF_PLASTIC) {
        const float avg = V3(m.ratio).average();
        return lambertPdf(si, L) * avg + phongPdf(m, si, L) * (1.0f - avg);
    }
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    if (m.type == CGPU_BSDF_LAMBERTIAN) {
        if (V.dot(Ns) * L.dot(Ns) <= 0.0f) return 0.0f;
        return L.absDot(Ns) * kInvPi;
    }
    if (m.type == CGPU_BSDF_CONDUCTOR_GGX) {
        const float VdotN = V.dot(Ns), LdotN = L.dot(Ns);
        if (VdotN * LdotN <= 0.0f) return 0.0f;
        const float sgn = static_cast<float>((0.0f < VdotN) - (VdotN < 0.0f));
        V3 H = (V + L) * sgn;
        if (H.isZero()) return 0.0f;
        H = H.normalize();
        const float alpha = roughnessToAlpha(m.roughness);
        const float D = ggxD(alpha, Ns, H);
        const float pdfH = std::abs(D * Ns.dot(H));
        const float pdfL = std::abs(pdfH / (4.0f * L.dot(H)));
        return std::isfinite(pdfL) ? pdfL : 0.0f;
    }
    if (m.type == CGPU_BSDF_DIELECTRIC_GGX) {
        V3 f;
        float pdf;
        roughDielectric(m, V3(1.0f), si.wi, L, si.Ns, &f, &pdf);
        return pdf;
    }
    return 0.0f;
}

V3 lambertEval(const Material& m, const Surface& si, const V3& L) {
    if (si.wi.dot(si.Ns) * L.dot(si.Ns) <= 0.0f) return V3(0.0f);
    return albedoAt(m, si.uvw) * kInvPi;
}
float lambertPdf(const Surface& si, const V3& L) {
    if (si.wi.dot(si.Ns) * L.dot(si.Ns) <= 0.0f) return 0.0f;
    return L.absDot(si.Ns) * kInvPi;
}

BsdfSample bsdfSample(const Material& m, const Surface& si, Rng& rng);

// phongBsdf.cpp:38-81 with hemisphere.cpp:50-69 (lobe around the normal)
BsdfSample phongSample(const Material& m, const Surface& si, Rng& rng) {
    BsdfSample out;
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    V3 z, x;
    buildCoordinateSystem(Ns, &z, &x);
    float u0, u1;
    rng.next2(&u0, &u1);
    const float phi = kTwoPi * u0;
    const float cosTheta = std::pow(u1, 1.0f / (m.exponent + 1.0f));
    const float sinTheta = std::sqrt(1.0f - cosTheta * cosTheta);
    V3 L(std::sin(phi) * sinTheta, cosTheta, std::cos(phi) * sinTheta);
    L = x * L.x + Ns * L.y + z * L.z;
    L = L.normalize();
    if (V.dot(Ns) * L.dot(Ns) <= 0.0f) return out;
    const V3 R = L.reflect(Ns);
    const float RdotV = std::max(R.dot(V), 0.0f);
    const float powerTerm = std::pow(RdotV, m.exponent);
    out.f = V3(powerTerm * phongBrdfFactor(m));
    out.L = L;
    out.pdf = powerTerm * phongPdfFactor(m);
    return out;
}

BsdfSample bsdfSample(const Material& m, const Surface& si, Rng& rng) {
    BsdfSample out;
    const V3& Ns = si.Ns;
    const V3& V = si.wi;
    if (m.type == CGPU_BSDF_PHONG) return phongSample(m, si, rng);
    if (m.type == CGPU_BSDF_PLASTIC) {  // mixedBsdf.cpp:59-155 (A Lambertian, B Phong)
        const V3 ratio(m.ratio);
        const float averageRatio = ratio.average();
        const float sample = rng.next();
        if (sample < ratio.average()) {
            Material a = m;
            a.type = CGPU_BSDF_LAMBERTIAN;
            const BsdfSample ls = bsdfSample(a, si, rng);
            if (!ls.valid()) return out;
            const V3 fA = ls.f, fB = phongEval(m, si, ls.L);
            out.f = ratio * fA + ratio.complement() * fB;
            out.L = ls.L;
            out.pdf = averageRatio * ls.pdf + (1.0f - averageRatio) * phongPdf(m, si, ls.L);
        } else {
            const BsdfSample ls = phongSample(m, si, rng);
            if (!ls.valid()) return out;
            const V3 fB = ls.f, fA = lambertEval(m, si, ls.L);
            out.f = ratio * fB + ratio.complement() * fA;  // as mixedBsdf.cpp:123-128 writes it
            out.L = ls.L;
            out.pdf = averageRatio * ls.pdf + (1.0f - averageRatio) * lambertPdf(si, ls.L);
        }
        return out;
    }
    if (m.type == CGPU_BSDF_MIRROR) {  // specularReflection.cpp:32-57
        const float VdotN = V.dot(Ns);
        const float NFactor = (VdotN > 0.0f) ? 1.0f : -1.0f;
        const V3 L = V.reflect(Ns * NFactor);
        const float LdotN = L.dot(Ns);
        const V3 reflectance = m.fresnel == CGPU_FRESNEL_CONDUCTOR ? schlick(m.f0, LdotN)
                                                                   : V3(dielectricFresnel(m.iorOuter, m.iorInner, LdotN));
        out.f = reflectance * albedoAt(m, si.uvw) / std::abs(LdotN);
        out.L = L;
        out.pdf = 1.0f;
        return out;
    }
    if (m.type == CGPU_BSDF_LAMBERTIAN) {  // lambertianDiffuse.cpp:46-81
        V3 z, x;
        buildCoordinateSystem(Ns, &z, &x);
        float u0, u1;
        rng.next2(&u0, &u1);
        // hemisphere.cpp:30-48
        const float phi = kTwoPi * u0;
        const float theta = std::acos(1.0f - 2.0f * u1) * 0.5f;
        const float c = std::cos(theta);
        const float sn = std::sqrt(1.0f - c * c);
        V3 L(std::sin(phi) * sn, c, std::cos(phi) * sn);
        const float pdf = c * kInvPi;
        L = x * L.x + Ns * L.y + z * L.z;
        L = L.normalize();
        if (V.dot(Ns) <= 0.0f) L = -L;
        out.f = albedoAt(m, si.uvw) * kInvPi;
        out.L = L;
        out.pdf = pdf;
        return out;
    }
    if (m.type == CGPU_BSDF_CONDUCTOR_GGX) {  // conductorMicrofacet.cpp:68-124
        const float nf = V.dot(Ns) > 0.0f ? 1.0f : -1.0f;
        const float alpha = roughnessToAlpha(m.roughness);
        V3 z, x;
        buildCoordinateSystem(Ns, &z, &x);
        float u0, u1;
        rng.next2(&u0, &u1);
        V3 H = ggxSampleH(alpha, u0, u1);
        H = x * H.x + Ns * H.y + z * H.z;
        H = H.normalize();
        const V3 L = V.reflect(H * nf);
        const float VdotN = V.dot(Ns), LdotN = L.dot(Ns), LdotH = L.dot(H), NdotH = Ns.dot(H);
        if (VdotN * LdotN <= 0.0f) return out;
        const V3 F = schlick(m.f0, LdotH);
        const float D = ggxD(alpha, Ns, H);
        const float G = ggxG(alpha, V, L, Ns, H);
        const float pdfH = std::abs(D * NdotH);
        const float pdfL = std::abs(pdfH / (4.0f * LdotH));
        if (!std::isfinite(pdfL)) return out;
        out.f = F * G * D / (4.0f * std::abs(VdotN * LdotN));
        out.L = L;
        out.pdf = pdfL;
        return out;
    }
    if (m.type == CGPU_BSDF_GLASS) {  // specularDielectric.cpp:35-127
        const float VdotN = V.dot(Ns);
        const float R = dielectricFresnel(m.iorOuter, m.iorInner, VdotN);
        const V3 reflectance(R);
        const float pr = reflectance.average();
        const float u = rng.next();
        const V3 alb = albedoAt(m, si.uvw);
        if (u < pr) {
            const float nf = VdotN > 0.0f ? 1.0f : -1.0f;
            const V3 L = V.reflect(Ns * nf);
            const float LdotN = L.absDot(Ns);
            out.f = alb * reflectance / LdotN;
            out.L = L;
            out.pdf = pr;
        } else {
            float etaI = m.iorOuter, etaT = m.iorInner;
            V3 L;
            if (!canRefract(V, Ns, etaI, etaT, &L)) return out;
            const float cosI = L.dot(Ns);
            const V3 Rt(dielectricFresnel(m.iorOuter, m.iorInner, cosI));
            if (cosI < 0.0f) std::swap(etaI, etaT);
            const float btdf = (etaT * etaT) / (etaI * etaI);
            const float LdotN = std::abs(cosI);
            const V3 trans = Rt.complement();
            out.f = alb * trans * btdf / LdotN;
            out.L = L;
            out.pdf = 1.0f - pr;
        }
        return out;
    }
    if (m.type == CGPU_BSDF_DIELECTRIC_GGX) {
        const float cv = V.dot(Ns);
        if (cv == 0.0f) return out;
        const V3 Nv = cv > 0.0f ? Ns : -Ns;
        const float etaV = cv > 0.0f ? m.iorOuter : m.iorInner;
        const float etaL = cv > 0.0f ? m.iorInner : m.iorOuter;
        V3 z, x;
        buildCoordinateSystem(Nv, &z, &x);
        float u0, u1;
        rng.next2(&u0, &u1);
        V3 H = ggxSampleH(roughnessToAlpha(m.roughness), u0, u1);
        H = (x * H.x + Nv * H.y + z * H.z).normalize();
        const float VH = V.dot(H);
        const float u = rng.next();
        if (VH <= 0.0f) return out;
        const float F = dielectricFresnel(etaV, etaL, VH);
        V3 L;
        if (u < F) {
            L = H * (2.0f * VH) - V;
        } else {
            const float ratio = etaV / etaL;
            const float sinT2 = ratio * ratio * (1.0f - VH * VH);
            if (sinT2 >= 1.0f) return out;
            const float cosT = std::sqrt(1.0f - sinT2);
            L = (V * (-ratio) + H * (ratio * VH - cosT)).normalize();
        }
        roughDielectric(m, albedoAt(m, si.uvw), V, L, Ns, &out.f, &out.pdf);
        out.L = L;
        return out;
    }
    return out;  // absorber: invalid (absorberBsdf.cpp)
}

// ---------------------------------------------------------------- lights ---
struct LightSample { V3 pos, N, radiance; float pdfW = 0.0f; bool valid() const { return !radiance.isZero() && pdfW > 0.0f; } };

bool canEmit(const Light& l, const V3& dir, const V3& N) { return (dir.dot(N) >= 0.0f) != l.backFace; }  // areaLight.cpp:24-28

// Environment light.  The reference samples its sky with a z-up inverse
// (infiniteSphere.cpp:62-78) of a y-up lookup (sphericalMapper.cpp:14-28), so
// its NEE and BSDF sampling see differently rotated skies; this restatement
// (and the CUDA library) use the y-up mapping for both.  Unpinned against the
// reference.
V3 envDir(float u, float v) {
    const float st = std::sin((1.0f - v) * kPi), ct = std::cos((1.0f - v) * kPi);
    return V3(st * std::sin(kTwoPi * u), ct, st * std::cos(kTwoPi * u));
}
V3 envUvw(const V3& d) {
    const V3 n = d.normalize();
    const float theta = std::acos(std::min(std::max(n.y, -1.0f), 1.0f));
    float phi = std::atan2(n.x, n.z);
    if (phi < 0.0f) phi += kTwoPi;
    return V3(phi * 0.1591549430918953f, (kPi - theta) * kInvPi, 0.0f);  // constant::inv_two_pi
}
V3 texel(const Scene& s, int tex, const V3& uvw) {
    const Texture& t = s.textures[size_t(tex)];
    const float u = uvw.x - std::floor(uvw.x), v = uvw.y - std::floor(uvw.y);
    int x = static_cast<int>(u * t.w), y = static_cast<int>(v * t.h);
    x = x < t.w ? x : x - 1;
    y = y < t.h ? y : y - 1;
    const float* p = &t.texels[3 * (size_t(y) * t.w + x)];
    return V3(p[0], p[1], p[2]);
}
int cdfFind(const float* cdf, int n, float u) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cdf[mid] <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}
float envPdfW(const Scene& s, const V3& dir) {
    const V3 uvw = envUvw(dir);
    const float st = std::sin((1.0f - uvw.y) * kPi);
    if (st <= 0.0f) return 0.0f;
    const Texture& t = s.textures[size_t(s.envTex)];
    const int iy = std::max(std::min(int(uvw.y * t.h), t.h - 1), 0);
    const int ix = std::max(std::min(int(uvw.x * t.w), t.w - 1), 0);
    const float* c = &s.envCond[size_t(iy) * (t.w + 1)];
    const float pdf = (s.envMarg[iy + 1] - s.envMarg[iy]) * float(t.h) * (c[ix + 1] - c[ix]) * float(t.w);
    return pdf / (2.0f * kPi * kPi * st);
}

// singleAreaLight.cpp:54-85 with the position samplers of
// triangle.cpp:162-193 (sampleWarp.cpp:10-19) and rectangle.cpp:134-169.
LightSample lightSample(const Scene& s, const Light& l, const V3& target, Rng& rng) {
    LightSample out;
    if (l.prim < 0) {  // environment: Distribution2D row from .y, column from .x
        const Texture& t = s.textures[size_t(s.envTex)];
        float sx, sy;
        rng.next2(&sx, &sy);
        const int iy = cdfFind(s.envMarg.data(), t.h, sy);
        const float* c = &s.envCond[size_t(iy) * (t.w + 1)];
        const int ix = cdfFind(c, t.w, sx);
        const float m0 = s.envMarg[iy], m1 = s.envMarg[iy + 1], c0 = c[ix], c1 = c[ix + 1];
        float dy = sy - m0, dx = sx - c0;
        if (m1 > m0) dy /= m1 - m0;
        if (c1 > c0) dx /= c1 - c0;
        const float v = std::min(std::max((float(iy) + dy) / float(t.h), 0.0f), 1.0f);
        const float u = std::min(std::max((float(ix) + dx) / float(t.w), 0.0f), 1.0f);
        const float pdfUv = (m1 - m0) * float(t.h) * (c1 - c0) * float(t.w);
        const float st = std::sin((1.0f - v) * kPi);
        if (st <= 0.0f || !(pdfUv > 0.0f)) return out;
        out.pos = target + envDir(u, v) * 1.0e6f;
        out.pdfW = pdfUv / (2.0f * kPi * kPi * st);
        out.radiance = texel(s, s.envTex, V3(u, v, 0.0f));
        return out;
    }
    const Prim& pr = s.prims[l.prim];
    V3 P, Ns;
    float pdfA;
    if (pr.kind == CGPU_PRIM_TRIANGLE) {
        const Triangle& t = s.tris[pr.slot];
        float u0, u1;
        rng.next2(&u0, &u1);
        const float sa = std::sqrt(u0);
        const float ss = 1.0f - sa, st = sa * u1;
        P = t.a + t.eAB * ss + t.eAC * st;
        const V3 b = barycentric(t, P);
        const V3 Ng = triNormal(t);
        V3 n = b.x * t.nA + b.y * t.nB + b.z * t.nC;
        Ns = n.isZero() ? Ng : n;
        pdfA = 1.0f / triArea(t);
    } else {
        const Rectangle& r = s.rects[pr.slot];
        V3 eA = r.eA, eB = r.eB;
        if (eA.length() < eB.length()) std::swap(eA, eB);
        const float longW = eA.length(), shortW = eB.length();
        float a, b;
        do {
            a = rng.next();
            b = rng.next();
        } while (b > shortW / longW);
        P = r.vB + eA * a + eB.normalize() * (b * eA.length());
        Ns = rectNormal(r);
        pdfA = 1.0f / rectArea(r);
    }
    if (!(pdfA > 0.0f)) return out;
    const V3 emitVec = target - P;
    if (!canEmit(l, emitVec, Ns)) return out;
    const float d2 = emitVec.lengthSquared();
    const float cosE = (emitVec / std::sqrt(d2)).absDot(Ns);
    if (cosE <= 0.0f) return out;
    out.pos = P;
    out.N = Ns;
    out.pdfW = pdfA * d2 / cosE;
    out.radiance = l.radiance;
    return out;
}

float lightArea(const Scene& s, const Light& l) {
    const Prim& pr = s.prims[l.prim];
    return pr.kind == CGPU_PRIM_TRIANGLE ? triArea(s.tris[pr.slot]) : rectArea(s.rects[pr.slot]);
}

// singleAreaLight.cpp:39-52
V3 emittance(const Light& l, const Surface& si) {
    if (!canEmit(l, si.wi, si.Ns)) return V3(0.0f);
    return l.radiance;
}
// singleAreaLight.cpp:87-109
float lightPdfW(const Scene& s, const Light& l, const Surface& si, const V3& target) {
    const V3 emitVec = target - si.P;
    if (!canEmit(l, si.wi, si.Ns)) return 0.0f;
    const float c = si.wi.absDot(si.Ns);
    if (c <= 0.0f) return 0.0f;
    const float pdfA = 1.0f / lightArea(s, l);
    return pdfA * emitVec.lengthSquared() / c;
}

// Scene::sampleOneLight through the light cluster: UniformLightCluster
// (uniformLightCluster.cpp:15-24, Random::nextIndex) or PowerLightCluster
// (powerLightCluster.cpp:29-36: Distribution1D::sampleDiscrete, whose
// continuousToDiscrete scans the CDF from the top, distribution1D.cpp:115-125).
std::size_t pickLight(const Scene& s, Rng& rng, float* pdf) {
    if (s.lightCdf.empty()) {
        *pdf = 1.0f / static_cast<float>(s.lights.size());
        return rng.index(0, s.lights.size());
    }
    const float u = rng.next();
    std::size_t i = s.lights.size() - 1;
    while (i > 0 && !(s.lightCdf[i] <= u)) --i;
    *pdf = s.lightCdf[i + 1] - s.lightCdf[i];
    return i;
}

float misPower(float a, float b) {  // tMis.h:21-47
    const float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}

// directLightEvaluator.cpp:18-109
V3 directLight(const Scene& s, const Surface& si, const Material& m, int lightIndex, Rng& rng) {
    V3 result(0.0f);
    if (m.type == CGPU_BSDF_ABSORBER) return result;
    const Light& l = s.lights[lightIndex];
    const V3 P = si.P, Ns = si.Ns;
    {
        const LightSample ls = lightSample(s, l, P, rng);
        if (ls.valid()) {
            const V3 Lv = ls.pos - P;
            const float dist = Lv.length();
            const V3 L = Lv / dist;
            Ray shadow;
            shadow.o = P;
            shadow.d = L.normalize();
            shadow.maxT = dist - kRayEps;
            if (!occluded(s, shadow)) {
                const V3 f = bsdfEval(m, si, L);
                const V3 factor = f * L.absDot(Ns);
                const float bp = bsdfPdf(m, si, L);
                const float w = misPower(ls.pdfW, bp);
                result += w * ls.radiance * factor / ls.pdfW;
            }
        }
    }
    {
        const BsdfSample bs = bsdfSample(m, si, rng);
        if (bs.valid()) {
            Ray r;
            r.o = P;
            r.d = bs.L.normalize();
            Surface hit;
            if (intersect(s, r, &hit)) {
                if (s.prims[hit.prim].light == lightIndex) {
                    const V3 factor = bs.f * bs.L.absDot(Ns);
                    const V3 rad = emittance(l, hit);
                    const float lp = lightPdfW(s, l, hit, P);
                    const float w = misPower(bs.pdf, lp);
                    result += w * rad * factor / bs.pdf;
                }
            } else if (lightIndex == s.envLight) {
                const V3 factor = bs.f * bs.L.absDot(Ns);
                const V3 rad = texel(s, s.envTex, envUvw(r.d));
                const float w = misPower(bs.pdf, envPdfW(s, r.d));
                result += w * rad * factor / bs.pdf;
            }
        }
    }
    return result;
}

// ptEstimator.cpp:25-123
V3 estimate(const Scene& s, Ray ray, Rng& rng) {
    V3 L(0.0f), T(1.0f);
    bool countEmission = true;
    for (int bounce = 0; bounce < s.maxDepth; ++bounce) {
        Surface si;
        if (!intersect(s, ray, &si)) {
            if (s.envLight >= 0 && countEmission) L += T * texel(s, s.envTex, envUvw(ray.d));
            break;
        }
        const Prim& pr = s.prims[si.prim];
        const Material& m = s.mats[pr.material];
        if (pr.light >= 0 && countEmission) {
            L += T * emittance(s.lights[pr.light], si);
        }
        if (!isSpecular(m.type)) {
            countEmission = false;
            float pick;
            const std::size_t li = pickLight(s, rng, &pick);
            const V3 direct = directLight(s, si, m, static_cast<int>(li), rng) / pick;
            L += T * direct;
        } else {
            countEmission = true;
        }
        const BsdfSample bs = bsdfSample(m, si, rng);
        if (!bs.valid()) break;
        const float LdotN = bs.L.absDot(si.Ns);
        T *= bs.f * LdotN / bs.pdf;
        if (bounce > 2) {  // russianRoulette.cpp:9-28
            const float q = std::min(std::max(1.0f - T.maxComponent(), 0.05f), 1.0f);
            const float u = rng.next();
            if (u > q) T = T * (1.0f / (1.0f - q));
            else break;
        }
        if (T.isZero()) break;
        ray = Ray();
        ray.o = si.P;
        ray.d = bs.L.normalize();
    }
    return L;
}

// perspectivePinholeCamera.cpp:52-73 with the film->camera transform of :32-50
// and the camera->world lookAt of tMatrix4.ipp:47-60.
Ray cameraRay(const Scene& s, double fx, double fy) {
    const float x = static_cast<float>(fx), y = static_cast<float>(fy);
    const float cx = s.sx * x + s.tx;
    const float cy = s.sy * y + s.ty;
    const float cz = -s.offset;
    V3 d(s.camX.x * cx + s.camY.x * cy + s.camZ.x * cz,
         s.camX.y * cx + s.camY.y * cy + s.camZ.y * cz,
         s.camX.z * cx + s.camY.z * cy + s.camZ.z * cz);
    Ray r;
    r.o = s.camPos;
    r.d = d.normalize();
    return r;
}

// Sample layout shared with the CUDA library: sample `si` of a pixel takes
// stratum si of the floor(sqrt(spp))^2 grid (strata beyond it are uniform),
// jittered by the first two draws of the path stream.  This is the set the
// reference's StratifiedSampler produces (stratifiedSampler.cpp:38-73) without
// its shuffle, which only reorders samples within a pixel.
void jitter(int spp, uint32_t si, Rng& rng, float* jx, float* jy) {
    const int base = static_cast<int>(std::floor(std::sqrt(static_cast<float>(spp))));
    const float u0 = rng.next(), u1 = rng.next();
    if (static_cast<int>(si) < base * base) {
        const float inv = 1.0f / static_cast<float>(base);
        *jx = (static_cast<float>(si % base) + u0) * inv;
        *jy = (static_cast<float>(si / base) + u1) * inv;
    } else {
        *jx = u0;
        *jy = u1;
    }
}

V3 vload(const float* p) { return V3(p[0], p[1], p[2]); }

Scene* create(const cgpu_scene_desc* d) {
    auto s = std::make_unique<Scene>();
    s->W = d->width; s->H = d->height; s->maxDepth = d->max_depth; s->spp = d->spp > 0 ? d->spp : 1;
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const cgpu_material& m = d->materials[i];
        s->mats.push_back({m.type, vload(m.albedo), vload(m.f0), m.roughness, m.ior_outer, m.ior_inner, m.albedo_texture,
                           m.exponent, m.diffuse_ratio, m.fresnel});
    }
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        Texture t;
        t.w = d->textures[i].width;
        t.h = d->textures[i].height;
        t.texels.assign(d->textures[i].texels, d->textures[i].texels + size_t(t.w) * t.h * 3);
        s->textures.push_back(std::move(t));
    }
    for (uint32_t i = 0; i < d->num_primitives; ++i) {
        const int kind = d->prim_kind ? d->prim_kind[i] : CGPU_PRIM_TRIANGLE;
        const float* v = d->prim_vertices + 9 * static_cast<std::size_t>(i);
        Prim p{kind, d->prim_material[i], -1, 0};
        if (kind == CGPU_PRIM_TRIANGLE) {
            Triangle t;
            t.a = vload(v); t.b = vload(v + 3); t.c = vload(v + 6);
            t.eAB = t.b - t.a; t.eAC = t.c - t.a;
            const V3 N0 = t.eAB.cross(t.eAC);
            const V3 N = N0.isZero() ? V3(0.0f, 1.0f, 0.0f) : N0.normalize();
            t.nA = t.nB = t.nC = N;
            if (d->prim_normals) {  // triangleMesh.cpp:24-28 (setN* ignores zero normals)
                const float* n = d->prim_normals + 9 * static_cast<std::size_t>(i);
                if (!vload(n).isZero()) t.nA = vload(n);
                if (!vload(n + 3).isZero()) t.nB = vload(n + 3);
                if (!vload(n + 6).isZero()) t.nC = vload(n + 6);
            }
            t.uA = V3(0, 0, 0); t.uB = V3(1, 0, 0); t.uC = V3(0, 1, 0);
            if (d->prim_uvws) {
                const float* u = d->prim_uvws + 9 * static_cast<std::size_t>(i);
                t.uA = vload(u); t.uB = vload(u + 3); t.uC = vload(u + 6);
            }
            p.slot = static_cast<int>(s->tris.size());
            s->tris.push_back(t);
        } else if (kind == CGPU_PRIM_SPHERE) {
            p.slot = static_cast<int>(s->spheres.size());
            s->spheres.push_back(Sphere{vload(v), v[3]});
        } else {
            Rectangle r;
            r.vA = vload(v); r.vB = vload(v + 3); r.vC = vload(v + 6);
            r.eA = r.vA - r.vB; r.eB = r.vC - r.vB;
            r.vD = r.vB + r.eA + r.eB;
            p.slot = static_cast<int>(s->rects.size());
            s->rects.push_back(r);
        }
        s->prims.push_back(p);
    }
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const cgpu_area_light& l = d->lights[i];
        Light L;
        L.prim = l.primitive;
        L.backFace = l.back_face_emit != 0;
        const V3 color = vload(l.color);
        const V3 unit = color / color.sum();
        const V3 total = unit * l.watt;
        s->lights.push_back(L);
        const float area = lightArea(*s, s->lights.back());
        s->lights.back().radiance = total / area * kInvPi;  // singleAreaLight.cpp:32-36
        s->prims[l.primitive].light = static_cast<int>(i);
    }
    if (d->environment_texture > 0) {  // same weights and CDFs as the CUDA library's upload
        const int tex = d->environment_texture - 1;
        const Texture& t = s->textures[size_t(tex)];
        const int W = t.w, H = t.h;
        s->envTex = tex;
        s->envMarg.assign(size_t(H) + 1, 0.0f);
        s->envCond.assign(size_t(H) * (W + 1), 0.0f);
        std::vector<double> rows(static_cast<size_t>(H), 0.0);
        double total = 0.0;
        for (int y = 0; y < H; ++y) {
            const double st = std::sin((1.0 - (y + 0.5) / H) * 3.14159265358979323846);
            double acc = 0.0;
            std::vector<double> wrow(static_cast<size_t>(W));
            for (int x = 0; x < W; ++x) {
                const float* p = &t.texels[3 * (size_t(y) * W + x)];
                const double lum = 0.2126 * p[0] + 0.7152 * p[1] + 0.0722 * p[2];
                wrow[size_t(x)] = std::max(lum, 0.0) * st;
                acc += wrow[size_t(x)];
            }
            float* c = &s->envCond[size_t(y) * (W + 1)];
            double run = 0.0;
            for (int x = 0; x < W; ++x) {
                run += acc > 0.0 ? wrow[size_t(x)] / acc : 1.0 / W;
                c[x + 1] = float(run);
            }
            c[W] = 1.0f;
            rows[size_t(y)] = acc;
            total += acc;
        }
        double run = 0.0;
        for (int y = 0; y < H; ++y) {
            run += rows[size_t(y)] / total;
            s->envMarg[size_t(y) + 1] = float(run);
        }
        s->envMarg[size_t(H)] = 1.0f;
        Light env;
        env.prim = -1;
        env.backFace = false;
        s->envLight = static_cast<int>(s->lights.size());
        s->lights.push_back(env);
    }
    if (d->light_cluster == CGPU_LIGHT_CLUSTER_POWER) {
        // approximate fluxes: SingleAreaLight::approximateFlux (singleAreaLight.cpp:170-187),
        // luminance with the weights of rgbSpectrum.cpp:33-37; the sky as
        // EnvironmentLight::approximateFlux (environmentLight.cpp:32-50, 125-139) with R
        // half the diagonal of the primitives' bounds
        auto luminance = [](const V3& c) { return 0.0126f * c.x + 0.7152f * c.y + 0.0722f * c.z; };
        const std::size_t n = s->lights.size();
        std::vector<float> flux(n);
        for (std::size_t i = 0; i < n; ++i) {
            const Light& L = s->lights[i];
            if (static_cast<int>(i) == s->envLight) {
                const Texture& t = s->textures[size_t(s->envTex)];
                float background = 0.0f;
                for (int y = 0; y < t.h; ++y) {
                    const float v = (static_cast<float>(y) + 0.5f) / static_cast<float>(t.h);
                    const float st = std::sin((1.0f - v) * kPi);
                    for (int x = 0; x < t.w; ++x) {
                        const float* p = &t.texels[3 * (size_t(y) * t.w + x)];
                        background += luminance(V3(p[0], p[1], p[2])) * st;
                    }
                }
                V3 lo(std::numeric_limits<float>::infinity()), hi(-std::numeric_limits<float>::infinity());
                auto grow = [&](const V3& q) {
                    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], q[k]); hi[k] = std::max(hi[k], q[k]); }
                };
                for (const Triangle& tr : s->tris) { grow(tr.a); grow(tr.b); grow(tr.c); }
                for (const Rectangle& r : s->rects) { grow(r.vA); grow(r.vB); grow(r.vC); grow(r.vD); }
                const V3 e = hi - lo;
                const float R = std::sqrt(e.x * e.x + e.y * e.y + e.z * e.z) * 0.5f;
                flux[i] = background * 12.566370614359172f * R * R;
            } else {
                const float f = luminance(L.radiance) * lightArea(*s, L) * kPi;
                flux[i] = f > 0.0f ? f : 1.0f;  // AreaLight::_defaultFlux (areaLight.cpp:30-32)
            }
        }
        // Distribution1D (distribution1D.cpp:10-41)
        std::vector<float>& cdf = s->lightCdf;
        cdf.assign(n + 1, 0.0f);
        const float delta = 1.0f / static_cast<float>(n);
        for (std::size_t i = 1; i <= n; ++i) cdf[i] = cdf[i - 1] + flux[i - 1] * delta;
        const float sum = cdf[n];
        if (sum > 0.0f) {
            const float inv = 1.0f / sum;
            for (std::size_t i = 1; i <= n; ++i) cdf[i] *= inv;
        } else {
            for (std::size_t i = 1; i <= n; ++i) cdf[i] = static_cast<float>(i) * delta;
        }
        cdf[n] = 1.0f;
    }
    std::vector<BuildItem> items(s->prims.size());
    for (std::size_t i = 0; i < s->prims.size(); ++i) {
        primBound(*s, static_cast<int>(i), &items[i].lo, &items[i].hi);
        items[i].c = (items[i].lo + items[i].hi) * 0.5f;
        items[i].idx = static_cast<int>(i);
    }
    if (!items.empty()) buildRec(*s, items, 0, static_cast<int>(items.size()));
    // camera
    const V3 pos = vload(d->cam_position), dir = vload(d->cam_direction), up = vload(d->cam_up);
    s->camPos = pos;
    s->camZ = (-dir).normalize();
    s->camX = up.cross(s->camZ).normalize();
    s->camY = s->camZ.cross(s->camX);
    const double sw = d->sensor_width_mm > 0 ? d->sensor_width_mm : 36.0;
    const double aspect = static_cast<double>(d->width) / static_cast<double>(d->height);
    const double sh = sw / aspect;
    const float halfFovRad = static_cast<float>(d->fov_degrees * 0.5) * 0.0174532925199432f;
    s->offset = static_cast<float>((sw * 0.5) / std::tan(halfFovRad));
    s->sx = static_cast<float>(sw / d->width);
    s->sy = static_cast<float>(-sh / d->height);
    s->tx = static_cast<float>(-(sw * 0.5));
    s->ty = static_cast<float>(sh * 0.5);
    return s.release();
}


// ------------------------------------------------------ FP64 gradient ----
// Reference gradient for the adjoint (which has no counterpart in the
// reference renderer): forward-mode dual numbers over an FP64 evaluation of
// the same estimator with detached sampling - every random decision, sampled
// direction, pdf, MIS weight and roulette probability is taken from the FP32
// path above (so paths are identical), while the BSDF values, albedo texels,
// GGX roughness and emitted radiance carry tangents.  d/dtheta of the path's
// FP64 radiance is then exactly the detached path derivative.
constexpr int kMaxTangents = 16;
struct Dual {
    double v = 0.0;
    double t[kMaxTangents] = {0};
};
struct DualParam { int kind; int index; int channel; };  // kind 0 texel float, 1 roughness, 2 radiance
int g_ntan = 0;
const DualParam* g_params = nullptr;

Dual dconst(double v) { Dual d; d.v = v; return d; }
Dual operator+(const Dual& a, const Dual& b) { Dual r; r.v = a.v + b.v; for (int i = 0; i < g_ntan; ++i) r.t[i] = a.t[i] + b.t[i]; return r; }
Dual operator-(const Dual& a, const Dual& b) { Dual r; r.v = a.v - b.v; for (int i = 0; i < g_ntan; ++i) r.t[i] = a.t[i] - b.t[i]; return r; }
Dual operator*(const Dual& a, const Dual& b) { Dual r; r.v = a.v * b.v; for (int i = 0; i < g_ntan; ++i) r.t[i] = a.t[i] * b.v + a.v * b.t[i]; return r; }
Dual operator*(const Dual& a, double s) { Dual r; r.v = a.v * s; for (int i = 0; i < g_ntan; ++i) r.t[i] = a.t[i] * s; return r; }
Dual operator/(const Dual& a, const Dual& b) { Dual r; r.v = a.v / b.v; for (int i = 0; i < g_ntan; ++i) r.t[i] = (a.t[i] * b.v - a.v * b.t[i]) / (b.v * b.v); return r; }
Dual dsqrt(const Dual& a) { Dual r; r.v = std::sqrt(a.v); for (int i = 0; i < g_ntan; ++i) r.t[i] = a.t[i] / (2.0 * r.v); return r; }
struct D3 { Dual c[3]; };
D3 d3(const V3& v) { D3 r; r.c[0] = dconst(v.x); r.c[1] = dconst(v.y); r.c[2] = dconst(v.z); return r; }
D3 operator*(const D3& a, const D3& b) { D3 r; for (int k = 0; k < 3; ++k) r.c[k] = a.c[k] * b.c[k]; return r; }
D3 operator*(const D3& a, const Dual& s) { D3 r; for (int k = 0; k < 3; ++k) r.c[k] = a.c[k] * s; return r; }
D3 operator*(const D3& a, double s) { D3 r; for (int k = 0; k < 3; ++k) r.c[k] = a.c[k] * s; return r; }
D3 operator+(const D3& a, const D3& b) { D3 r; for (int k = 0; k < 3; ++k) r.c[k] = a.c[k] + b.c[k]; return r; }

Dual param_value(int kind, int index, int channel, double v) {
    Dual d = dconst(v);
    for (int i = 0; i < g_ntan; ++i)
        if (g_params[i].kind == kind && g_params[i].index == index && g_params[i].channel == channel) d.t[i] = 1.0;
    return d;
}

D3 albedoDual(const Scene& s, const Material& m, const V3& uvw) {
    if (m.tex < 0) return d3(m.albedo);
    const Texture& t = s.textures[size_t(m.tex)];
    const float u = uvw.x - std::floor(uvw.x), v = uvw.y - std::floor(uvw.y);
    int x = static_cast<int>(u * t.w), y = static_cast<int>(v * t.h);
    x = x < t.w ? x : x - 1;
    y = y < t.h ? y : y - 1;
    int base = 0;
    for (int i = 0; i < m.tex; ++i) base += s.textures[size_t(i)].w * s.textures[size_t(i)].h * 3;
    const int off = base + 3 * (y * t.w + x);
    D3 r;
    for (int k = 0; k < 3; ++k) r.c[k] = param_value(0, off + k, 0, t.texels[size_t(3 * (y * t.w + x) + k)]);
    return r;
}

D3 radianceDual(const Scene& s, int li) {
    const V3& L = s.lights[size_t(li)].radiance;
    D3 r;
    for (int k = 0; k < 3; ++k) r.c[k] = param_value(2, li, k, L[k]);
    return r;
}

// GGX D * G with alpha(roughness) carrying tangents (isotropicGgx.cpp:11-69)
Dual ggxDG(const Scene& s, int mi, const Material& m, const V3& V, const V3& L, const V3& N, const V3& H) {
    const float NdotH = N.dot(H);
    if (NdotH <= 0.0f) return dconst(0.0);
    const float VdotH = V.dot(H), VdotN = V.dot(N), LdotH = L.dot(H), LdotN = L.dot(N);
    if (!((VdotH * VdotN > 0.0f) && (LdotH * LdotN > 0.0f))) return dconst(0.0);
    Dual r = param_value(1, mi, 0, m.roughness);
    Dual a;
    if (m.roughness > 0.001f && double(m.roughness) * m.roughness > 0.001) a = r * r;
    else a = dconst(roughnessToAlpha(m.roughness));
    const Dual a2 = a * a;
    const double c2 = double(NdotH) * NdotH, c4 = c2 * c2, tan2 = (1.0 - c2) / c2;
    const Dual q = a2 + dconst(tan2);
    const Dual D = a2 / (q * q * (kPi * c4));
    auto G1 = [&](double c) {
        const double cc = c * c;
        const double tv = (1.0 - cc) / cc;
        return dconst(2.0) / (dconst(1.0) + dsqrt(dconst(1.0) + a2 * tv));
    };
    return D * G1(VdotN) * G1(LdotN);
}

// BSDF value with tangents, at the same directions the FP32 path used
D3 bsdfDual(const Scene& s, int mi, const Surface& si, const V3& L) {
    const Material& m = s.mats[size_t(mi)];
    const V3& N = si.Ns;
    const V3& V = si.wi;
    if (m.type == CGPU_BSDF_LAMBERTIAN) {
        if (V.dot(N) * L.dot(N) <= 0.0f) return d3(V3(0.0f));
        return albedoDual(s, m, si.uvw) * (1.0 / kPi);
    }
    if (m.type == CGPU_BSDF_CONDUCTOR_GGX) {
        const float VdotN = V.dot(N), LdotN = L.dot(N);
        if (VdotN * LdotN <= 0.0f) return d3(V3(0.0f));
        const float sgn = static_cast<float>((0.0f < VdotN) - (VdotN < 0.0f));
        V3 H = (V + L) * sgn;
        if (H.isZero()) return d3(V3(0.0f));
        H = H.normalize();
        const V3 F = schlick(m.f0, L.dot(H));
        return d3(F) * (ggxDG(s, mi, m, V, L, N, H) * (1.0 / (4.0 * std::abs(double(VdotN) * LdotN))));
    }
    if (m.type == CGPU_BSDF_DIELECTRIC_GGX) {
        // the FP32 value of the path, times d ln(D G) / d theta: roughness
        // enters the Walter et al. BRDF / BTDF only through D and G, at the
        // reflection or refraction half vector of roughDielectric
        V3 f;
        float pdf;
        roughDielectric(m, albedoAt(m, si.uvw), V, L, N, &f, &pdf);
        if (f.isZero()) return d3(V3(0.0f));
        const float cv = V.dot(N), cl = L.dot(N);
        const V3 Nv = cv > 0.0f ? N : -N;
        V3 H;
        if (cv * cl > 0.0f) {
            H = (V + L).normalize();
        } else {
            const float etaV = cv > 0.0f ? m.iorOuter : m.iorInner;
            const float etaL = cv > 0.0f ? m.iorInner : m.iorOuter;
            H = (V + L * (etaL / etaV)).normalize();
            if (H.dot(Nv) < 0.0f) H = -H;
        }
        const Dual dg = ggxDG(s, mi, m, V, L, Nv, H);
        if (dg.v == 0.0) return d3(f);
        return d3(f) * (dg * (1.0 / dg.v));
    }
    return d3(bsdfEval(m, si, L));  // no differentiable parameter of this BSDF here
}

D3 estimateDual(const Scene& s, Ray ray, Rng& rng) {
    D3 L = d3(V3(0.0f)), T = d3(V3(1.0f));
    V3 Tf(1.0f);
    bool countEmission = true;
    for (int bounce = 0; bounce < s.maxDepth; ++bounce) {
        Surface si;
        if (!intersect(s, ray, &si)) break;
        const Prim& pr = s.prims[si.prim];
        const Material& m = s.mats[pr.material];
        if (pr.light >= 0 && countEmission && canEmit(s.lights[pr.light], si.wi, si.Ns))
            L = L + T * radianceDual(s, pr.light);
        if (!isSpecular(m.type)) {
            countEmission = false;
            float pickf;
            const std::size_t li = pickLight(s, rng, &pickf);
            const double pick = s.lightCdf.empty() ? 1.0 / double(s.lights.size()) : double(pickf);
            if (m.type != CGPU_BSDF_ABSORBER) {
                const Light& l = s.lights[li];
                const LightSample ls = lightSample(s, l, si.P, rng);
                if (ls.valid()) {
                    const V3 Lv = ls.pos - si.P;
                    const float dist = Lv.length();
                    const V3 Ld = Lv / dist;
                    Ray shadow;
                    shadow.o = si.P;
                    shadow.d = Ld.normalize();
                    shadow.maxT = dist - kRayEps;
                    if (!occluded(s, shadow)) {
                        const float w = misPower(ls.pdfW, bsdfPdf(m, si, Ld));
                        const D3 f = bsdfDual(s, pr.material, si, Ld);
                        L = L + T * (radianceDual(s, int(li)) * f * (double(w) * Ld.absDot(si.Ns) / ls.pdfW / pick));
                    }
                }
                const BsdfSample bs = bsdfSample(m, si, rng);
                if (bs.valid()) {
                    Ray r;
                    r.o = si.P;
                    r.d = bs.L.normalize();
                    Surface hit;
                    if (intersect(s, r, &hit) && s.prims[hit.prim].light == int(li)) {
                        const Light& hl = s.lights[li];
                        if (canEmit(hl, hit.wi, hit.Ns)) {
                            const float lp = lightPdfW(s, hl, hit, si.P);
                            const float w = misPower(bs.pdf, lp);
                            const D3 f = bsdfDual(s, pr.material, si, bs.L);
                            L = L + T * (radianceDual(s, int(li)) * f * (double(w) * bs.L.absDot(si.Ns) / bs.pdf / pick));
                        }
                    }
                }
            }
        } else {
            countEmission = true;
        }
        const BsdfSample bs = bsdfSample(m, si, rng);
        if (!bs.valid()) break;
        const float LdotN = bs.L.absDot(si.Ns);
        Tf *= bs.f * LdotN / bs.pdf;
        if (m.type == CGPU_BSDF_LAMBERTIAN || m.type == CGPU_BSDF_CONDUCTOR_GGX || m.type == CGPU_BSDF_DIELECTRIC_GGX)
            T = T * (bsdfDual(s, pr.material, si, bs.L) * (double(LdotN) / bs.pdf));
        else
            T = T * d3(bs.f * LdotN / bs.pdf);
        if (bounce > 2) {
            const float q = std::min(std::max(1.0f - Tf.maxComponent(), 0.05f), 1.0f);
            const float u = rng.next();
            if (u > q) {
                Tf = Tf * (1.0f / (1.0f - q));
                T = T * (1.0 / (1.0 - double(q)));
            } else {
                break;
            }
        }
        if (Tf.isZero()) break;
        ray = Ray();
        ray.o = si.P;
        ray.d = bs.L.normalize();
    }
    return L;
}

}  // namespace port

// ---------------------------------------------------------- film filters --
// Filters (core/film/filter/*.cpp) and FilmTile::addSample
// (core/film/filmTile.cpp:36-66) restated: the filter constants as the
// constructors compute them, the footprint clipped to the tile of the
// sample's own pixel (Film::getTileBound, core/film/film.cpp:204-211).
struct FilmFilter {
    int type = CGPU_FILTER_BOX;
    float hx = 0.5f, hy = 0.5f;
    float expX = 0.0f, expY = 0.0f, edge = 0.0f, amp = 1.0f;  // gaussianFilter.cpp:9-25
    float b = 0.0f, c = 0.0f;                                 // mitchellFilter.cpp:7-15
    int tw = 16, th = 16;
};

FilmFilter makeFilmFilter(const cgpu_film_filter& f) {
    FilmFilter F;
    F.type = f.type;
    float w = f.width, h = f.height;
    if (f.type == CGPU_FILTER_BOX) {
        if (w == 0.0f) w = 1.0f;
        if (h == 0.0f) h = 1.0f;
    }
    F.hx = w / 2.0f;  // Filter::filterHalfSize (filter.cpp:19-21)
    F.hy = h / 2.0f;
    F.tw = f.tile_width ? f.tile_width : 16;
    F.th = f.tile_height ? f.tile_height : 16;
    if (f.type == CGPU_FILTER_GAUSSIAN) {
        F.expX = -1.0f / (2.0f * f.sigma_x * f.sigma_x);
        F.expY = -1.0f / (2.0f * f.sigma_y * f.sigma_y);
        F.amp = f.amplitude;
        F.edge = F.amp * std::exp(F.expX * F.hx * F.hx + F.expY * F.hy * F.hy);
    }
    F.b = f.b;
    F.c = f.c;
    return F;
}

float mitchell1D(const FilmFilter& F, float d) {  // mitchellFilter.cpp:21-42
    const float a = std::fabs(d);
    const float den = 1.0f / 6.0f;
    if (a < 1.0f) return ((12.0f - 9.0f * F.b - 6.0f * F.c) * a * a * a + (-18.0f + 12.0f * F.b + 6.0f * F.c) * a * a +
                          (6.0f - 2.0f * F.b)) * den;
    if (a < 2.0f) return ((-F.b - 6.0f * F.c) * a * a * a + (6.0f * F.b + 30.0f * F.c) * a * a +
                          (-12.0f * F.b - 48.0f * F.c) * a + (8.0f * F.b + 24.0f * F.c)) * den;
    return 0.0f;
}

float filterEval(const FilmFilter& F, float x, float y) {
    switch (F.type) {
        case CGPU_FILTER_GAUSSIAN: {  // gaussianFilter.cpp:27-32
            const float v = F.amp * std::exp(F.expX * x * x + F.expY * y * y);
            return std::max(0.0f, v - F.edge);
        }
        case CGPU_FILTER_MITCHELL: return mitchell1D(F, x) * mitchell1D(F, y);  // mitchellFilter.cpp:17-19
        case CGPU_FILTER_CONE:  // coneFilter.cpp:11-15
            return std::max(F.hx - std::fabs(x), 0.0f) * std::max(F.hy - std::fabs(y), 0.0f);
        default: return 1.0f;  // boxFilter.cpp:9-11
    }
}

// One sample into an H x W x 7 FP64 film {sum w r,g,b; sum w r^2,g^2,b^2; sum w}.
void filterSplat(const FilmFilter& F, int W, int H, float x, float y, const float* rgb, double* film) {
    if (!(std::isfinite(rgb[0]) && std::isfinite(rgb[1]) && std::isfinite(rgb[2]))) return;  // filmTile.cpp:21-28
    const int ix = static_cast<int>(std::floor(x)), iy = static_cast<int>(std::floor(y));
    const int tx0 = ix / F.tw * F.tw, ty0 = iy / F.th * F.th;
    const int tx1 = std::min(tx0 + F.tw, W), ty1 = std::min(ty0 + F.th, H);
    const float minX = std::max(x - F.hx, static_cast<float>(tx0)), minY = std::max(y - F.hy, static_cast<float>(ty0));
    const float maxX = std::min(x + F.hx, static_cast<float>(tx1)), maxY = std::min(y + F.hy, static_cast<float>(ty1));
    const int x0 = static_cast<int>(std::ceil(minX - 0.5f)), y0 = static_cast<int>(std::ceil(minY - 0.5f));
    const int x1 = static_cast<int>(std::floor(maxX - 0.5f) + 1), y1 = static_cast<int>(std::floor(maxY - 0.5f) + 1);
    for (int py = y0; py < y1; ++py)
        for (int px = x0; px < x1; ++px) {
            const float w = filterEval(F, px - (x - 0.5f), py - (y - 0.5f));
            double* o = film + 7 * static_cast<std::size_t>(py * W + px);
            for (int k = 0; k < 3; ++k) {
                o[k] += static_cast<double>(rgb[k] * w);
                o[3 + k] += static_cast<double>(w) * rgb[k] * rgb[k];
            }
            o[6] += w;
        }
}

extern "C" {

// n samples {x, y} / {r, g, b} in the given order into `film` (H x W x 7).
void port_filter_splat(const cgpu_film_filter* f, int32_t W, int32_t H, uint64_t n, const float* xy, const float* rgb,
                       double* film) {
    const FilmFilter F = makeFilmFilter(*f);
    for (uint64_t i = 0; i < n; ++i) filterSplat(F, W, H, xy[2 * i], xy[2 * i + 1], rgb + 3 * i, film);
}

// Film positions of samples [first, first + count) of every pixel, sample-major
// (count x H x W x 2): pixel + the stratified jitter of the path stream.
void port_sample_positions(void* sp, uint64_t seed, uint32_t scene_index, uint32_t first, uint32_t count, float* xy) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    for (uint32_t k = 0; k < count; ++k)
        for (int iy = 0; iy < s.H; ++iy)
            for (int ix = 0; ix < s.W; ++ix) {
                const uint32_t pixel = static_cast<uint32_t>(iy * s.W + ix);
                port::Rng rng;
                rng.s.key = oracle_rng::path_key(seed, scene_index, pixel, first + k);
                rng.s.counter = 0;
                float jx, jy;
                port::jitter(s.spp, first + k, rng, &jx, &jy);
                float* o = xy + 2 * (static_cast<std::size_t>(k) * s.W * s.H + pixel);
                o[0] = static_cast<float>(ix) + jx;
                o[1] = static_cast<float>(iy) + jy;
            }
}

void* port_scene_create(const cgpu_scene_desc* desc) { return port::create(desc); }
void port_scene_destroy(void* s) { delete static_cast<port::Scene*>(s); }
int port_num_bvh_nodes(void* s) { return static_cast<int>(static_cast<port::Scene*>(s)->nodes.size()); }

void port_camera_rays(void* sp, const double* xy, uint32_t n, float* out) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    for (uint32_t i = 0; i < n; ++i) {
        const port::Ray r = port::cameraRay(s, xy[2 * i], xy[2 * i + 1]);
        float* o = out + 6 * static_cast<std::size_t>(i);
        o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z; o[3] = r.d.x; o[4] = r.d.y; o[5] = r.d.z;
    }
}

// For each primitive and direction octant o (bit k: direction component k
// negative), its position in the leaf order of this tree's traversal
// (traverse: the second child first on a node whose split axis the ray
// runs down), 8 per primitive.  Of two primitives hit at the same distance
// the traversal keeps the later one.
void port_visit_ranks(void* sp, uint32_t* out) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    if (s.nodes.empty()) return;
    for (int o = 0; o < 8; ++o) {
        uint32_t pos = 0;
        std::vector<int> stack{0};
        while (!stack.empty()) {
            const int cur = stack.back();
            stack.pop_back();
            const port::Scene::Node& n = s.nodes[static_cast<std::size_t>(cur)];
            if (n.second < 0) {
                for (int i = 0; i < n.count; ++i) out[8 * static_cast<std::size_t>(s.order[n.prim + i]) + o] = pos++;
                continue;
            }
            const bool secondFirst = ((o >> n.axis) & 1) != 0;
            stack.push_back(secondFirst ? cur + 1 : n.second);
            stack.push_back(secondFirst ? n.second : cur + 1);
        }
    }
}

// rays: 8 floats each (org, t_min, dir, t_max)
void port_trace(void* sp, const float* rays, uint32_t n, int32_t* prim, float* t, int32_t* occ) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 8 * static_cast<std::size_t>(i);
        port::Ray ray;
        ray.o = port::V3(r[0], r[1], r[2]);
        ray.d = port::V3(r[4], r[5], r[6]).normalize();  // Ray ctor normalises (ray.cpp:19-30)
        ray.minT = r[3];
        ray.maxT = r[7];
        port::Ray a = ray;
        const int p = port::traverse(s, a, false);
        prim[i] = p;
        t[i] = p >= 0 ? a.maxT : 0.0f;
        if (occ) occ[i] = port::occluded(s, ray) ? 1 : 0;
    }
}

void port_paths(void* sp, const double* xy, const uint64_t* keys, uint32_t n, float* rgb, uint32_t* draws) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    port::g_scene = &s;
    for (uint32_t i = 0; i < n; ++i) {
        port::Rng rng;
        rng.s.key = keys[i];
        rng.s.counter = 0;
        const port::Ray r = port::cameraRay(s, xy[2 * i], xy[2 * i + 1]);
        const port::V3 L = port::estimate(s, r, rng);
        rgb[3 * i] = L.x; rgb[3 * i + 1] = L.y; rgb[3 * i + 2] = L.z;
        if (draws) draws[i] = rng.s.counter;
    }
}

// Renders samples [first, first + count) of rows [row0, row1) with `threads`
// host threads.  film: W*H*7 doubles (sum rgb, sum sq rgb, accepted count);
// path_rgb (optional): count*W*H*3 floats, sample-major.
void port_render(void* sp, uint64_t seed, uint32_t scene_index, uint32_t first, uint32_t count,
                 int32_t row0, int32_t row1, int32_t threads, double* film, float* path_rgb) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    port::g_scene = &s;
    std::atomic<int> next{row0};
    auto worker = [&]() {
        for (;;) {
            const int iy = next.fetch_add(1);
            if (iy >= row1) break;
            for (int ix = 0; ix < s.W; ++ix) {
                const uint32_t pixel = static_cast<uint32_t>(iy * s.W + ix);
                for (uint32_t k = 0; k < count; ++k) {
                    const uint32_t si = first + k;
                    port::Rng rng;
                    rng.s.key = oracle_rng::path_key(seed, scene_index, pixel, si);
                    rng.s.counter = 0;
                    float jx, jy;
                    port::jitter(s.spp, si, rng, &jx, &jy);
                    const float fx = static_cast<float>(ix) + jx, fy = static_cast<float>(iy) + jy;
                    const port::Ray r = port::cameraRay(s, fx, fy);
                    const port::V3 L = port::estimate(s, r, rng);
                    if (path_rgb) {
                        float* o = path_rgb + 3 * (static_cast<std::size_t>(k) * s.W * s.H + pixel);
                        o[0] = L.x; o[1] = L.y; o[2] = L.z;
                    }
                    if (film && L.finite()) {  // filmTile.cpp:21-28 drops NaN / Inf samples
                        double* px = film + 7 * static_cast<std::size_t>(pixel);
                        px[0] += L.x; px[1] += L.y; px[2] += L.z;
                        px[3] += static_cast<double>(L.x) * L.x;
                        px[4] += static_cast<double>(L.y) * L.y;
                        px[5] += static_cast<double>(L.z) * L.z;
                        px[6] += 1.0;
                    }
                }
            }
        }
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
    }
}


// FP64 reference gradient of loss = sum_pixels dLdI . image over samples
// [0, spp) (paths keyed like the CUDA renderer): params = K (kind, index,
// channel) triples, kind 0 = texel float (index into the concatenated
// textures), 1 = roughness of material `index`, 2 = radiance of light
// `index` channel `channel`; grad: K doubles.
void port_adjoint_fp64(void* sp, uint64_t seed, uint32_t scene_index, uint32_t spp, const float* dLdI,
                       const int32_t* params, int32_t K, int32_t threads, double* grad) {
    const port::Scene& s = *static_cast<port::Scene*>(sp);
    port::g_scene = &s;
    std::vector<port::DualParam> ps(static_cast<size_t>(K));
    for (int i = 0; i < K; ++i) ps[size_t(i)] = port::DualParam{params[3 * i], params[3 * i + 1], params[3 * i + 2]};
    port::g_params = ps.data();
    port::g_ntan = K;
    std::vector<std::vector<double>> acc(static_cast<size_t>(std::max(threads, 1)), std::vector<double>(size_t(K), 0.0));
    std::atomic<int> next{0};
    auto worker = [&](int tid) {
        for (;;) {
            const int iy = next.fetch_add(1);
            if (iy >= s.H) break;
            for (int ix = 0; ix < s.W; ++ix) {
                const uint32_t pixel = static_cast<uint32_t>(iy * s.W + ix);
                const float* d = dLdI + 3 * size_t(pixel);
                if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) continue;
                for (uint32_t si = 0; si < spp; ++si) {
                    port::Rng rng;
                    rng.s.key = oracle_rng::path_key(seed, scene_index, pixel, si);
                    rng.s.counter = 0;
                    float jx, jy;
                    port::jitter(s.spp, si, rng, &jx, &jy);
                    const port::Ray r = port::cameraRay(s, static_cast<float>(ix) + jx, static_cast<float>(iy) + jy);
                    const port::D3 L = port::estimateDual(s, r, rng);
                    if (!(std::isfinite(L.c[0].v) && std::isfinite(L.c[1].v) && std::isfinite(L.c[2].v))) continue;
                    for (int k = 0; k < 3; ++k)
                        for (int i = 0; i < K; ++i) acc[size_t(tid)][size_t(i)] += double(d[k]) / spp * L.c[k].t[i];
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < std::max(threads, 1); ++t) pool.emplace_back(worker, t);
    for (auto& t : pool) t.join();
    for (int i = 0; i < K; ++i) {
        grad[i] = 0.0;
        for (auto& a : acc) grad[i] += a[size_t(i)];
    }
}

}  // extern "C"
