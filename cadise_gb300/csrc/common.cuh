// Device math, the per-path random stream and small helpers shared by every
// kernel of the library.  FP32 throughout (the reference's `real` is float,
// source/math/type/fundamentalType.h:20).
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#ifndef __CUDACC__
// Host compilation of the device headers (the CPU check of the kernel logic
// in tests/native/ and the host-side scene build): plain C++ stand-ins for
// the CUDA intrinsics these headers use, with the same arithmetic meaning.
#include <algorithm>
#include <cstring>
using std::fabs;
using std::isfinite;
using std::sqrt;
inline float fabsf(float x) { return std::fabs(x); }
inline float sqrtf(float x) { return std::sqrt(x); }
template <typename T>
inline T __ldg(const T* p) { return *p; }
inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
inline int __float_as_int(float f) { int u; std::memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float __int_as_float(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline void sincospif(float x, float* s, float* c) {
    const double a = 3.14159265358979323846 * double(x);
    *s = float(std::sin(a));
    *c = float(std::cos(a));
}
using std::max;
using std::min;
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) { unsigned long long o = *p; *p += v; return o; }
inline unsigned atomicAdd(unsigned* p, unsigned v) { unsigned o = *p; *p += v; return o; }
inline double atomicAdd(double* p, double v) { double o = *p; *p += v; return o; }
// one thread is a whole warp on the host
inline unsigned __activemask() { return 1u; }
inline int __any_sync(unsigned, int pred) { return pred; }
#endif

#define CG_HD __host__ __device__ __forceinline__
#define CG_D __device__ __forceinline__

namespace cg {

// ------------------------------------------------------------ float3 ops --
CG_HD float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
CG_HD float3 splat3(float s) { return make_float3(s, s, s); }
CG_HD float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
CG_HD float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
CG_HD float3 operator-(float3 a) { return mk(-a.x, -a.y, -a.z); }
CG_HD float3 operator*(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
CG_HD float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
CG_HD float3 operator*(float s, float3 a) { return mk(a.x * s, a.y * s, a.z * s); }
CG_HD float3& operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
CG_HD float3& operator*=(float3& a, float3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; return a; }
CG_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CG_HD float absdot(float3 a, float3 b) { return fabsf(dot(a, b)); }
CG_HD float3 cross(float3 a, float3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
CG_HD float len2(float3 a) { return dot(a, a); }
CG_HD float len(float3 a) { return sqrtf(len2(a)); }
// scalar division and normalisation multiply by the reciprocal, as the
// reference's TVector does (source/math/tVector.ipp:103-111, 346-351)
CG_HD float3 divs(float3 a, float s) { const float inv = 1.0f / s; return a * inv; }
CG_HD float3 normalize(float3 a) { return a * (1.0f / len(a)); }
CG_HD bool is_zero(float3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
CG_HD float max_comp(float3 a) { float m = a.x; if (a.y > m) m = a.y; if (a.z > m) m = a.z; return m; }
CG_HD float sum3(float3 a) { return a.x + a.y + a.z; }
CG_HD bool finite3(float3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
CG_HD float comp(float3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
CG_HD float3 f3(float4 a) { return mk(a.x, a.y, a.z); }
// V.reflect(N) = 2 |V.N| N - V   (tVector.ipp:462-465)
CG_HD float3 reflect(float3 v, float3 n) { return n * (2.0f * absdot(v, n)) - v; }

constexpr float kPi = 3.1415926535897932f;
constexpr float kInvPi = 0.3183098861837906f;
constexpr float kRayEps = 0.001f;       // constant::ray_epsilon (math/constant.h:9-11)
constexpr float kFloatMax = 3.402823466e+38f;

// Orthonormal frame with `y` as the up axis (source/math/math.cpp:36-58).
CG_HD void frame_from_y(float3 y, float3* z, float3* x) {
    float3 zz;
    if (fabsf(y.x) > fabsf(y.y)) {
        zz = mk(-y.z, 0.0f, y.x) * (1.0f / sqrtf(y.x * y.x + y.z * y.z));
    } else {
        zz = mk(0.0f, y.z, -y.y) * (1.0f / sqrtf(y.y * y.y + y.z * y.z));
    }
    *z = zz;
    *x = cross(y, zz);
}

// ------------------------------------------------------------ path stream --
// SplitMix64 (Steele, Lea & Flood 2014) seeded with a per-path key: draw i is
// finalize(key + (i + 1) * golden_gamma); the top 24 bits give a float in
// [0, 1).  A path is replayed exactly from (seed, scene, pixel, sample).
CG_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
CG_HD uint64_t path_key(uint64_t seed, uint32_t scene, uint32_t pixel, uint32_t sample) {
    const uint64_t s = mix64(seed ^ (0xD1B54A32D192ED03ull * (uint64_t(scene) + 1)));
    return mix64(s ^ ((uint64_t(sample) << 32) | uint64_t(pixel)));
}

struct Rng {
    uint64_t key;
    uint32_t ctr;
    CG_HD float next() {
        const uint64_t x = mix64(key + (uint64_t(ctr) + 1) * 0x9E3779B97F4A7C15ull);
        ++ctr;
        return float(uint32_t(x >> 40)) * (1.0f / 16777216.0f);
    }
    // The reference fills its 2-D samples as Vector2R(nextReal(), nextReal())
    // and GCC evaluates those arguments right to left: the first draw lands
    // in .y.  Same order here so a path consumes its stream identically.
    CG_HD void next2(float* x, float* y) { *y = next(); *x = next(); }
    // Random::nextIndex(lo, hi) of source/math/random.cpp:21-26
    CG_HD int index(int n) {
        const int i = int(0.0f + next() * float(n));
        return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    }
};

// -------------------------------------------------------- warp helpers ----
#ifdef __CUDACC__
// Warp-aggregated append: one atomicAdd per warp; returns this lane's slot.
CG_D int warp_append(int* counter, bool want) {
    const unsigned mask = __activemask();
    const unsigned ballot = __ballot_sync(mask, want);
    if (ballot == 0) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return want ? base + __popc(ballot & ((1u << lane) - 1u)) : -1;
}
#endif

}  // namespace cg
