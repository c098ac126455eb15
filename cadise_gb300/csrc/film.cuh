// Film reconstruction filters and the reference's sample footprint.
//
// The footprint and weights follow FilmTile::addSample
// (source/core/film/filmTile.cpp:36-66) in FP32: a sample at film position
// (px, py) reaches the pixels [ceil(max(px - hx, tile x0) - 1/2),
// floor(min(px + hx, tile x1) - 1/2) + 1) (and the same in y) of the tile its
// own pixel lies in, with weight filter(ix - (px - 1/2), iy - (py - 1/2)).
// Filters: box (boxFilter.cpp:9-11), Gaussian (gaussianFilter.cpp:27-32),
// Mitchell-Netravali (Mitchell & Netravali, "Reconstruction Filters in
// Computer Graphics", SIGGRAPH 1988; mitchellFilter.cpp:17-42), cone
// (coneFilter.cpp:11-15).
#pragma once

#include "../../include/cadise_gpu.h"
#include "common.cuh"
#include "scene_device.cuh"

namespace cg {

CG_HD float mitchell_1d(float b, float c, float d) {
    const float x = fabsf(d);
    const float sixth = 1.0f / 6.0f;
    if (x < 1.0f)
        return ((12.0f - 9.0f * b - 6.0f * c) * x * x * x + (-18.0f + 12.0f * b + 6.0f * c) * x * x + (6.0f - 2.0f * b)) *
               sixth;
    if (x < 2.0f)
        return ((-b - 6.0f * c) * x * x * x + (6.0f * b + 30.0f * c) * x * x + (-12.0f * b - 48.0f * c) * x +
                (8.0f * b + 24.0f * c)) *
               sixth;
    return 0.0f;
}

CG_HD float filter_weight(const FilterD& F, float x, float y) {
    switch (F.type) {
        case CGPU_FILTER_GAUSSIAN: {
            const float v = F.p3 * expf(F.p0 * x * x + F.p1 * y * y);
            return fmaxf(0.0f, v - F.p2);
        }
        case CGPU_FILTER_MITCHELL: return mitchell_1d(F.p0, F.p1, x) * mitchell_1d(F.p0, F.p1, y);
        case CGPU_FILTER_CONE: return fmaxf(F.hx - fabsf(x), 0.0f) * fmaxf(F.hy - fabsf(y), 0.0f);
        default: return 1.0f;
    }
}

// Pixel range [*a, *b) one axis of a sample's footprint covers, clipped to
// the tile [t0, t1).
CG_HD void footprint_1d(float p, float half, int t0, int t1, int* a, int* b) {
    const float lo = fmaxf(p - half, float(t0));
    const float hi = fminf(p + half, float(t1));
    *a = int(ceilf(lo - 0.5f));
    *b = int(floorf(hi - 0.5f) + 1.0f);
}

// How far (in pixels) a sample's footprint can reach from its own pixel, with
// one pixel of margin for the rounding of the bounds.
CG_HD int footprint_reach(float half) { return int(ceilf(half + 0.5f)) + 1; }

// Gather form of the footprint rule, for one pixel (ix, iy) of a W x H film:
// the samples of the pixels of its own tile whose footprint covers it, in a
// fixed order (source rows, source pixels, samples).  fetch(k, sx, sy, &v,
// &pos) gives sample k of pixel (sx, sy) and returns false for a sample the
// film drops (NaN / Inf).  Adds sum w v, sum w v^2 and sum w.
template <class Fetch>
CG_HD void filter_gather(const FilterD& F, int W, int H, int ix, int iy, uint32_t nsamples, Fetch&& fetch, double* s,
                         double* q, double* n) {
    const int tx0 = ix / F.tile_w * F.tile_w, ty0 = iy / F.tile_h * F.tile_h;
    const int tx1 = min(tx0 + F.tile_w, W), ty1 = min(ty0 + F.tile_h, H);
    const int rx = footprint_reach(F.hx), ry = footprint_reach(F.hy);
    const int sx0 = max(tx0, ix - rx), sx1 = min(tx1 - 1, ix + rx);
    const int sy0 = max(ty0, iy - ry), sy1 = min(ty1 - 1, iy + ry);
    for (int sy = sy0; sy <= sy1; ++sy)
        for (int sx = sx0; sx <= sx1; ++sx)
            for (uint32_t k = 0; k < nsamples; ++k) {
                float3 v;
                float2 pos;
                if (!fetch(k, sx, sy, &v, &pos)) continue;
                int xa, xb, ya, yb;
                footprint_1d(pos.x, F.hx, tx0, tx1, &xa, &xb);
                footprint_1d(pos.y, F.hy, ty0, ty1, &ya, &yb);
                if (ix < xa || ix >= xb || iy < ya || iy >= yb) continue;
                const float w = filter_weight(F, float(ix) - (pos.x - 0.5f), float(iy) - (pos.y - 0.5f));
                s[0] += double(v.x * w);
                s[1] += double(v.y * w);
                s[2] += double(v.z * w);
                q[0] += double(w) * v.x * v.x;
                q[1] += double(w) * v.y * v.y;
                q[2] += double(w) * v.z * v.z;
                *n += double(w);
            }
}

}  // namespace cg
