// Reference harness: drives the reference renderer's OWN object files.
//
// Test infrastructure only.  oracle/Makefile compiles every reference source
// except source/cadise/cadise.cpp (its main) and source/math/random.cpp (its
// RNG) and links them with this file.  Nothing here re-implements reference
// behaviour; it loads a CRSD scene through the reference's own tokenizer and
// factories and calls:
//
//   Camera::spawnPrimaryRay        core/camera/perspectivePinholeCamera.cpp:52-73
//   Accelerator::isIntersecting    core/intersector/accelerator/bvh/bvhAccelerator.cpp:40-97
//   Accelerator::isOccluded        core/intersector/accelerator/bvh/bvhAccelerator.cpp:99-156
//   BruteForceAccelerator          core/intersector/accelerator/bruteForceAccelerator.cpp:26-43
//   EnergyEstimator::estimate      core/estimator/ptEstimator.cpp:25-123
//   Sampler::requestSample2D       core/sampler/category/stratifiedSampler.cpp:38-73
//
// cadise::Random (source/math/random.h) is interposed with the seeded
// per-path stream of oracle_rng.h so that a render is reproducible.
//
// Commands (binary little-endian I/O, see tests/golden/make_golden.py):
//   camera <scene.crsd> <in: N x {f64 fx, f64 fy}>           <out: N x 6 f32 (o, d)>
//   trace  <scene.crsd> <in: N x 8 f32 {o, tmin, d, tmax}>    <out: N x {i32 bvh_prim, f32 bvh_t, i32 bf_prim, f32 bf_t, i32 occluded}>
//   trace-bvh  the same without the brute-force query (bf_prim / bf_t repeat
//          the BVH's answer), for scenes too large for a brute-force loop
//   texel  <scene.crsd> <texture name> <in: N x 3 f32 uvw>    <out: N x 3 f32 rgb>
//          RgbImageTexture::evaluate (core/texture/category/rgbImageTexture.cpp:8-15)
//   paths  <scene.crsd> <in: N x {f64 fx, f64 fy, u64 key}>   <out: N x {f32 r, g, b, u32 draws}>
//   render <scene.crsd> <out: H x W x 7 f64> <spp> <seed> <threads>
//          (sum r,g,b, sum of squares r,g,b, accepted sample count)
//   filmtile <scene.crsd> <in: N x {f32 x, f32 y, f32 r, g, b}> <out: H x W x 4 f64>
//          the scene's film filter through FilmTile::addSample
//          (core/film/filmTile.cpp:36-66) on the 16 x 16 (tile-size-x/y) tiles
//          of Film::getTileBound (core/film/film.cpp:204-211): per pixel the
//          sensor's sum of w r, w g, w b and sum of w
//   render-tiles <scene.crsd> <out: H x W x 7 f64> <spp> <seed> <threads>
//          the render loop above with the scene's film filter: every pass of up
//          to 256 samples per pixel goes through a fresh FilmTile per tile, whose
//          sensors are then added in FP64 (sum w r,g,b, zeros, sum w)
//
// Image textures: the reference reads pictures through stb
// (file-io/pictureLoader.cpp), which has no float RGB format.  A
// texture-spectrum block of type "image" whose filename ends in .pfm is built
// here in memory instead - the reference's own TImage and RgbImageTexture
// (core/texture/category/tImageTexture.ipp:11-27) with the block's sample and
// wrap modes - from the PFM's rows in file order, so that row 0 is the
// picture's bottom row, as the reference's loader lays out every picture
// (stbi_set_flip_vertically_on_load: uv starts at the lower-left corner).

#include "core/camera/camera.h"
#include "core/estimator/energyEstimator.h"
#include "core/film/film.h"
#include "core/film/filmTile.h"
#include "core/film/filter/filter.h"
#include "core/film/rgbRadianceSensor.h"
#include "core/instantiator/instantiator.h"
#include "core/intersector/accelerator/accelerator.h"
#include "core/intersector/accelerator/bruteForceAccelerator.h"
#include "core/intersector/intersector.h"
#include "core/intersector/primitive/primitive.h"
#include "core/intersector/primitiveInfo.h"
#include "core/light/cluster/lightCluster.h"
#include "core/light/light.h"
#include "core/ray.h"
#include "core/sampler/sampleRecord2D.h"
#include "core/sampler/sampler.h"
#include "core/scene.h"
#include "core/spectrum/spectrum.h"
#include "core/surface/bsdf/bsdf.h"
#include "core/texture/tTexture.h"
#include "core/texture/category/rgbImageTexture.h"
#include "core/texture/eTextureSampleMode.h"
#include "core/texture/eTextureWrapMode.h"
#include "math/type/imageType.h"
#include "file-io/scene-description/eSdClassType.h"
#include "file-io/scene-description/sdData.h"
#include "file-io/scene-description/tokenizer.h"
#include "math/random.h"
#include "math/type/mapType.h"

#include "oracle_rng.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace cadise {

static thread_local oracle_rng::Stream g_stream;

// Interposed: same signature as source/math/random.h.
real Random::nextReal() { return g_stream.next(); }

// Interposed: the index formula of source/math/random.cpp:21-26 over the
// interposed stream (min + u * (max - min), clamped into [min, max - 1]).
std::size_t Random::nextIndex(const std::size_t minIndex, const std::size_t maxIndex) {
    const std::size_t interval = maxIndex - minIndex;
    const std::size_t idx = static_cast<std::size_t>(minIndex + nextReal() * interval);
    if (idx < minIndex) return minIndex;
    if (idx > maxIndex - 1) return maxIndex - 1;
    return idx;
}

}  // namespace cadise

using namespace cadise;

namespace {

struct LoadedScene {
    std::string text;  // SdData keeps string_views into this buffer
    std::vector<std::shared_ptr<SdData>> blocks;
    std::shared_ptr<SdData> film, camera, renderer, accel, cluster;
    StringKeyMap<TTexture<real>> realTextures;
    StringKeyMap<TTexture<Spectrum>> spectrumTextures;
    StringKeyMap<Bsdf> bsdfs;
    StringKeyMap<Primitive> primitives;
    std::vector<std::shared_ptr<Intersector>> intersectors;
    std::vector<std::shared_ptr<Light>> lights;
    std::shared_ptr<Primitive> background;
    std::shared_ptr<Accelerator> accelerator;
    std::shared_ptr<Accelerator> bruteForce;
    std::shared_ptr<LightCluster> lightCluster;
    std::shared_ptr<Scene> scene;
    std::shared_ptr<Camera> cam;
    std::shared_ptr<EnergyEstimator> estimator;
    std::shared_ptr<Sampler> sampler;
    std::map<const void*, int> primIndex;  // Primitive* -> CRSD creation order
    int width = 0, height = 0;
};

std::string readStripped(const char* path) {
    FILE* f = std::fopen(path, "r");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", path);
        std::exit(2);
    }
    std::string s;
    int ch;
    while ((ch = std::fgetc(f)) != EOF) {
        if (ch == '#') {
            while ((ch = std::fgetc(f)) != EOF && ch != '\n') {
            }
        } else {
            s.push_back(static_cast<char>(ch));
        }
    }
    std::fclose(f);
    return s;
}

std::string dirOf(const char* path) {
    const std::string p(path);
    const std::size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string() : p.substr(0, k + 1);
}

// PFM ("PF", width, height, scale, then float RGB rows) into the reference's
// RgbImageTexture, rows in file order (row 0 = the picture's bottom row).
std::shared_ptr<TTexture<Spectrum>> pfmTexture(const std::string& file, const std::string_view& wrap) {
    std::ifstream f(file, std::ios::binary);
    std::string magic;
    int w = 0, h = 0;
    float scale = 0.0f;
    f >> magic >> w >> h >> scale;
    f.get();
    if (!f || magic != "PF" || w <= 0 || h <= 0) {
        std::fprintf(stderr, "cannot read PFM %s\n", file.c_str());
        std::exit(2);
    }
    std::vector<float> raw(static_cast<std::size_t>(w) * h * 3);
    f.read(reinterpret_cast<char*>(raw.data()), static_cast<std::streamsize>(raw.size() * sizeof(float)));
    HdrImage image(w, h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float* px = &raw[(static_cast<std::size_t>(y) * w + x) * 3];
            image.setPixelValue(x, y, Vector3R(px[0], px[1], px[2]));
        }
    const ETextureWrapMode mode = wrap == "clamp" ? ETextureWrapMode::CLAMP : ETextureWrapMode::REPEAT;
    return std::make_shared<RgbImageTexture>(image, ETextureSampleMode::NEAREST, mode);
}

std::unique_ptr<LoadedScene> load(const char* path) {
    auto ls = std::make_unique<LoadedScene>();
    ls->text = readStripped(path);
    std::string_view view(ls->text);
    Tokenizer tok;
    std::size_t start = 0, end = 0;
    while ((end = view.find_first_of('}', start)) != std::string_view::npos) {
        auto data = tok.tokenize(view.substr(start, end - start + 1));
        ls->blocks.push_back(data);
        switch (data->classType()) {
            case ESdClassType::FILM: ls->film = data; break;
            case ESdClassType::CAMERA: ls->camera = data; break;
            case ESdClassType::RENDERER: ls->renderer = data; break;
            case ESdClassType::ACCELERATOR: ls->accel = data; break;
            case ESdClassType::LIGHT_CLUSTER: ls->cluster = data; break;
            case ESdClassType::TEXTURE_REAL:
                ls->realTextures.insert({std::string(data->findString("name")),
                                         instantiator::makeRealTexture(data, ls->realTextures, ls->spectrumTextures)});
                break;
            case ESdClassType::TEXTURE_SPECTRUM: {
                const std::string fn(data->findString("filename"));
                const bool pfm = data->findString("type") == "image" && fn.size() > 4 &&
                                 fn.compare(fn.size() - 4, 4, ".pfm") == 0;
                ls->spectrumTextures.insert(
                    {std::string(data->findString("name")),
                     pfm ? pfmTexture(fn[0] == '/' ? fn : dirOf(path) + fn, data->findString("wrap-mode"))
                         : instantiator::makeSpectrumTexture(data, ls->realTextures, ls->spectrumTextures)});
                break;
            }
            case ESdClassType::MATERIAL:
                ls->bsdfs.insert({std::string(data->findString("name")),
                                  instantiator::makeBsdf(data, ls->realTextures, ls->spectrumTextures, ls->bsdfs)});
                break;
            case ESdClassType::LIGHT: {
                auto light = instantiator::makeLight(data, ls->primitives, ls->background);
                ls->lights.push_back(light);
                break;
            }
            case ESdClassType::PRIMITIVE: {
                const std::size_t before = ls->intersectors.size();
                instantiator::makePrimitive(data, ls->bsdfs, &ls->intersectors, &ls->primitives);
                for (std::size_t i = before; i < ls->intersectors.size(); ++i) {
                    const Primitive* p = dynamic_cast<const Primitive*>(ls->intersectors[i].get());
                    ls->primIndex[p] = static_cast<int>(i);
                }
                break;
            }
            default: break;
        }
        start = end + 1;
    }
    ls->accelerator = instantiator::makeAccelerator(ls->accel, ls->intersectors);
    ls->bruteForce = std::make_shared<BruteForceAccelerator>(ls->intersectors);
    ls->lightCluster = instantiator::makeLightCluster(ls->cluster, ls->lights);
    ls->scene = std::make_shared<Scene>(ls->accelerator, ls->lightCluster);
    if (ls->background) ls->scene->setBackgroundSphere(ls->background.get());
    ls->cam = instantiator::makeCamera(ls->camera);
    ls->width = ls->film->findInt32("image-width", 1024);
    ls->height = ls->film->findInt32("image-height", 768);
    ls->cam->setResolution(Vector2S(static_cast<std::size_t>(ls->width), static_cast<std::size_t>(ls->height)));
    ls->cam->updateTransform();
    ls->estimator = instantiator::makeEstimator(ls->renderer);
    ls->sampler = instantiator::makeSampler(ls->renderer);
    return ls;
}

template <typename T>
std::vector<T> readAll(const char* path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<T> out(bytes.size() / sizeof(T));
    std::memcpy(out.data(), bytes.data(), out.size() * sizeof(T));
    return out;
}

void writeAll(const char* path, const void* data, std::size_t bytes) {
    std::ofstream f(path, std::ios::binary);
    f.write(static_cast<const char*>(data), static_cast<std::streamsize>(bytes));
}

int primOf(const LoadedScene& ls, const PrimitiveInfo& info) {
    auto it = ls.primIndex.find(info.primitive());
    return it == ls.primIndex.end() ? -2 : it->second;
}

int cmdCamera(const LoadedScene& ls, const char* in, const char* out) {
    const auto xy = readAll<double>(in);
    const std::size_t n = xy.size() / 2;
    std::vector<float> res(n * 6);
    for (std::size_t i = 0; i < n; ++i) {
        Ray r;
        ls.cam->spawnPrimaryRay(Vector2D(xy[2 * i], xy[2 * i + 1]), &r);
        for (int k = 0; k < 3; ++k) {
            res[6 * i + k] = r.origin()[k];
            res[6 * i + 3 + k] = r.direction()[k];
        }
    }
    writeAll(out, res.data(), res.size() * sizeof(float));
    return 0;
}

int cmdTrace(const LoadedScene& ls, const char* in, const char* out, bool bruteForce) {
    const auto rays = readAll<float>(in);
    const std::size_t n = rays.size() / 8;
    struct Rec { int32_t bvhPrim; float bvhT; int32_t bfPrim; float bfT; int32_t occluded; };
    std::vector<Rec> res(n);
    for (std::size_t i = 0; i < n; ++i) {
        const float* r = &rays[8 * i];
        const Vector3R o(r[0], r[1], r[2]), d(r[4], r[5], r[6]);
        Ray a(o, d, r[3], r[7]);
        PrimitiveInfo pa;
        Rec rec{-1, 0.0f, -1, 0.0f, 0};
        if (ls.accelerator->isIntersecting(a, pa)) {
            rec.bvhPrim = primOf(ls, pa);
            rec.bvhT = a.maxT();
        }
        if (bruteForce) {
            Ray b(o, d, r[3], r[7]);
            PrimitiveInfo pb;
            if (ls.bruteForce->isIntersecting(b, pb)) {
                rec.bfPrim = primOf(ls, pb);
                rec.bfT = b.maxT();
            }
        } else {
            rec.bfPrim = rec.bvhPrim;
            rec.bfT = rec.bvhT;
        }
        Ray c(o, d, r[3], r[7]);
        rec.occluded = ls.accelerator->isOccluded(c) ? 1 : 0;
        res[i] = rec;
    }
    writeAll(out, res.data(), res.size() * sizeof(Rec));
    return 0;
}

int cmdTexel(const LoadedScene& ls, const char* name, const char* in, const char* out) {
    const auto it = ls.spectrumTextures.find(std::string(name));
    if (it == ls.spectrumTextures.end()) {
        std::fprintf(stderr, "no texture %s\n", name);
        return 2;
    }
    const auto uvw = readAll<float>(in);
    const std::size_t n = uvw.size() / 3;
    std::vector<float> res(n * 3);
    for (std::size_t i = 0; i < n; ++i) {
        Spectrum v;
        it->second->evaluate(Vector3R(uvw[3 * i], uvw[3 * i + 1], uvw[3 * i + 2]), &v);
        Vector3R rgb;
        v.transformToRgb(&rgb);
        for (int k = 0; k < 3; ++k) res[3 * i + k] = rgb[k];
    }
    writeAll(out, res.data(), res.size() * sizeof(float));
    return 0;
}

int cmdPaths(const LoadedScene& ls, const char* in, const char* out) {
    struct Q { double fx, fy; uint64_t key; };
    const auto qs = readAll<Q>(in);
    struct R { float r, g, b; uint32_t draws; };
    std::vector<R> res(qs.size());
    for (std::size_t i = 0; i < qs.size(); ++i) {
        g_stream.key = qs[i].key;
        g_stream.counter = 0;
        Ray primary;
        ls.cam->spawnPrimaryRay(Vector2D(qs[i].fx, qs[i].fy), &primary);
        Spectrum radiance;
        ls.estimator->estimate(*ls.scene, primary, &radiance);
        Vector3R rgb;
        radiance.transformToRgb(&rgb);
        res[i] = R{rgb[0], rgb[1], rgb[2], g_stream.counter};
    }
    writeAll(out, res.data(), res.size() * sizeof(R));
    return 0;
}

// The reference tile loop (core/renderer/render-work/estimatorTileWork.cpp:32-61)
// with an FP64 box-filtered film in place of the FP32 FilmTile: per pixel the
// reference sampler draws its stratified 2-D set from a per-pixel stream, then
// every sample runs the reference estimator on its own path stream.
int cmdRender(const LoadedScene& ls, const char* out, int spp, uint64_t seed, int threads) {
    const int W = ls.width, H = ls.height;
    std::vector<double> film(static_cast<std::size_t>(W) * H * 7, 0.0);
    std::atomic<int> nextRow{0};
    auto worker = [&]() {
        for (;;) {
            const int iy = nextRow.fetch_add(1);
            if (iy >= H) break;
            for (int ix = 0; ix < W; ++ix) {
                const uint32_t pixel = static_cast<uint32_t>(iy * W + ix);
                g_stream.key = oracle_rng::path_key(seed, 0, pixel, 0xFFFFFFFFu);
                g_stream.counter = 0;
                auto s = ls.sampler->clone(static_cast<std::size_t>(spp));
                auto rec = s->requestSample2D();
                double* px = &film[static_cast<std::size_t>(pixel) * 7];
                for (int si = 0; si < spp; ++si) {
                    const Vector2R jitter = rec->nextSample();
                    const double fx = ix + static_cast<double>(jitter.x());
                    const double fy = iy + static_cast<double>(jitter.y());
                    const uint64_t pixelKey = g_stream.key;
                    const uint32_t pixelCtr = g_stream.counter;
                    g_stream.key = oracle_rng::path_key(seed, 0, pixel, static_cast<uint32_t>(si));
                    g_stream.counter = 0;
                    Ray primary;
                    ls.cam->spawnPrimaryRay(Vector2D(fx, fy), &primary);
                    Spectrum radiance;
                    ls.estimator->estimate(*ls.scene, primary, &radiance);
                    g_stream.key = pixelKey;
                    g_stream.counter = pixelCtr;
                    Vector3R rgb;
                    radiance.transformToRgb(&rgb);
                    if (!(std::isfinite(rgb[0]) && std::isfinite(rgb[1]) && std::isfinite(rgb[2]))) continue;
                    for (int k = 0; k < 3; ++k) {
                        px[k] += rgb[k];
                        px[3 + k] += static_cast<double>(rgb[k]) * rgb[k];
                    }
                    px[6] += 1.0;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    writeAll(out, film.data(), film.size() * sizeof(double));
    return 0;
}

// The film's tiles with the scene's filter, as the reference's Film lays them out.
struct TileSet {
    int W = 0, H = 0, tw = 16, th = 16, ntx = 0, nty = 0;
    std::shared_ptr<Filter> filter;
    std::vector<std::unique_ptr<FilmTile>> tiles;

    explicit TileSet(const LoadedScene& ls) {
        W = ls.width;
        H = ls.height;
        tw = ls.film->findInt32("tile-size-x", 16);
        th = ls.film->findInt32("tile-size-y", 16);
        ntx = (W + tw - 1) / tw;
        nty = (H + th - 1) / th;
        filter = instantiator::makeFilter(ls.film);
        reset();
    }
    void reset() {
        tiles.clear();
        for (int ty = 0; ty < nty; ++ty)
            for (int tx = 0; tx < ntx; ++tx) {
                const Vector2I lo(tx * tw, ty * th);
                const Vector2I hi(std::min(lo.x() + tw, W), std::min(lo.y() + th, H));
                tiles.push_back(std::make_unique<FilmTile>(AABB2I(lo, hi), filter.get()));
            }
    }
    FilmTile& tileOfPixel(int ix, int iy) { return *tiles[static_cast<std::size_t>((iy / th) * ntx + ix / tw)]; }
    // adds tile `t`'s sensors to an H x W x stride FP64 film at channels {0,1,2} and `wchan`
    void drain(std::size_t t, double* film, int stride, int wchan) const {
        const FilmTile& ft = *tiles[t];
        const Vector2I& a = ft.tileBound().minVertex();
        const Vector2I& b = ft.tileBound().maxVertex();
        for (int iy = a.y(); iy < b.y(); ++iy)
            for (int ix = a.x(); ix < b.x(); ++ix) {
                const RgbRadianceSensor& s = ft.getSensor(ix - a.x(), iy - a.y());
                double* px = film + static_cast<std::size_t>(iy * W + ix) * stride;
                px[0] += s.r();
                px[1] += s.g();
                px[2] += s.b();
                px[wchan] += s.weight();
            }
    }
};

int cmdFilmTile(const LoadedScene& ls, const char* in, const char* out) {
    const auto v = readAll<float>(in);
    const std::size_t n = v.size() / 5;
    TileSet ts(ls);
    for (std::size_t i = 0; i < n; ++i) {
        const float* r = &v[5 * i];
        const int ix = static_cast<int>(std::floor(r[0])), iy = static_cast<int>(std::floor(r[1]));
        // the Spectrum overload, which drops NaN / Inf samples as the render loop's does
        ts.tileOfPixel(ix, iy).addSample(Vector2R(r[0], r[1]), Spectrum(Vector3R(r[2], r[3], r[4])));
    }
    std::vector<double> film(static_cast<std::size_t>(ts.W) * ts.H * 4, 0.0);
    for (std::size_t t = 0; t < ts.tiles.size(); ++t) ts.drain(t, film.data(), 4, 3);
    writeAll(out, film.data(), film.size() * sizeof(double));
    return 0;
}

int cmdRenderTiles(const LoadedScene& ls, const char* out, int spp, uint64_t seed, int threads) {
    const int W = ls.width, H = ls.height;
    TileSet ts(ls);
    std::vector<double> film(static_cast<std::size_t>(W) * H * 7, 0.0);
    const int per = std::min(spp, 256), passes = (spp + per - 1) / per;
    std::atomic<int> nextTile{0};
    auto worker = [&]() {
        for (;;) {
            const int t = nextTile.fetch_add(1);
            if (t >= static_cast<int>(ts.tiles.size())) break;
            FilmTile& base = *ts.tiles[static_cast<std::size_t>(t)];
            const AABB2I bound = base.tileBound();
            for (int pass = 0; pass < passes; ++pass) {
                FilmTile ft(bound, ts.filter.get());
                const uint64_t pseed = seed + static_cast<uint64_t>(pass);
                for (int iy = bound.minVertex().y(); iy < bound.maxVertex().y(); ++iy)
                    for (int ix = bound.minVertex().x(); ix < bound.maxVertex().x(); ++ix) {
                        const uint32_t pixel = static_cast<uint32_t>(iy * W + ix);
                        g_stream.key = oracle_rng::path_key(pseed, 0, pixel, 0xFFFFFFFFu);
                        g_stream.counter = 0;
                        auto s = ls.sampler->clone(static_cast<std::size_t>(per));
                        auto rec = s->requestSample2D();
                        for (int si = 0; si < per; ++si) {
                            const Vector2R pos = Vector2I(ix, iy).asType<real>() + rec->nextSample();
                            const uint64_t pixelKey = g_stream.key;
                            const uint32_t pixelCtr = g_stream.counter;
                            g_stream.key = oracle_rng::path_key(pseed, 0, pixel, static_cast<uint32_t>(si));
                            g_stream.counter = 0;
                            Ray primary;
                            ls.cam->spawnPrimaryRay(pos.asType<float64>(), &primary);
                            Spectrum radiance;
                            ls.estimator->estimate(*ls.scene, primary, &radiance);
                            g_stream.key = pixelKey;
                            g_stream.counter = pixelCtr;
                            ft.addSample(pos, radiance);
                        }
                    }
                const Vector2I& a = bound.minVertex();
                const Vector2I& b = bound.maxVertex();
                for (int iy = a.y(); iy < b.y(); ++iy)
                    for (int ix = a.x(); ix < b.x(); ++ix) {
                        const RgbRadianceSensor& sn = ft.getSensor(ix - a.x(), iy - a.y());
                        double* px = &film[static_cast<std::size_t>(iy * W + ix) * 7];
                        px[0] += sn.r();
                        px[1] += sn.g();
                        px[2] += sn.b();
                        px[6] += sn.weight();
                    }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    writeAll(out, film.data(), film.size() * sizeof(double));
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_harness <camera|trace|paths|render> <scene.crsd> ...\n");
        return 2;
    }
    const std::string cmd = argv[1];
    auto ls = load(argv[2]);
    if (cmd == "camera" && argc >= 5) return cmdCamera(*ls, argv[3], argv[4]);
    if (cmd == "trace" && argc >= 5) return cmdTrace(*ls, argv[3], argv[4], true);
    if (cmd == "trace-bvh" && argc >= 5) return cmdTrace(*ls, argv[3], argv[4], false);
    if (cmd == "texel" && argc >= 6) return cmdTexel(*ls, argv[3], argv[4], argv[5]);
    if (cmd == "paths" && argc >= 5) return cmdPaths(*ls, argv[3], argv[4]);
    if (cmd == "filmtile" && argc >= 5) return cmdFilmTile(*ls, argv[3], argv[4]);
    if (cmd == "render-tiles" && argc >= 7) {
        return cmdRenderTiles(*ls, argv[3], std::atoi(argv[4]), std::strtoull(argv[5], nullptr, 10), std::atoi(argv[6]));
    }
    if (cmd == "render" && argc >= 7) {
        return cmdRender(*ls, argv[3], std::atoi(argv[4]), std::strtoull(argv[5], nullptr, 10), std::atoi(argv[6]));
    }
    std::fprintf(stderr, "bad command\n");
    return 2;
}
