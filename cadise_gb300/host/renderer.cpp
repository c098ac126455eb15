// Host interface mirror (see cadise_host.h).
#include "cadise_host.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace cadise_gb300 {

Device::Device(int device, void* stream) {
    cgpu_options o{};
    o.device = device;
    o.stream = stream;
    const cgpu_status s = cgpu_create(&ctx_, &o);
    if (s != CGPU_OK) throw Error(s, std::string("cgpu_create: ") + cgpu_status_string(s));
}

Device::~Device() { cgpu_destroy(ctx_); }

void Device::check(cgpu_status s) const {
    if (s != CGPU_OK) throw Error(s, std::string(cgpu_status_string(s)) + ": " + cgpu_last_error(ctx_));
}

Scene::Scene(std::shared_ptr<Device> device, const std::string& crsd_path) : device_(std::move(device)) {
    cgpu_crsd_scene* sc = nullptr;
    char err[512] = {0};
    const cgpu_status s = cgpu_crsd_load_file(crsd_path.c_str(), &sc, err, sizeof(err));
    if (s != CGPU_OK) throw Error(s, std::string("CRSD: ") + err);
    cgpu_crsd_settings_get(sc, &settings_);
    const cgpu_scene_desc* d = cgpu_crsd_desc(sc);
    width_ = d->width;
    height_ = d->height;
    const cgpu_status u = cgpu_scene_upload(device_->ctx(), d, &id_);
    cgpu_crsd_free(sc);
    device_->check(u);
}

Scene::Scene(std::shared_ptr<Device> device, const cgpu_scene_desc& desc) : device_(std::move(device)) {
    width_ = desc.width;
    height_ = desc.height;
    std::snprintf(settings_.renderer_type, sizeof(settings_.renderer_type), "cuda-sampling");
    settings_.spp = desc.spp;
    settings_.max_depth = desc.max_depth;
    settings_.mode = CGPU_MODE_WAVEFRONT;
    settings_.use_graph = 1;
    settings_.seed = 1;
    device_->check(cgpu_scene_upload(device_->ctx(), &desc, &id_));
}

Scene::~Scene() {
    if (id_ >= 0) cgpu_scene_release(device_->ctx(), id_);
}

void CudaBvhAccelerator::evaluateBound(Vector3* lo, Vector3* hi) const {
    cgpu_scene_info info{};
    scene_->device()->check(cgpu_scene_info_get(scene_->device()->ctx(), scene_->id(), &info));
    *lo = Vector3{info.bounds_min[0], info.bounds_min[1], info.bounds_min[2]};
    *hi = Vector3{info.bounds_max[0], info.bounds_max[1], info.bounds_max[2]};
}

static cgpu_ray to_c(const Ray& r) {
    cgpu_ray c;
    c.org[0] = r.origin.x; c.org[1] = r.origin.y; c.org[2] = r.origin.z;
    c.dir[0] = r.direction.x; c.dir[1] = r.direction.y; c.dir[2] = r.direction.z;
    c.t_min = r.minT;
    c.t_max = r.maxT;
    return c;
}

void CudaBvhAccelerator::intersectBatch(std::vector<Ray>& rays, std::vector<PrimitiveInfo>& infos) const {
    std::vector<cgpu_ray> c(rays.size());
    for (size_t i = 0; i < rays.size(); ++i) c[i] = to_c(rays[i]);
    std::vector<cgpu_hit> h(rays.size());
    scene_->device()->check(cgpu_trace_closest(scene_->device()->ctx(), scene_->id(), c.data(), uint32_t(c.size()), h.data()));
    infos.resize(rays.size());
    for (size_t i = 0; i < rays.size(); ++i) {
        infos[i] = PrimitiveInfo{h[i].primitive, h[i].u, h[i].v};
        if (h[i].primitive >= 0) rays[i].maxT = h[i].t;
    }
}

void CudaBvhAccelerator::occludedBatch(const std::vector<Ray>& rays, std::vector<uint8_t>& occluded) const {
    std::vector<cgpu_ray> c(rays.size());
    for (size_t i = 0; i < rays.size(); ++i) c[i] = to_c(rays[i]);
    occluded.resize(rays.size());
    scene_->device()->check(cgpu_trace_any(scene_->device()->ctx(), scene_->id(), c.data(), uint32_t(c.size()), occluded.data()));
}

bool CudaBvhAccelerator::isIntersecting(Ray& ray, PrimitiveInfo& info) const {
    std::vector<Ray> r{ray};
    std::vector<PrimitiveInfo> i;
    intersectBatch(r, i);
    ray = r[0];
    info = i[0];
    return info.primitive >= 0;
}

bool CudaBvhAccelerator::isOccluded(const Ray& ray) const {
    std::vector<uint8_t> o;
    occludedBatch(std::vector<Ray>{ray}, o);
    return o[0] != 0;
}

Film::Film(int width, int height)
    : sum(size_t(width) * height * 3), sumSq(size_t(width) * height * 3), count(size_t(width) * height), w_(width), h_(height) {}

std::vector<float> Film::resolve() const {
    std::vector<float> out(size_t(w_) * h_ * 3, 0.0f);
    for (size_t p = 0; p < count.size(); ++p) {
        if (count[p] <= 0.0) continue;
        for (int k = 0; k < 3; ++k) out[3 * p + k] = float(sum[3 * p + k] / count[p]);
    }
    return out;
}

void Film::savePpm(const std::string& path) const {
    const std::vector<float> img = resolve();
    std::ofstream f(path, std::ios::binary);
    f << "P6\n" << w_ << " " << h_ << "\n255\n";
    for (float v : img) {
        const float c = v <= 0.0031308f ? 12.92f * v : 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f;
        const float q = std::fmin(std::fmax(c, 0.0f), 1.0f) * 255.0f + 0.5f;
        const unsigned char b = static_cast<unsigned char>(q);
        f.write(reinterpret_cast<const char*>(&b), 1);
    }
}

void Film::savePfm(const std::string& path) const {
    const std::vector<float> img = resolve();
    std::ofstream f(path, std::ios::binary);
    f << "PF\n" << w_ << " " << h_ << "\n-1.0\n";
    for (int y = h_ - 1; y >= 0; --y) f.write(reinterpret_cast<const char*>(&img[size_t(y) * w_ * 3]), std::streamsize(w_) * 12);
}

void CudaSamplingRenderer::render() const {
    if (!scene_ || !film_) throw Error(CGPU_ERR_INVALID_ARGUMENT, "renderer needs a scene and a film");
    cgpu_ctx* ctx = scene_->device()->ctx();
    const int32_t id = scene_->id();
    cgpu_render_params p{};
    p.scenes = &id;
    p.num_scenes = 1;
    p.first_sample = 0;
    p.num_samples = uint32_t(spp_);
    p.seed = seed_;
    p.mode = mode_;
    p.use_graph = graph_ ? 1 : 0;
    const auto t0 = std::chrono::steady_clock::now();
    scene_->device()->check(cgpu_film_clear(ctx, id));
    scene_->device()->check(cgpu_render(ctx, &p));
    scene_->device()->check(cgpu_film_read(ctx, id, film_->sum.data(), film_->sumSq.data(), film_->count.data()));
    last_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

std::unique_ptr<Renderer> makeRenderer(const cgpu_crsd_settings& s) {
    const std::string type = s.renderer_type;
    if (type == "sampling" || type == "cuda-sampling")
        return std::make_unique<CudaSamplingRenderer>(s.spp, s.mode, s.use_graph != 0, s.seed);
    return nullptr;
}

RenderSession::RenderSession(const std::string& crsd_path, int device) {
    device_ = std::make_shared<Device>(device);
    scene_ = std::make_shared<Scene>(device_, crsd_path);
    film_ = std::make_shared<Film>(scene_->width(), scene_->height());
    renderer_ = makeRenderer(scene_->settings());
    if (!renderer_) throw Error(CGPU_ERR_UNSUPPORTED, std::string("renderer type ") + scene_->settings().renderer_type);
    renderer_->setScene(scene_);
    renderer_->setFilm(film_);
}

void RenderSession::render() {
    const auto t0 = std::chrono::steady_clock::now();
    renderer_->render();
    ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void RenderSession::save(const std::string& stem) const {
    film_->savePpm(stem + ".ppm");
    film_->savePfm(stem + ".pfm");
}

}  // namespace cadise_gb300
