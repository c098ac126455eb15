// Host C++17 mirror of the reference renderer's interfaces for the path this
// library accelerates, implemented over the C ABI (include/cadise_gpu.h,
// include/cadise_crsd.h):
//
//   Renderer            source/core/renderer/renderer.h:11-29
//   Accelerator         source/core/intersector/accelerator/accelerator.h:7-13
//   Film                source/core/film/film.h:17-59 (FP64 sums instead of FP32 sensors)
//   makeRenderer        source/core/instantiator/rendererInstantiator.cpp:88-120
//   RenderDatabase      source/core/renderDatabase.cpp:39-135 (load -> prepare -> render)
//
// CudaSamplingRenderer is the drop-in for SamplingRenderer + PtEstimator
// (registered for CRSD renderer types "sampling" and "cuda-sampling");
// CudaBvhAccelerator answers the reference's per-ray queries and batched ones
// through the GPU BVH.  Errors are reported as cadise_gb300::Error.
#pragma once

#include "../../include/cadise_crsd.h"
#include "../../include/cadise_gpu.h"

#include <cfloat>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cadise_gb300 {

class Error : public std::runtime_error {
public:
    Error(cgpu_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    cgpu_status status;
};

struct Vector3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
};

// ray.cpp:14-16 defaults: minT = ray_epsilon (1e-3), maxT = FLT_MAX.
struct Ray {
    Vector3 origin;
    Vector3 direction;
    float minT = 0.001f;
    float maxT = FLT_MAX;
};

struct PrimitiveInfo {
    int32_t primitive = -1;  // creation-order index; -1: none
    float u = 0.0f, v = 0.0f;
};

// A GPU context (one CUDA stream) shared by the objects below.
class Device {
public:
    explicit Device(int device = 0, void* stream = nullptr);
    ~Device();
    Device(const Device&) = delete;
    Device& operator=(const Device&) = delete;
    cgpu_ctx* ctx() const { return ctx_; }
    void check(cgpu_status s) const;

private:
    cgpu_ctx* ctx_ = nullptr;
};

// The scene of one CRSD file, resident on the device.
class Scene {
public:
    Scene(std::shared_ptr<Device> device, const std::string& crsd_path);
    Scene(std::shared_ptr<Device> device, const cgpu_scene_desc& desc);
    ~Scene();
    int32_t id() const { return id_; }
    const cgpu_crsd_settings& settings() const { return settings_; }
    int width() const { return width_; }
    int height() const { return height_; }
    std::shared_ptr<Device> device() const { return device_; }

private:
    std::shared_ptr<Device> device_;
    cgpu_crsd_settings settings_{};
    int32_t id_ = -1;
    int width_ = 0, height_ = 0;
};

class Accelerator {
public:
    virtual ~Accelerator() = default;
    virtual void evaluateBound(Vector3* lo, Vector3* hi) const = 0;
    virtual bool isIntersecting(Ray& ray, PrimitiveInfo& info) const = 0;
    virtual bool isOccluded(const Ray& ray) const = 0;
};

class CudaBvhAccelerator : public Accelerator {
public:
    explicit CudaBvhAccelerator(std::shared_ptr<Scene> scene) : scene_(std::move(scene)) {}
    void evaluateBound(Vector3* lo, Vector3* hi) const override;
    // one ray per call, as the reference's interface; shrinks ray.maxT on a hit
    bool isIntersecting(Ray& ray, PrimitiveInfo& info) const override;
    bool isOccluded(const Ray& ray) const override;
    // batched forms (the ones to use on a GPU)
    void intersectBatch(std::vector<Ray>& rays, std::vector<PrimitiveInfo>& infos) const;
    void occludedBatch(const std::vector<Ray>& rays, std::vector<uint8_t>& occluded) const;

private:
    std::shared_ptr<Scene> scene_;
};

// Per-pixel FP64 accumulation: sum, sum of squares, accepted sample count.
class Film {
public:
    Film(int width, int height);
    int width() const { return w_; }
    int height() const { return h_; }
    std::vector<double> sum, sumSq, count;
    // mean radiance per pixel (Film::save normalisation, film.cpp:159-196)
    std::vector<float> resolve() const;
    // 8-bit sRGB binary PPM (forward gamma of source/math/math.cpp:92-99) and
    // linear little-endian PFM
    void savePpm(const std::string& path) const;
    void savePfm(const std::string& path) const;

private:
    int w_, h_;
};

class Renderer {
public:
    virtual ~Renderer() = default;
    virtual void render() const = 0;
    void setScene(std::shared_ptr<Scene> scene) { scene_ = std::move(scene); }
    void setFilm(std::shared_ptr<Film> film) { film_ = std::move(film); }

protected:
    std::shared_ptr<Scene> scene_;
    std::shared_ptr<Film> film_;
};

// SamplingRenderer + PtEstimator on the GPU: renders the scene's spp samples
// per pixel (wavefront by default) and reads the FP64 film back.
class CudaSamplingRenderer : public Renderer {
public:
    CudaSamplingRenderer(int spp, int mode, bool graph, uint64_t seed)
        : spp_(spp), mode_(mode), graph_(graph), seed_(seed) {}
    void render() const override;
    double lastRenderMs() const { return last_ms_; }

private:
    int spp_, mode_;
    bool graph_;
    uint64_t seed_;
    mutable double last_ms_ = 0.0;
};

// Factory keyed by the CRSD renderer type; returns nullptr for unknown types
// like the reference's instantiator.
std::unique_ptr<Renderer> makeRenderer(const cgpu_crsd_settings& settings);

// RenderDatabase-style session: load a CRSD file, build the scene on the
// device, render, save.
class RenderSession {
public:
    explicit RenderSession(const std::string& crsd_path, int device = 0);
    void render();
    void save(const std::string& stem) const;  // <stem>.ppm + <stem>.pfm
    const Film& film() const { return *film_; }
    std::shared_ptr<Scene> scene() const { return scene_; }
    double renderMs() const { return ms_; }

private:
    std::shared_ptr<Device> device_;
    std::shared_ptr<Scene> scene_;
    std::shared_ptr<Film> film_;
    std::unique_ptr<Renderer> renderer_;
    double ms_ = 0.0;
};

}  // namespace cadise_gb300
