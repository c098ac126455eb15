// Path-replay adjoint: d(loss)/d(albedo texels, GGX roughness, emitter radiance).
//
// No counterpart in the reference (it has no differentiable rendering).  The
// estimator is PtEstimator's (source/core/estimator/ptEstimator.cpp:25-123),
// run by the same plan_vertex / mis_resolve functions as the forward kernels.
// Method: path replay backpropagation (Vicini, Speierer & Jakob, "Path Replay
// Backpropagation", SIGGRAPH 2021) with detached sampling - sampling pdfs, MIS
// weights and roulette probabilities are held constant, so
//   d/dtheta E[L] = E[ sum over terms  term * d ln(term)/d theta ].
// A path's radiance is a sum of terms (emission, NEE light sample, NEE BSDF
// sample) at each vertex j, and every later term carries the continuation
// weight f_j cos / pdf of vertex j.  Each path is replayed twice from its
// seed (no stored vertices): replay 1 gives the total L; replay 2 walks the
// vertices again with R_j = L - (terms so far), the radiance still to come:
//   albedo texel at a Lambert vertex j:  dL += delta * (A_j + B_j + R_j) / albedo_j
//   roughness of vertex j's material:   dL += delta . (A_j g(w_l) + B_j g(w_b) + R_j g(w_c)),
//                                        g = d ln f / d roughness
//   radiance of a light:                dL += delta * (term / Le)
// with delta = d loss / d pixel / spp.  Gradients are reduced in FP64
// (shared-memory block sums for roughness and radiance, global atomics for
// texels).
#include "internal.h"
#include "adjoint.cuh"

#include <algorithm>
#include <vector>

namespace cg {

struct AdjArgs {
    const SceneD* scenes;
    int scene;
    uint32_t npix, width, spp_total, first;
    uint64_t npaths;
    uint64_t seed;
    const float* dLdI;
    double* g_tex;
    const int* tex_offset;  // per texture: first float of its block in g_tex
    double* g_rough;
    double* g_rad;
    int nmat, nlight;
};

CG_D void shared_add(double* sh, int i, double v) {
    if (v != 0.0) atomicAdd(sh + i, v);
}

// Roughness and radiance reduce in shared memory, texels in global memory.
struct BlockSink {
    double* shr;
    double* shl;
    double* g_tex;
    const int* tex_offset;
    CG_D void rough(int m, double v) { shared_add(shr, m, v); }
    CG_D void rad(int i, double v) { shared_add(shl, i, v); }
    CG_D void tex(int t, int k, double v) { atomicAdd(g_tex + tex_offset[t] + k, v); }
};

// 64 registers (8 blocks of 128 threads per SM): the spills cost less than the
// latency the extra resident warps hide (measured: 208 ms against 265 ms at
// the 142 registers it would take).
__global__ void __launch_bounds__(128, 8) k_adjoint(AdjArgs a) {
    extern __shared__ double sh[];  // [0, nmat) roughness, [nmat, nmat + 3 nlight) radiance
    const int nsh = a.nmat + 3 * a.nlight;
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) sh[i] = 0.0;
    __syncthreads();
    BlockSink sink{sh, sh + a.nmat, a.g_tex, a.tex_offset};
    const SceneD& S = a.scenes[a.scene];
    for (uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < a.npaths; p += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t pixel = uint32_t(p % a.npix);
        const uint32_t sample = a.first + uint32_t(p / a.npix);
        const float inv_spp = 1.0f / float(a.spp_total);
        const float3 delta = mk(a.dLdI[3 * pixel] * inv_spp, a.dLdI[3 * pixel + 1] * inv_spp, a.dLdI[3 * pixel + 2] * inv_spp);
        if (is_zero(delta)) continue;
        PathId id;
        id.scene = a.scene;
        id.pixel = pixel;
        id.sample = sample;
        id.width = a.width;
        adjoint_path(S, id, a.seed, delta, a.nlight, sink);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.nmat; i += blockDim.x)
        if (sink.shr[i] != 0.0) atomicAdd(a.g_rough + i, sink.shr[i]);
    for (int i = threadIdx.x; i < 3 * a.nlight; i += blockDim.x)
        if (sink.shl[i] != 0.0) atomicAdd(a.g_rad + i, sink.shl[i]);
}

}  // namespace cg

// ================================================================ host side ==
using namespace cg;

namespace {

bool valid(cgpu_ctx* ctx, int32_t s) { return ctx && s >= 0 && s < int32_t(ctx->scenes.size()) && ctx->scenes[s].live; }

uint64_t texel_floats(const SceneSlot& sl) {
    uint64_t n = 0;
    for (const TextureD& t : sl.h_texs) n += uint64_t(t.width) * t.height * 3;
    return n;
}

}  // namespace

extern "C" {

cgpu_status cgpu_param_counts_get(cgpu_ctx* ctx, int32_t scene, cgpu_param_counts* out) {
    if (!ctx || !out) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "param_counts: unknown scene id");
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    out->texel_floats = texel_floats(sl);
    out->materials = uint32_t(sl.h_mats.size());
    out->lights = uint32_t(sl.num_area_lights);
    return CGPU_OK;
}

cgpu_status cgpu_params_get(cgpu_ctx* ctx, int32_t scene, float* texels, float* roughness, float* radiance) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "params_get: unknown scene id");
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    cudaSetDevice(ctx->device);
    if (texels) {
        size_t off = 0;
        for (const TextureD& t : sl.h_texs) {
            const size_t n = size_t(t.width) * t.height * 3;
            cudaError_t e = cudaMemcpy(texels + off, t.texels, n * sizeof(float), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cg_cuda(ctx, e, "params_get texels");
            off += n;
        }
    }
    if (roughness)
        for (size_t i = 0; i < sl.h_mats.size(); ++i) roughness[i] = sl.h_mats[i].roughness;
    if (radiance)
        for (size_t i = 0; i < size_t(sl.num_area_lights); ++i) {
            radiance[3 * i + 0] = sl.h_lights[i].radiance.x;
            radiance[3 * i + 1] = sl.h_lights[i].radiance.y;
            radiance[3 * i + 2] = sl.h_lights[i].radiance.z;
        }
    return CGPU_OK;
}

cgpu_status cgpu_params_set(cgpu_ctx* ctx, int32_t scene, const float* texels, const float* roughness,
                            const float* radiance) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "params_set: unknown scene id");
    SceneSlot& sl = ctx->scenes[size_t(scene)];
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (texels) {
        size_t off = 0;
        for (const TextureD& t : sl.h_texs) {
            const size_t n = size_t(t.width) * t.height * 3;
            cudaError_t e = cudaMemcpy(const_cast<float*>(t.texels), texels + off, n * sizeof(float), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cg_cuda(ctx, e, "params_set texels");
            off += n;
        }
    }
    if (roughness) {
        for (size_t i = 0; i < sl.h_mats.size(); ++i) {
            MaterialD& m = sl.h_mats[i];
            if (!(roughness[i] >= 0.0f)) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "params_set: negative roughness");
            m.roughness = roughness[i];
            const float safe = roughness[i] > 0.001f ? roughness[i] : 0.001f;
            m.alpha = safe * safe > 0.001f ? safe * safe : 0.001f;
        }
        cudaError_t e = cudaMemcpy(sl.d_mats, sl.h_mats.data(), sl.h_mats.size() * sizeof(MaterialD), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "params_set roughness");
    }
    if (radiance) {
        for (size_t i = 0; i < size_t(sl.num_area_lights); ++i)
            sl.h_lights[i].radiance = make_float3(radiance[3 * i], radiance[3 * i + 1], radiance[3 * i + 2]);
        cudaError_t e = cudaMemcpy(sl.d_lights, sl.h_lights.data(), sl.h_lights.size() * sizeof(LightD), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cg_cuda(ctx, e, "params_set radiance");
    }
    return CGPU_OK;
}

cgpu_status cgpu_adjoint_forward(cgpu_ctx* ctx, int32_t scene, uint32_t spp, uint64_t seed, float* image_out) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "adjoint_forward: unknown scene id");
    if (spp == 0) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "adjoint_forward: spp must be positive");
    cudaSetDevice(ctx->device);
    cgpu_status st = cg_film_clear(ctx, scene);
    if (st != CGPU_OK) return st;
    cgpu_render_params p{};
    p.scenes = &scene;
    p.num_scenes = 1;
    p.first_sample = 0;
    p.num_samples = spp;
    p.seed = seed;
    p.mode = CGPU_MODE_WAVEFRONT;
    p.use_graph = 1;
    st = cg_render_batches(ctx, &p);
    if (st != CGPU_OK || !image_out) return st;
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    const size_t npix = size_t(sl.width) * sl.height;
    std::vector<double> sum(npix * 3), cnt(npix);
    cudaError_t e = cudaMemcpyAsync(sum.data(), sl.film.sum, npix * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), sl.film.count, npix * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cg_cuda(ctx, e, "adjoint_forward readback");
    for (size_t i = 0; i < npix; ++i)
        for (int k = 0; k < 3; ++k) image_out[3 * i + k] = cnt[i] > 0.0 ? float(sum[3 * i + k] / cnt[i]) : 0.0f;
    return cg_check_status(ctx);
}

cgpu_status cgpu_set_adjoint_mode(cgpu_ctx* ctx, int32_t mode) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (mode != CGPU_MODE_MEGAKERNEL && mode != CGPU_MODE_WAVEFRONT)
        return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "set_adjoint_mode: unknown mode");
    ctx->adjoint_schedule = mode;
    return CGPU_OK;
}

cgpu_status cgpu_adjoint_backward(cgpu_ctx* ctx, int32_t scene, uint32_t spp, uint64_t seed, const float* dLdI,
                                  double* grad_texels, double* grad_roughness, double* grad_radiance) {
    if (!ctx) return CGPU_ERR_INVALID_ARGUMENT;
    if (!valid(ctx, scene)) return cg_fail(ctx, CGPU_ERR_NOT_FOUND, "adjoint_backward: unknown scene id");
    if (!dLdI || spp == 0) return cg_fail(ctx, CGPU_ERR_INVALID_ARGUMENT, "adjoint_backward: bad arguments");
    cudaSetDevice(ctx->device);
    cgpu_status st = cg_sync_tables(ctx);
    if (st != CGPU_OK) return st;
    const SceneSlot& sl = ctx->scenes[size_t(scene)];
    const size_t npix = size_t(sl.width) * sl.height;
    const uint64_t ntex = texel_floats(sl);
    const int nmat = int(sl.h_mats.size()), nlight = sl.num_area_lights;
    const size_t shared_bytes = size_t(nmat + 3 * nlight) * sizeof(double);
    if (shared_bytes > 96 * 1024) return cg_fail(ctx, CGPU_ERR_UNSUPPORTED, "adjoint_backward: too many materials and lights");
    std::vector<int> offs(sl.h_texs.size());
    {
        int o = 0;
        for (size_t i = 0; i < sl.h_texs.size(); ++i) {
            offs[i] = o;
            o += sl.h_texs[i].width * sl.h_texs[i].height * 3;
        }
    }
    float* d_dl = nullptr;
    double *d_gt = nullptr, *d_gr = nullptr, *d_gl = nullptr;
    int* d_off = nullptr;
    cudaError_t e = cudaMalloc(&d_dl, npix * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_gt, std::max<uint64_t>(ntex, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_gr, std::max(nmat, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_gl, std::max(3 * nlight, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_off, std::max<size_t>(offs.size(), 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_dl, dLdI, npix * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && !offs.empty())
        e = cudaMemcpyAsync(d_off, offs.data(), offs.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gt, 0, std::max<uint64_t>(ntex, 1) * sizeof(double), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gr, 0, std::max(nmat, 1) * sizeof(double), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gl, 0, std::max(3 * nlight, 1) * sizeof(double), ctx->stream);
    if (e == cudaSuccess && ctx->adjoint_schedule == CGPU_MODE_WAVEFRONT) {
        AdjBufs ab{};
        ab.dLdI = d_dl;
        ab.g_tex = d_gt;
        ab.tex_offset = d_off;
        ab.g_rough = d_gr;
        ab.g_rad = d_gl;
        ab.nmat = nmat;
        ab.nlight = nlight;
        ab.inv_spp = 1.0f / float(spp);
        const cgpu_status ws = cg_adjoint_wavefront(ctx, scene, spp, seed, ab);
        if (ws != CGPU_OK) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(d_dl);
            cudaFree(d_gt);
            cudaFree(d_gr);
            cudaFree(d_gl);
            cudaFree(d_off);
            return ws;
        }
    } else if (e == cudaSuccess) {
        AdjArgs a;
        a.scenes = ctx->d_scenes;
        a.scene = scene;
        a.npix = uint32_t(npix);
        a.width = uint32_t(sl.width);
        a.spp_total = spp;
        a.first = 0;
        a.npaths = uint64_t(npix) * spp;
        a.seed = seed;
        a.dLdI = d_dl;
        a.g_tex = d_gt;
        a.tex_offset = d_off;
        a.g_rough = d_gr;
        a.g_rad = d_gl;
        a.nmat = nmat;
        a.nlight = nlight;
        int per_sm = 0;
        cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, int(shared_bytes));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint, 128, shared_bytes);
        const uint64_t need = (a.npaths + 127) / 128;
        const int grid = int(std::max<uint64_t>(1, std::min<uint64_t>(need, uint64_t(ctx->num_sms) * std::max(per_sm, 1))));
        k_adjoint<<<grid, 128, shared_bytes, ctx->stream>>>(a);
        e = cudaGetLastError();
        ctx->stats.kernel_launches = 1;
    }
    if (e == cudaSuccess && grad_texels && ntex)
        e = cudaMemcpyAsync(grad_texels, d_gt, ntex * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && grad_roughness)
        e = cudaMemcpyAsync(grad_roughness, d_gr, size_t(nmat) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && grad_radiance)
        e = cudaMemcpyAsync(grad_radiance, d_gl, size_t(3 * nlight) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_dl);
    cudaFree(d_gt);
    cudaFree(d_gr);
    cudaFree(d_gl);
    cudaFree(d_off);
    const cgpu_status fin = cg_cuda(ctx, e, "adjoint_backward");
    return fin != CGPU_OK ? fin : cg_check_status(ctx);
}

}  // extern "C"
