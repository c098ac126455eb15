/*
 * cadise_gpu.h - C ABI of the GB300 (sm_103a) path tracer.
 *
 * Plain C types only: host pointers, sizes and status codes.  Every function
 * returns a cgpu_status and never aborts; cgpu_last_error() gives the message
 * of the last failure on a context.  One context owns one CUDA stream and is
 * used from one host thread at a time.
 *
 * What each entry point replaces in the reference renderer (paths relative to
 * the reference project):
 *
 *   cgpu_create / cgpu_destroy     RenderDatabase::prepareRender wiring
 *                                  (source/core/renderDatabase.cpp:78-131)
 *   cgpu_scene_upload              makePrimitive / makeBsdf / makeLight /
 *                                  makeLightCluster + Scene ctor
 *                                  (source/core/instantiator/primitiveInstantiator.cpp:92-129,
 *                                   bsdfInstantiator.cpp:177-221, lightInstantiator.cpp:80-103,
 *                                   source/core/scene.cpp:13-22)
 *                                  and the BVH build of makeAccelerator
 *                                  (source/core/instantiator/acceleratorInstantiator.cpp:57-80,
 *                                   source/core/intersector/accelerator/bvh/bvhAccelerator.cpp:10-32)
 *   cgpu_trace_closest             Accelerator::isIntersecting / Scene::isIntersecting
 *                                  (source/core/intersector/accelerator/accelerator.h:7-13,
 *                                   bvh/bvhAccelerator.cpp:40-97, source/core/scene.cpp:30-65)
 *   cgpu_trace_any                 Accelerator::isOccluded / Scene::isOccluded
 *                                  (bvh/bvhAccelerator.cpp:99-156, source/core/scene.cpp:67-77)
 *   cgpu_camera_rays               Camera::spawnPrimaryRay
 *                                  (source/core/camera/perspectivePinholeCamera.cpp:52-73)
 *   cgpu_path_radiance             EnergyEstimator::estimate of PtEstimator
 *                                  (source/core/estimator/energyEstimator.h:12-30,
 *                                   source/core/estimator/ptEstimator.cpp:25-123)
 *   cgpu_render                    Renderer::render of SamplingRenderer
 *                                  (source/core/renderer/renderer.h:11-29,
 *                                   source/core/renderer/sampling/samplingRenderer.cpp:33-68,
 *                                   render-work/estimatorTileWork.cpp:32-61)
 *   cgpu_film_read / _clear        Film::mergeWithFilmTile / Film::save accumulation
 *                                  (source/core/film/film.cpp:79-99,159-196)
 *   cgpu_adjoint_*                 no counterpart in the reference (it has no
 *                                  differentiable rendering)
 */
#ifndef CADISE_GPU_H
#define CADISE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGPU_ABI_VERSION 5

typedef enum cgpu_status {
    CGPU_OK = 0,
    CGPU_ERR_INVALID_ARGUMENT = 1,
    CGPU_ERR_CUDA = 2,
    CGPU_ERR_OUT_OF_MEMORY = 3,
    CGPU_ERR_TIMEOUT = 4, /* a device-side iteration budget ran out (cgpu_set_visit_budget) */
    CGPU_ERR_UNSUPPORTED = 5,
    CGPU_ERR_NOT_FOUND = 6,
    CGPU_ERR_PARSE = 7,
    CGPU_ERR_NO_DEVICE = 8
} cgpu_status;

typedef struct cgpu_ctx cgpu_ctx;

/* ---------------------------------------------------------------- scene -- */

/* Primitive kinds, one per reference intersector (primitiveInstantiator.cpp:92-129).
 * A sphere (sphere.cpp) stores centre and radius in the first 4 of its 9 vertex
 * floats; spheres cannot emit (the reference leaves their position sampling
 * unimplemented, sphere.cpp:137-141). */
enum { CGPU_PRIM_TRIANGLE = 0, CGPU_PRIM_RECTANGLE = 1, CGPU_PRIM_SPHERE = 2 };

/* BSDF kinds keyed like the reference's CRSD material types (bsdfInstantiator.cpp:177-221). */
enum {
    CGPU_BSDF_LAMBERTIAN = 0,       /* "matte-lambertian"      lambertianDiffuse.cpp        */
    CGPU_BSDF_CONDUCTOR_GGX = 1,    /* "conductor-microfacet"  conductorMicrofacet.cpp      */
    CGPU_BSDF_GLASS = 2,            /* "glass"                 specularDielectric.cpp       */
    CGPU_BSDF_ABSORBER = 3,         /* "absorb"                absorberBsdf.cpp             */
    CGPU_BSDF_DIELECTRIC_GGX = 4,   /* "dielectric-microfacet" (no reference counterpart)   */
    CGPU_BSDF_MIRROR = 5,           /* "mirror"                specularReflection.cpp       */
    CGPU_BSDF_PHONG = 6,            /* "phong"                 phongBsdf.cpp                */
    CGPU_BSDF_PLASTIC = 7           /* "plastic": MixedBsdf(Lambertian, Phong, ratio)
                                                               mixedBsdf.cpp, bsdfInstantiator.cpp:104-116 */
};
/* Fresnel term of a mirror (bsdfInstantiator.cpp:38-64). */
enum { CGPU_FRESNEL_CONDUCTOR = 0, CGPU_FRESNEL_DIELECTRIC = 1 };

typedef struct cgpu_material {
    int32_t type;            /* CGPU_BSDF_* */
    int32_t albedo_texture;  /* index into cgpu_scene_desc.textures, or -1 for constant albedo */
    float albedo[3];         /* albedo; plastic: diffuse albedo */
    float f0[3];             /* Schlick F0 of the conductor (and of a conductor-Fresnel mirror) */
    float roughness;         /* CRSD "roughness"; alpha = max(max(r, 1e-3)^2, 1e-3) */
    float ior_outer;
    float ior_inner;
    float exponent;          /* phong "exponent", plastic "specular-exponent" */
    float diffuse_ratio;     /* plastic "diffuse-ratio" */
    int32_t fresnel;         /* mirror: CGPU_FRESNEL_* */
    int32_t reserved[2];
} cgpu_material;

/* RGB float texture, nearest texel with repeat wrap (rgbImageTexture.cpp:8-15). */
typedef struct cgpu_texture {
    int32_t width;
    int32_t height;
    const float* texels; /* width * height * 3, row-major; row y holds v in [y / height, (y + 1) / height),
                            so row 0 is the picture's bottom row (the reference lays pictures out
                            bottom-up: its loader flips them vertically, file-io/pictureLoader.cpp) */
} cgpu_texture;

/* One-sided area emitter on a primitive (singleAreaLight.cpp:20-37):
 * L = color / sum(color) * watt / (area * pi). */
typedef struct cgpu_area_light {
    int32_t primitive;       /* index into the primitive arrays */
    float color[3];
    float watt;
    int32_t back_face_emit;
} cgpu_area_light;

/* Film reconstruction filter (filterInstantiator.cpp:16-57, filters under
 * core/film/filter/).  As FilmTile::addSample does (filmTile.cpp:36-66), a
 * sample at film position (x, y) adds weight w = filter(pixel centre - (x, y))
 * to every pixel within half the filter's size of it, clipped to the film
 * tile (tile_width x tile_height pixels, from the film's origin) its own pixel
 * lies in; the film then holds sum w L, sum w L^2 and sum w per pixel.
 * A zero-initialised filter is the reference's default box of size 1 (the
 * sample's own pixel, weight 1): width / height 0 mean 1 for CGPU_FILTER_BOX,
 * tile sizes 0 mean 16.  Gaussian, Mitchell and cone filters use the fields as
 * given (the CRSD loader fills in the reference's defaults). */
enum {
    CGPU_FILTER_BOX = 0,       /* weight 1 (boxFilter.cpp:9-11) */
    CGPU_FILTER_GAUSSIAN = 1,  /* max(0, a exp(-x^2 / 2 sx^2 - y^2 / 2 sy^2) - edge value) (gaussianFilter.cpp:9-38) */
    CGPU_FILTER_MITCHELL = 2,  /* Mitchell-Netravali (b, c), separable (mitchellFilter.cpp:17-42) */
    CGPU_FILTER_CONE = 3       /* max(w/2 - |x|, 0) max(h/2 - |y|, 0) (coneFilter.cpp:11-15) */
};
typedef struct cgpu_film_filter {
    int32_t type;                       /* CGPU_FILTER_* */
    float width, height;                /* full size in pixels */
    float sigma_x, sigma_y, amplitude;  /* gaussian */
    float b, c;                         /* mitchell */
    int32_t tile_width, tile_height;    /* film tile clipping the footprint */
} cgpu_film_filter;

typedef struct cgpu_scene_desc {
    /* film + camera (filmInstantiator.cpp:13-30, cameraInstantiator.cpp:27-45) */
    int32_t width;
    int32_t height;
    float cam_position[3];
    float cam_direction[3];
    float cam_up[3];
    float fov_degrees;       /* horizontal FOV over the sensor width */
    float sensor_width_mm;   /* reference default 36 */
    /* estimator (estimatorInstantiator.cpp:18-24) */
    int32_t max_depth;
    int32_t spp;             /* sample count of one full render (strata layout) */

    /* primitives in the reference's creation order */
    uint32_t num_primitives;
    const int32_t* prim_kind;      /* CGPU_PRIM_*; NULL means every primitive is a triangle */
    const float* prim_vertices;    /* 9 floats per primitive: triangle vA vB vC, rectangle v1 v2 v3 */
    const float* prim_normals;     /* optional, 9 per primitive (triangle vertex normals) */
    const float* prim_uvws;        /* optional, 9 per primitive (triangle vertex uvw) */
    const int32_t* prim_material;  /* one material index per primitive */

    uint32_t num_materials;
    const cgpu_material* materials;
    uint32_t num_textures;
    const cgpu_texture* textures;
    uint32_t num_lights;
    const cgpu_area_light* lights;

    /* Environment light (environmentLight.cpp:16-105): 1 + index into
     * `textures` of an RGB latitude-longitude radiance map lighting the scene
     * from infinity, 0 for none.  It joins the uniform light pick after the
     * area lights. */
    int32_t environment_texture;

    /* Light selection (CRSD light-cluster block, lightClusterInstantiator.cpp:21-45):
     * CGPU_LIGHT_CLUSTER_UNIFORM picks every light with the same probability
     * (uniformLightCluster.cpp:15-24); CGPU_LIGHT_CLUSTER_POWER in proportion to
     * its approximate flux, computed once at upload (powerLightCluster.cpp:9-48). */
    int32_t light_cluster;

    cgpu_film_filter filter;
} cgpu_scene_desc;

enum { CGPU_LIGHT_CLUSTER_UNIFORM = 0, CGPU_LIGHT_CLUSTER_POWER = 1 };

typedef struct cgpu_scene_info {
    uint32_t num_primitives;
    uint32_t num_triangles;   /* rectangles count twice */
    uint32_t num_bvh_nodes;   /* 4-wide quantized nodes of 64 B */
    uint32_t num_lights;
    uint64_t device_bytes;    /* scene + BVH bytes resident on the device */
    double build_ms;          /* whole scene build + upload time */
    float bounds_min[3];
    float bounds_max[3];
    double bvh_ms;            /* BVH build alone */
    int32_t bvh_builder;      /* CGPU_BVH_BUILDER_HOST_SAH, _GPU_PLOC or _GPU_SAH: the one used */
    int32_t reserved;
} cgpu_scene_info;

/* BVH builder of the following uploads (cgpu_set_bvh_builder):
 *   AUTO      GPU_PLOC from CGPU_BVH_GPU_MIN_PRIMITIVES primitives up with more than
 *             CGPU_BVH_GPU_MIN_PRIMS_PER_SAMPLE primitives per path sample of one full render
 *             (width * height * spp), where its faster build outweighs its 12-25 % slower tree; else
 *             GPU_SAH from CGPU_BVH_GPU_SAH_MIN_PRIMITIVES primitives up; else HOST_SAH (default)
 *   HOST_SAH  binned SAH on the host threads (bvh_build.cpp)
 *   GPU_PLOC  parallel locally-ordered clustering on the GPU (bvh_gpu.cu)
 *   GPU_SAH   the host build's binned SAH run on the GPU (bvh_sah_gpu.cu): the same tree but below
 *             the host's unstable-partition median splits, 14-22x faster than the host
 * Renders do not depend on the builder: closest hits keep, on an exact tie
 * of distance, the lower primitive index, whatever the tree. */
enum { CGPU_BVH_BUILDER_AUTO = 0, CGPU_BVH_BUILDER_HOST_SAH = 1, CGPU_BVH_BUILDER_GPU_PLOC = 2, CGPU_BVH_BUILDER_GPU_SAH = 3 };
#define CGPU_BVH_GPU_MIN_PRIMITIVES 1000000
#define CGPU_BVH_GPU_MIN_PRIMS_PER_SAMPLE 0.01
#define CGPU_BVH_GPU_SAH_MIN_PRIMITIVES 65536

/* -------------------------------------------------------------- context -- */

typedef struct cgpu_options {
    int32_t device;             /* CUDA device ordinal */
    void* stream;               /* cudaStream_t to launch on; NULL: the library creates one */
    uint32_t max_paths;         /* paths in flight per wavefront batch; 0 = automatic */
    int32_t flags;              /* reserved, 0 */
} cgpu_options;

cgpu_status cgpu_create(cgpu_ctx** out_ctx, const cgpu_options* options);
void cgpu_destroy(cgpu_ctx* ctx);
const char* cgpu_last_error(const cgpu_ctx* ctx);
const char* cgpu_status_string(cgpu_status status);
int32_t cgpu_abi_version(void);
/* Waits for the context stream; CGPU_ERR_TIMEOUT if a traversal since the
 * last check ran out of its visit budget (below). */
cgpu_status cgpu_synchronize(cgpu_ctx* ctx);

/* Device-side iteration budget of every BVH traversal (no counterpart in the
 * reference, whose accelerator asserts and aborts on a broken tree,
 * fundamental/assertion.cpp:14-25): a ray that makes more than `visits` node
 * and leaf visits stops, keeps the hit it holds (or none) and is counted on
 * the device, so a corrupted tree cannot keep a kernel running.  0 (the
 * default) is 5 x the scene's nodes + 64 per ray, which a correct traversal
 * never reaches: it reaches every inner node and every leaf at most once.
 * Asynchronous calls (cgpu_render, cgpu_trace_*_device) do not wait for the
 * count; the next call that synchronises the context - cgpu_synchronize,
 * cgpu_film_read, cgpu_trace_closest / _any, cgpu_path_radiance,
 * cgpu_render_paths, cgpu_adjoint_forward / _backward - returns
 * CGPU_ERR_TIMEOUT with the number of rays in cgpu_last_error and resets the
 * count; results computed since the previous check are then not valid, and
 * the context stays usable. */
cgpu_status cgpu_set_visit_budget(cgpu_ctx* ctx, uint32_t visits);

cgpu_status cgpu_set_bvh_builder(cgpu_ctx* ctx, int32_t builder);

/* Which of two primitives a closest-hit query keeps when the reference's own
 * test meets both at the same distance (coplanar overlapping primitives; a
 * ray through an edge two triangles share).  CGPU_TIE_ORDER_REFERENCE (the
 * default): the one the reference's BVH traversal reaches last
 * (bvhAccelerator.cpp:40-97 with triangle.cpp:81-86) - each upload builds the
 * reference's binary SAH tree on host threads beside the BVH build (about
 * 0.4 s per million primitives on 8 cores) and keeps 32 bytes per primitive
 * on the device.  CGPU_TIE_ORDER_INDEX: the lower primitive index, without
 * that build.  Applies to scenes uploaded afterwards. */
enum { CGPU_TIE_ORDER_REFERENCE = 0, CGPU_TIE_ORDER_INDEX = 1 };
cgpu_status cgpu_set_tie_order(cgpu_ctx* ctx, int32_t order);

cgpu_status cgpu_scene_upload(cgpu_ctx* ctx, const cgpu_scene_desc* desc, int32_t* out_scene);
cgpu_status cgpu_scene_release(cgpu_ctx* ctx, int32_t scene);
cgpu_status cgpu_scene_info_get(cgpu_ctx* ctx, int32_t scene, cgpu_scene_info* out_info);

/* ------------------------------------------------------------ ray queries -- */

/* 32-byte ray: origin, t_min, direction, t_max.  The direction is
 * normalised by the call, as the reference's Ray constructor does. */
typedef struct cgpu_ray {
    float org[3];
    float t_min;
    float dir[3];
    float t_max;
} cgpu_ray;

/* Closest hit: primitive = -1 on a miss.  t is the distance the reference
 * reports for that primitive (Moller-Trumbore for a triangle, the plane
 * distance for a rectangle); u, v are the barycentrics of vB and vC of a
 * triangle, recomputed from the hit point, or a rectangle's edge
 * coordinates (both divided by |eA|). */
typedef struct cgpu_hit {
    float t;
    int32_t primitive;
    float u;
    float v;
} cgpu_hit;

/* Host buffers in and out; copies are made on the context stream. */
cgpu_status cgpu_trace_closest(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* rays, uint32_t n, cgpu_hit* hits);
cgpu_status cgpu_trace_any(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* rays, uint32_t n, uint8_t* occluded);
/* Device buffers (already resident); asynchronous on the context stream. */
cgpu_status cgpu_trace_closest_device(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* d_rays, uint32_t n, cgpu_hit* d_hits);
cgpu_status cgpu_trace_any_device(cgpu_ctx* ctx, int32_t scene, const cgpu_ray* d_rays, uint32_t n, uint8_t* d_occluded);

/* Primary rays for film positions (x right, y down, in pixels): 6 floats (org, dir) each. */
cgpu_status cgpu_camera_rays(cgpu_ctx* ctx, int32_t scene, const double* film_xy, uint32_t n, float* out_rays);

/* --------------------------------------------------------------- render -- */

enum { CGPU_MODE_MEGAKERNEL = 0, CGPU_MODE_WAVEFRONT = 1 };

typedef struct cgpu_render_params {
    const int32_t* scenes;     /* scene ids rendered together (one launch sequence) */
    uint32_t num_scenes;
    uint32_t first_sample;     /* samples [first_sample, first_sample + num_samples) */
    uint32_t num_samples;      /* per pixel */
    uint64_t seed;
    int32_t mode;              /* CGPU_MODE_* */
    int32_t use_graph;         /* wavefront: replay a captured CUDA graph per pass */
    /* optional, one per scene: scene i renders samples
     * [first_sample, first_sample + scene_samples[i]); NULL: num_samples for all */
    const uint32_t* scene_samples;
} cgpu_render_params;

/* Accumulates into each scene's FP64 film on the device (asynchronous). */
cgpu_status cgpu_render(cgpu_ctx* ctx, const cgpu_render_params* params);
cgpu_status cgpu_film_clear(cgpu_ctx* ctx, int32_t scene);
/* Film read-back: each pointer may be NULL; sizes width*height*3 / *3 / *1 doubles. */
cgpu_status cgpu_film_read(cgpu_ctx* ctx, int32_t scene, double* sum_rgb, double* sum_sq_rgb, double* count);

/* Allocation-free variant of cgpu_render (no counterpart in the reference):
 * the wavefront render of samples [first_sample, first_sample + num_samples)
 * of one scene into its film, with every device buffer of the call in one
 * static 80 MiB array of this library instead of memory from cudaMalloc.
 * For callers that must not allocate or free device memory at render time
 * (cudaMalloc / cudaFree synchronise the device and may fail under memory
 * pressure): a caller with its own memory budget, or one that keeps a render
 * inside a latency-bound loop.  Same kernels, paths and results as
 * cgpu_render (the film may differ in the last FP64 bits: batches split
 * differently).  Limits, else CGPU_ERR_INVALID_ARGUMENT with the reason in
 * cgpu_last_error: width * height <= 262144 pixels, max_depth <= 62, scene
 * id < 64.  Nothing in the scratch needs to start at zero: each batch's
 * setup kernel zeroes the queue counters and writes the batch tables, and
 * generate writes every path's state before it is read.  The first call on
 * a device looks the scratch up (cudaGetSymbolAddress) and, with lazy module
 * loading, loads the library's device code, which reserves the array: make
 * one call before relying on the no-allocation property.  One scratch per
 * device and process: calls that overlap in time (any contexts, streams or
 * threads on one device) race on it and must be serialised by the caller.
 * Asynchronous on the context stream, like cgpu_render.  Counting
 * (cgpu_set_counting) and per-kernel timing (cgpu_set_profiling) do not
 * apply to this call: afterwards cgpu_render_stats_get reports its paths,
 * batches and kernel launches, and zero for the ray, node and triangle
 * counters and for h2d_bytes (it copies nothing). */
cgpu_status cgpu_render_noalloc(cgpu_ctx* ctx, int32_t scene, uint32_t first_sample, uint32_t num_samples,
                                uint64_t seed);

/* Per-path estimate for given film positions and path keys (path stream starts
 * at draw 0 with the estimator).  out_rgb: 3 floats per path. */
cgpu_status cgpu_path_radiance(cgpu_ctx* ctx, int32_t scene, int32_t mode, const double* film_xy,
                               const uint64_t* keys, uint32_t n, float* out_rgb);
/* Per-path radiance of a render pass layout: pixel-major within each sample,
 * out_rgb: num_samples * width * height * 3 floats (does not touch the film). */
cgpu_status cgpu_render_paths(cgpu_ctx* ctx, int32_t scene, int32_t mode, uint32_t first_sample,
                              uint32_t num_samples, uint64_t seed, float* out_rgb);

/* Device-side counters of the last render (for throughput and roofline). */
typedef struct cgpu_render_stats {
    uint64_t paths;
    uint64_t closest_rays;        /* counting renders only (cgpu_set_counting), else 0 */
    uint64_t any_rays;
    uint64_t node_visits;         /* 4-wide nodes fetched by closest-hit rays */
    uint64_t triangle_tests;      /* triangles tested by closest-hit rays */
    uint64_t any_node_visits;     /* ... by any-hit rays */
    uint64_t any_triangle_tests;
    uint64_t h2d_bytes;           /* host->device bytes the last cgpu_render copied (batch tables) */
    uint32_t kernel_launches;     /* kernels this library launched in the last cgpu_render */
    uint32_t batches;             /* path batches the last cgpu_render ran */
    uint64_t tie_rays;            /* counting renders: closest-hit rays the persistent pass left to the tie rule */
} cgpu_render_stats;
cgpu_status cgpu_render_stats_get(cgpu_ctx* ctx, cgpu_render_stats* out_stats);
/* Count rays, node fetches and triangle tests in every following render (slower). */
cgpu_status cgpu_set_counting(cgpu_ctx* ctx, int32_t enabled);

/* ------------------------------------------------------------ autotune -- */
typedef struct cgpu_tuning {
    int32_t block_trace;   /* threads per block: extend, shadow and megakernel (32..1024, multiple of 32) */
    int32_t block_shade;   /* threads per block: shade-by-BSDF kernels */
    uint32_t max_paths;    /* paths in flight per wavefront batch; 0 = automatic (2^21, at least one frame) */
    int32_t traversal;     /* 0: one ray per thread per grid-stride step; 1: persistent warps that hand a
                              finished lane the next ray at once; 2: persistent while-while closest-hit
                              pass that refills a warp's finished lanes once fewer than refill_closest
                              of its lanes still trace; 3: 2 plus the same persistent while-while form
                              for the any-hit pass (refill_any) */
    int32_t reorder;       /* 1, 2, 3: before each closest-hit pass after the first, sort its rays by
                              direction octant and origin (Morton order of 9, 7 or 4 bits per axis in the
                              scene bounds; 4, 3 or 2 radix passes), so that a warp traces neighbouring
                              rays (traversal 0, 2 and 3); 4: by direction octant alone (one radix pass);
                              0: queue order (default; cgpu_autotune does not search it: on the
                              1 M-triangle field the sort costs about what it saves) */
    int32_t refill_closest;/* queue compaction of the persistent closest-hit pass (traversal 2 and 3):
                              after each round of leaves a warp whose unfinished rays number fewer than
                              this stores its finished lanes' hits and takes the next rays of the queue
                              for them; 1..32, 0 = 24 */
    int32_t refill_any;    /* the same threshold for the persistent any-hit pass (traversal 3); 0 = 24 */
} cgpu_tuning;
cgpu_status cgpu_tuning_get(cgpu_ctx* ctx, cgpu_tuning* out_tuning);
cgpu_status cgpu_tuning_set(cgpu_ctx* ctx, const cgpu_tuning* tuning);
/* Times wavefront passes of `scenes` (`samples` samples each) over a small
 * search of cgpu_tuning values (traversal variant, block sizes, the refill
 * thresholds of the persistent passes, 2^20..2^24 paths in flight) and
 * applies the fastest.  With a cache path, a result
 * stored for the same GPU, scene sizes and sample count is reused without
 * timing and new results are appended (one JSON object per line). */
cgpu_status cgpu_autotune(cgpu_ctx* ctx, const int32_t* scenes, uint32_t num_scenes, uint32_t samples,
                          const char* cache_path, cgpu_tuning* out_tuning);

/* -------------------------------------------------------------- adjoint -- */
/* Differentiable parameters of an uploaded scene: the texels of every albedo
 * texture (concatenated in texture order, RGB floats), one GGX roughness per
 * material (CRSD "roughness"), one emitted radiance RGB per area light. */
typedef struct cgpu_param_counts {
    uint64_t texel_floats;
    uint32_t materials;
    uint32_t lights;
} cgpu_param_counts;
cgpu_status cgpu_param_counts_get(cgpu_ctx* ctx, int32_t scene, cgpu_param_counts* out_counts);
/* Any pointer may be NULL to skip that group. */
cgpu_status cgpu_params_get(cgpu_ctx* ctx, int32_t scene, float* texels, float* roughness, float* radiance);
cgpu_status cgpu_params_set(cgpu_ctx* ctx, int32_t scene, const float* texels, const float* roughness,
                            const float* radiance);
/* Forward pass: clears the film, renders samples [0, spp) with `seed` and
 * returns the mean image (width * height * 3 floats; may be NULL). */
cgpu_status cgpu_adjoint_forward(cgpu_ctx* ctx, int32_t scene, uint32_t spp, uint64_t seed, float* image_out);
/* Backward pass: replays the same path samples from their seeds and writes
 * d loss / d parameter (FP64) for d loss / d image (width * height * 3
 * floats, host).  Output arrays are overwritten; any may be NULL. */
cgpu_status cgpu_adjoint_backward(cgpu_ctx* ctx, int32_t scene, uint32_t spp, uint64_t seed,
                                  const float* d_loss_d_image, double* grad_texels, double* grad_roughness,
                                  double* grad_radiance);
/* Schedule of cgpu_adjoint_backward: CGPU_MODE_WAVEFRONT (default; a forward
 * wavefront pass for each path's radiance, then a wavefront replay with a
 * gradient kernel after each traversal pass) or CGPU_MODE_MEGAKERNEL (one
 * thread replays one path twice).  Both compute the same estimator on the
 * same path samples; they differ in FP64 summation order only. */
cgpu_status cgpu_set_adjoint_mode(cgpu_ctx* ctx, int32_t mode);

/* Per-kernel CUDA-event timing of the following renders (launches are made
 * one by one instead of through the captured graph while it is on, and the
 * shadow pass runs after the extend pass instead of beside it, so that each
 * kernel is timed alone). */
enum {
    CGPU_KERNEL_GENERATE = 0,
    CGPU_KERNEL_EXTEND = 1,     /* closest-hit traversal of continuation rays */
    CGPU_KERNEL_SHADOW = 2,     /* any-hit traversal */
    CGPU_KERNEL_SHADE = 3,      /* all shade-by-BSDF kernels */
    CGPU_KERNEL_SPLAT = 4,
    CGPU_KERNEL_MEGAKERNEL = 5,
    CGPU_KERNEL_REORDER = 6,    /* sort keys + radix sort of a closest-hit queue (tuning.reorder) */
    CGPU_KERNEL_MIS_OCCL = 7,   /* MIS rays that meet their light: is a primitive before the light's hit */
    CGPU_KERNEL_TIES = 8,       /* closest-hit rays the persistent pass left to the tie rule (cgpu_set_tie_order) */
    CGPU_KERNEL_CLASSES = 9
};
typedef struct cgpu_kernel_times {
    double ms[CGPU_KERNEL_CLASSES];
    uint32_t launches[CGPU_KERNEL_CLASSES];
} cgpu_kernel_times;
cgpu_status cgpu_set_profiling(cgpu_ctx* ctx, int32_t enabled);
/* Totals over the last cgpu_render call. */
cgpu_status cgpu_kernel_times_get(cgpu_ctx* ctx, cgpu_kernel_times* out_times);

#ifdef __cplusplus
}
#endif

#endif /* CADISE_GPU_H */
