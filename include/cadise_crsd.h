/*
 * cadise_crsd.h - CRSD scene loading for the GB300 path tracer (C ABI).
 *
 * Parses the reference renderer's scene description format (CRSD) into the
 * flat cgpu_scene_desc of cadise_gpu.h.  Replaces, for this library:
 *
 *   SdParser::parseSd                (source/file-io/scene-description/sdParser.cpp:19-61)
 *   Tokenizer::tokenize              (source/file-io/scene-description/tokenizer.cpp:12-246)
 *   SdData::find* / get*Texture      (source/file-io/scene-description/sdData.h:40-63, sdData.cpp:98-140)
 *   RenderDatabase::setUpData        (source/core/renderDatabase.cpp:39-76)
 *   instantiator::makePrimitive / makeBsdf / makeLight / make*Texture / makeCamera /
 *   makeFilm / makeRenderer settings (source/core/instantiator/*.cpp)
 *
 * Host-only: no GPU is touched.  Errors are returned as status codes with a
 * message, never by exiting the process (the reference exits on a missing
 * file, sdParser.cpp:39-42).
 */
#ifndef CADISE_CRSD_H
#define CADISE_CRSD_H

#include "cadise_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cgpu_crsd_scene cgpu_crsd_scene;

typedef struct cgpu_crsd_settings {
    char renderer_type[32];   /* "sampling" or "cuda-sampling" */
    char estimator[16];       /* "pt" */
    char sampler[16];         /* "stratified" | "random" */
    char output_filename[256];
    int32_t spp;              /* renderer sample-number (default 4) */
    int32_t max_depth;        /* estimator max-depth (default 10000) */
    int32_t mode;             /* CGPU_MODE_* from [mode string "wavefront" | "megakernel"] */
    int32_t use_graph;        /* [graph bool], default true */
    uint64_t seed;            /* [seed int32], default 1 */
} cgpu_crsd_settings;

/* err (optional) receives a NUL-terminated message on failure. */
cgpu_status cgpu_crsd_load_file(const char* path, cgpu_crsd_scene** out_scene, char* err, size_t err_len);
cgpu_status cgpu_crsd_load_text(const char* text, size_t len, cgpu_crsd_scene** out_scene, char* err,
                                size_t err_len);
/* The scene as a cgpu_scene_desc; valid until cgpu_crsd_free. */
const cgpu_scene_desc* cgpu_crsd_desc(const cgpu_crsd_scene* scene);
cgpu_status cgpu_crsd_settings_get(const cgpu_crsd_scene* scene, cgpu_crsd_settings* out_settings);
/* Index of the first primitive created under `name` (the reference's name map
 * keeps the first), or -1. */
int32_t cgpu_crsd_primitive_index(const cgpu_crsd_scene* scene, const char* name);
void cgpu_crsd_free(cgpu_crsd_scene* scene);

#ifdef __cplusplus
}
#endif

#endif /* CADISE_CRSD_H */
