"""ctypes mirror of ``include/cadise_gpu.h`` and scene flattening.

:func:`flatten` turns a :class:`cadise_gb300.scenes.SceneSpec` into the flat,
caller-owned arrays of ``cgpu_scene_desc`` (primitives in the reference's
creation order: one per rectangle, one per mesh triangle - the order
``instantiator::makePrimitive`` appends intersectors in,
``source/core/instantiator/primitiveInstantiator.cpp:92-129``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List

import numpy as np

from . import scenes as S

CGPU_PRIM_TRIANGLE = 0
CGPU_PRIM_RECTANGLE = 1
CGPU_PRIM_SPHERE = 2

CGPU_BSDF_LAMBERTIAN = 0
CGPU_BSDF_CONDUCTOR_GGX = 1
CGPU_BSDF_GLASS = 2
CGPU_BSDF_ABSORBER = 3
CGPU_BSDF_DIELECTRIC_GGX = 4
CGPU_BSDF_MIRROR = 5
CGPU_BSDF_PHONG = 6
CGPU_BSDF_PLASTIC = 7

CGPU_MODE_MEGAKERNEL = 0
CGPU_MODE_WAVEFRONT = 1

BSDF_OF_TYPE = {
    S.LAMBERT: CGPU_BSDF_LAMBERTIAN,
    S.CONDUCTOR: CGPU_BSDF_CONDUCTOR_GGX,
    S.GLASS: CGPU_BSDF_GLASS,
    S.ROUGH_DIELECTRIC: CGPU_BSDF_DIELECTRIC_GGX,
    "absorb": CGPU_BSDF_ABSORBER,
    S.MIRROR: CGPU_BSDF_MIRROR,
    S.PHONG: CGPU_BSDF_PHONG,
    S.PLASTIC: CGPU_BSDF_PLASTIC,
}

STATUS_NAMES = {0: "CGPU_OK", 1: "CGPU_ERR_INVALID_ARGUMENT", 2: "CGPU_ERR_CUDA",
                3: "CGPU_ERR_OUT_OF_MEMORY", 4: "CGPU_ERR_TIMEOUT", 5: "CGPU_ERR_UNSUPPORTED",
                6: "CGPU_ERR_NOT_FOUND", 7: "CGPU_ERR_PARSE", 8: "CGPU_ERR_NO_DEVICE"}


class cgpu_material(C.Structure):
    _fields_ = [("type", C.c_int32), ("albedo_texture", C.c_int32), ("albedo", C.c_float * 3),
                ("f0", C.c_float * 3), ("roughness", C.c_float), ("ior_outer", C.c_float),
                ("ior_inner", C.c_float), ("exponent", C.c_float), ("diffuse_ratio", C.c_float),
                ("fresnel", C.c_int32), ("reserved", C.c_int32 * 2)]


class cgpu_texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("texels", C.POINTER(C.c_float))]


class cgpu_area_light(C.Structure):
    _fields_ = [("primitive", C.c_int32), ("color", C.c_float * 3), ("watt", C.c_float),
                ("back_face_emit", C.c_int32)]


CGPU_FILTER_BOX = 0
CGPU_FILTER_GAUSSIAN = 1
CGPU_FILTER_MITCHELL = 2
CGPU_FILTER_CONE = 3
FILTER_OF_NAME = {"box": CGPU_FILTER_BOX, "gaussian": CGPU_FILTER_GAUSSIAN, "mitchell": CGPU_FILTER_MITCHELL,
                  "cone": CGPU_FILTER_CONE}


class cgpu_film_filter(C.Structure):
    _fields_ = [("type", C.c_int32), ("width", C.c_float), ("height", C.c_float),
                ("sigma_x", C.c_float), ("sigma_y", C.c_float), ("amplitude", C.c_float),
                ("b", C.c_float), ("c", C.c_float), ("tile_width", C.c_int32), ("tile_height", C.c_int32)]


def film_filter_struct(f) -> "cgpu_film_filter":
    """cgpu_film_filter of a scenes.FilmFilter (None: the default box)."""
    out = cgpu_film_filter()
    if f is None:
        return out
    out.type = FILTER_OF_NAME[f.type]
    out.width, out.height = f.size()
    out.sigma_x, out.sigma_y, out.amplitude = f.sigma_x, f.sigma_y, f.amplitude
    out.b, out.c = f.b, f.c
    out.tile_width, out.tile_height = f.tile
    return out


class cgpu_scene_desc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("cam_position", C.c_float * 3), ("cam_direction", C.c_float * 3), ("cam_up", C.c_float * 3),
                ("fov_degrees", C.c_float), ("sensor_width_mm", C.c_float),
                ("max_depth", C.c_int32), ("spp", C.c_int32),
                ("num_primitives", C.c_uint32), ("prim_kind", C.POINTER(C.c_int32)),
                ("prim_vertices", C.POINTER(C.c_float)), ("prim_normals", C.POINTER(C.c_float)),
                ("prim_uvws", C.POINTER(C.c_float)), ("prim_material", C.POINTER(C.c_int32)),
                ("num_materials", C.c_uint32), ("materials", C.POINTER(cgpu_material)),
                ("num_textures", C.c_uint32), ("textures", C.POINTER(cgpu_texture)),
                ("num_lights", C.c_uint32), ("lights", C.POINTER(cgpu_area_light)),
                ("environment_texture", C.c_int32), ("light_cluster", C.c_int32),
                ("filter", cgpu_film_filter)]


class cgpu_scene_info(C.Structure):
    _fields_ = [("num_primitives", C.c_uint32), ("num_triangles", C.c_uint32),
                ("num_bvh_nodes", C.c_uint32), ("num_lights", C.c_uint32),
                ("device_bytes", C.c_uint64), ("build_ms", C.c_double),
                ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("bvh_ms", C.c_double), ("bvh_builder", C.c_int32), ("reserved", C.c_int32)]


CGPU_BVH_BUILDER_AUTO = 0
CGPU_BVH_BUILDER_HOST_SAH = 1
CGPU_BVH_BUILDER_GPU_PLOC = 2
CGPU_BVH_BUILDER_GPU_SAH = 3

CGPU_BVH_GPU_MIN_PRIMITIVES = 1000000
CGPU_BVH_GPU_MIN_PRIMS_PER_SAMPLE = 0.01
CGPU_BVH_GPU_SAH_MIN_PRIMITIVES = 65536

CGPU_TIE_ORDER_REFERENCE = 0
CGPU_TIE_ORDER_INDEX = 1


class cgpu_options(C.Structure):
    _fields_ = [("device", C.c_int32), ("stream", C.c_void_p), ("max_paths", C.c_uint32),
                ("flags", C.c_int32)]


class cgpu_ray(C.Structure):
    _fields_ = [("org", C.c_float * 3), ("t_min", C.c_float), ("dir", C.c_float * 3), ("t_max", C.c_float)]


class cgpu_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("primitive", C.c_int32), ("u", C.c_float), ("v", C.c_float)]


class cgpu_render_params(C.Structure):
    _fields_ = [("scenes", C.POINTER(C.c_int32)), ("num_scenes", C.c_uint32),
                ("first_sample", C.c_uint32), ("num_samples", C.c_uint32), ("seed", C.c_uint64),
                ("mode", C.c_int32), ("use_graph", C.c_int32), ("scene_samples", C.POINTER(C.c_uint32))]


class cgpu_render_stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("closest_rays", C.c_uint64), ("any_rays", C.c_uint64),
                ("node_visits", C.c_uint64), ("triangle_tests", C.c_uint64),
                ("any_node_visits", C.c_uint64), ("any_triangle_tests", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("kernel_launches", C.c_uint32), ("batches", C.c_uint32),
                ("tie_rays", C.c_uint64)]


class cgpu_crsd_settings(C.Structure):
    _fields_ = [("renderer_type", C.c_char * 32), ("estimator", C.c_char * 16), ("sampler", C.c_char * 16),
                ("output_filename", C.c_char * 256), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("mode", C.c_int32), ("use_graph", C.c_int32), ("seed", C.c_uint64)]


class cgpu_tuning(C.Structure):
    _fields_ = [("block_trace", C.c_int32), ("block_shade", C.c_int32), ("max_paths", C.c_uint32),
                ("traversal", C.c_int32), ("reorder", C.c_int32), ("refill_closest", C.c_int32),
                ("refill_any", C.c_int32)]


class cgpu_param_counts(C.Structure):
    _fields_ = [("texel_floats", C.c_uint64), ("materials", C.c_uint32), ("lights", C.c_uint32)]


class cgpu_kernel_times(C.Structure):
    _fields_ = [("ms", C.c_double * 9), ("launches", C.c_uint32 * 9)]


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@dataclass
class FlatScene:
    """Owns the numpy arrays a ``cgpu_scene_desc`` points into."""
    desc: cgpu_scene_desc
    kind: np.ndarray
    vertices: np.ndarray
    material: np.ndarray
    normals: object
    uvws: object
    materials: object
    lights: object
    textures: object
    texture_arrays: list
    prim_names: Dict[str, int]
    material_names: Dict[str, int]

    @property
    def ptr(self):
        return C.byref(self.desc)


def flatten(spec: "S.SceneSpec") -> FlatScene:
    mat_index = {m.name: i for i, m in enumerate(spec.materials)}
    tex_index = {t.name: i for i, t in enumerate(spec.textures)}
    n = spec.num_primitives()
    kind = np.zeros(n, dtype=np.int32)
    verts = np.zeros((n, 9), dtype=np.float32)
    mat = np.zeros(n, dtype=np.int32)
    has_normals = any(isinstance(p, S.TriangleMesh) and p.normals is not None for p in spec.primitives)
    has_uvws = any(isinstance(p, S.TriangleMesh) and p.uvws is not None for p in spec.primitives)
    normals = np.zeros((n, 9), dtype=np.float32) if has_normals else None
    uvws = None
    if has_uvws:
        uvws = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], dtype=np.float32), (n, 1))
    names: Dict[str, int] = {}
    i = 0
    for p in spec.primitives:
        if isinstance(p, (S.Rectangle, S.Triangle)):
            kind[i] = CGPU_PRIM_RECTANGLE if isinstance(p, S.Rectangle) else CGPU_PRIM_TRIANGLE
            verts[i] = np.array([*p.v1, *p.v2, *p.v3], dtype=np.float32)
            mat[i] = mat_index[p.material]
            names.setdefault(p.name, i)
            i += 1
        elif isinstance(p, S.Sphere):
            kind[i] = CGPU_PRIM_SPHERE
            verts[i, :4] = np.array([*p.center, p.radius], dtype=np.float32)
            mat[i] = mat_index[p.material]
            names.setdefault(p.name, i)
            i += 1
        else:
            m = p.positions.shape[0]
            kind[i:i + m] = CGPU_PRIM_TRIANGLE
            verts[i:i + m] = p.positions.reshape(m, 9)
            mat[i:i + m] = mat_index[p.material]
            if normals is not None and p.normals is not None:
                normals[i:i + m] = p.normals.reshape(m, 9)
            if uvws is not None and p.uvws is not None:
                uvws[i:i + m] = p.uvws.reshape(m, 9)
            # the reference's name map keeps the first triangle of a mesh
            names.setdefault(p.name, i)
            i += m
    mats = (cgpu_material * max(1, len(spec.materials)))()
    for j, m in enumerate(spec.materials):
        mats[j].type = BSDF_OF_TYPE[m.type]
        mats[j].albedo_texture = tex_index[m.albedo_texture] if m.albedo_texture else -1
        mats[j].albedo[:] = [float(x) for x in m.albedo]
        mats[j].f0[:] = [float(x) for x in m.f0]
        mats[j].roughness = float(m.roughness)
        mats[j].ior_outer = float(m.ior_outer)
        mats[j].ior_inner = float(m.ior_inner)
        mats[j].exponent = float(m.exponent)
        mats[j].diffuse_ratio = float(m.diffuse_ratio)
        mats[j].fresnel = 1 if m.fresnel == "dielectric" else 0
    lights = (cgpu_area_light * max(1, len(spec.lights)))()
    for j, lt in enumerate(spec.lights):
        lights[j].primitive = names[lt.primitive]
        lights[j].color[:] = [float(x) for x in lt.color]
        lights[j].watt = float(lt.watt)
        lights[j].back_face_emit = 1 if lt.back_face_emit else 0
    tex_arrays = [np.ascontiguousarray(t.texels, dtype=np.float32) for t in spec.textures]
    texs = (cgpu_texture * max(1, len(spec.textures)))()
    for j, a in enumerate(tex_arrays):
        texs[j].height, texs[j].width = int(a.shape[0]), int(a.shape[1])
        texs[j].texels = _fptr(a)
    d = cgpu_scene_desc()
    d.width, d.height = spec.width, spec.height
    d.cam_position[:] = [float(x) for x in spec.cam_position]
    d.cam_direction[:] = [float(x) for x in spec.cam_direction]
    d.cam_up[:] = [float(x) for x in spec.cam_up]
    d.fov_degrees = float(spec.fov)
    d.sensor_width_mm = float(spec.sensor_width_mm)
    d.max_depth = spec.max_depth
    d.spp = spec.spp
    d.num_primitives = n
    d.prim_kind = _iptr(kind)
    d.prim_vertices = _fptr(verts)
    d.prim_normals = _fptr(normals) if normals is not None else None
    d.prim_uvws = _fptr(uvws) if uvws is not None else None
    d.prim_material = _iptr(mat)
    d.num_materials = len(spec.materials)
    d.materials = mats
    d.num_textures = len(spec.textures)
    d.textures = texs
    d.num_lights = len(spec.lights)
    d.lights = lights
    d.environment_texture = tex_index[spec.environment] + 1 if spec.environment else 0
    d.light_cluster = {"uniform": 0, "power": 1}[spec.light_cluster]
    d.filter = film_filter_struct(spec.film_filter)
    return FlatScene(d, kind, verts, mat, normals, uvws, mats, lights, texs, tex_arrays, names, mat_index)
