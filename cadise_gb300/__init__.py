"""cadise_gb300 - the reference renderer's unidirectional path tracer on GB300.

The product is the C-ABI shared library ``_build/libcadise_gpu.so`` (header
``include/cadise_gpu.h``): hand-written sm_103a kernels for BVH traversal,
the NEE + MIS path estimator (megakernel and wavefront), the FP64 film and
the adjoint.  This package is a thin ctypes view of that ABI for tests,
benchmarks and Python callers; it never computes radiance itself and raises
if the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import abi
from .abi import (CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT, FlatScene, cgpu_hit, cgpu_options,
                  cgpu_ray, cgpu_render_params, cgpu_render_stats, cgpu_scene_info, flatten)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcadise_gpu.so")

# Every symbol include/cadise_gpu.h declares.
EXPORTED = [
    "cgpu_create", "cgpu_destroy", "cgpu_last_error", "cgpu_status_string", "cgpu_abi_version",
    "cgpu_synchronize", "cgpu_set_visit_budget", "cgpu_set_tie_order", "cgpu_set_bvh_builder", "cgpu_scene_upload", "cgpu_scene_release", "cgpu_scene_info_get",
    "cgpu_trace_closest", "cgpu_trace_any", "cgpu_trace_closest_device", "cgpu_trace_any_device",
    "cgpu_camera_rays", "cgpu_render", "cgpu_render_noalloc", "cgpu_film_clear", "cgpu_film_read", "cgpu_path_radiance",
    "cgpu_render_paths", "cgpu_render_stats_get", "cgpu_set_counting", "cgpu_set_profiling",
    "cgpu_kernel_times_get", "cgpu_param_counts_get", "cgpu_params_get", "cgpu_params_set",
    "cgpu_adjoint_forward", "cgpu_adjoint_backward", "cgpu_set_adjoint_mode", "cgpu_tuning_get", "cgpu_tuning_set", "cgpu_autotune",
    # include/cadise_crsd.h
    "cgpu_crsd_load_file", "cgpu_crsd_load_text", "cgpu_crsd_desc", "cgpu_crsd_settings_get",
    "cgpu_crsd_primitive_index", "cgpu_crsd_free",
]

KERNEL_CLASSES = ["generate", "extend", "shadow", "shade", "splat", "megakernel", "reorder", "mis_occl", "ties"]

_lib = None


class CgpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, str(status)), message))
        self.status = status


def build(verbose: bool = False) -> str:
    from .native_build import build as _build
    return _build(verbose=verbose)


def load(path: Optional[str] = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("cadise_gb300: CUDA library %s is not built; run cadise_gb300.build() "
                           "(there is no CPU fallback)" % p)
    L = C.CDLL(p)
    vp = C.c_void_p
    L.cgpu_create.argtypes = [C.POINTER(vp), C.POINTER(cgpu_options)]
    L.cgpu_destroy.argtypes = [vp]
    L.cgpu_destroy.restype = None
    L.cgpu_last_error.argtypes = [vp]
    L.cgpu_last_error.restype = C.c_char_p
    L.cgpu_status_string.argtypes = [C.c_int]
    L.cgpu_status_string.restype = C.c_char_p
    L.cgpu_abi_version.restype = C.c_int32
    L.cgpu_synchronize.argtypes = [vp]
    L.cgpu_set_visit_budget.argtypes = [vp, C.c_uint32]
    L.cgpu_set_tie_order.argtypes = [vp, C.c_int32]
    L.cgpu_scene_upload.argtypes = [vp, vp, C.POINTER(C.c_int32)]
    L.cgpu_scene_release.argtypes = [vp, C.c_int32]
    L.cgpu_scene_info_get.argtypes = [vp, C.c_int32, C.POINTER(cgpu_scene_info)]
    L.cgpu_trace_closest.argtypes = [vp, C.c_int32, vp, C.c_uint32, vp]
    L.cgpu_trace_any.argtypes = [vp, C.c_int32, vp, C.c_uint32, vp]
    L.cgpu_trace_closest_device.argtypes = [vp, C.c_int32, vp, C.c_uint32, vp]
    L.cgpu_trace_any_device.argtypes = [vp, C.c_int32, vp, C.c_uint32, vp]
    L.cgpu_camera_rays.argtypes = [vp, C.c_int32, vp, C.c_uint32, vp]
    L.cgpu_render.argtypes = [vp, C.POINTER(cgpu_render_params)]
    L.cgpu_render_noalloc.argtypes = [vp, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint64]
    L.cgpu_film_clear.argtypes = [vp, C.c_int32]
    L.cgpu_film_read.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.cgpu_path_radiance.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, C.c_uint32, vp]
    L.cgpu_render_paths.argtypes = [vp, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint64, vp]
    L.cgpu_render_stats_get.argtypes = [vp, C.POINTER(cgpu_render_stats)]
    L.cgpu_set_counting.argtypes = [vp, C.c_int32]
    L.cgpu_set_profiling.argtypes = [vp, C.c_int32]
    L.cgpu_kernel_times_get.argtypes = [vp, C.POINTER(abi.cgpu_kernel_times)]
    L.cgpu_param_counts_get.argtypes = [vp, C.c_int32, C.POINTER(abi.cgpu_param_counts)]
    L.cgpu_params_get.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.cgpu_params_set.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.cgpu_adjoint_forward.argtypes = [vp, C.c_int32, C.c_uint32, C.c_uint64, vp]
    L.cgpu_adjoint_backward.argtypes = [vp, C.c_int32, C.c_uint32, C.c_uint64, vp, vp, vp, vp]
    L.cgpu_set_adjoint_mode.argtypes = [vp, C.c_int32]
    L.cgpu_set_bvh_builder.argtypes = [vp, C.c_int32]
    L.cgpu_tuning_get.argtypes = [vp, C.POINTER(abi.cgpu_tuning)]
    L.cgpu_tuning_set.argtypes = [vp, C.POINTER(abi.cgpu_tuning)]
    L.cgpu_autotune.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_char_p, C.POINTER(abi.cgpu_tuning)]
    L.cgpu_crsd_load_file.argtypes = [C.c_char_p, C.POINTER(vp), C.c_char_p, C.c_size_t]
    L.cgpu_crsd_load_text.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(vp), C.c_char_p, C.c_size_t]
    L.cgpu_crsd_desc.argtypes = [vp]
    L.cgpu_crsd_desc.restype = C.POINTER(abi.cgpu_scene_desc)
    L.cgpu_crsd_settings_get.argtypes = [vp, C.POINTER(abi.cgpu_crsd_settings)]
    L.cgpu_crsd_primitive_index.argtypes = [vp, C.c_char_p]
    L.cgpu_crsd_primitive_index.restype = C.c_int32
    L.cgpu_crsd_free.argtypes = [vp]
    L.cgpu_crsd_free.restype = None
    _lib = L
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _tuning_dict(t) -> dict:
    return {"block_trace": t.block_trace, "block_shade": t.block_shade, "max_paths": t.max_paths,
            "traversal": t.traversal, "reorder": t.reorder, "refill_closest": t.refill_closest,
            "refill_any": t.refill_any}


class Context:
    """One library context: one CUDA stream, any number of scenes."""

    def __init__(self, device: int = 0, stream: Optional[int] = None, max_paths: int = 0):
        self.L = load()
        opt = cgpu_options(device=device, stream=stream or None, max_paths=max_paths, flags=0)
        h = C.c_void_p()
        st = self.L.cgpu_create(C.byref(h), C.byref(opt))
        if st != 0:
            raise CgpuError(st, "cgpu_create failed")
        self.h = h
        self._scenes = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.cgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise CgpuError(st, self.L.cgpu_last_error(self.h).decode())

    # ---------------------------------------------------------------- scenes
    def upload(self, scene) -> int:
        """Upload a SceneSpec, a FlatScene or a CrsdScene."""
        if isinstance(scene, CrsdScene):
            flat = scene
        else:
            flat = scene if isinstance(scene, FlatScene) else flatten(scene)
        sid = C.c_int32(-1)
        self._check(self.L.cgpu_scene_upload(self.h, C.addressof(flat.desc), C.byref(sid)))
        self._scenes[sid.value] = flat
        return sid.value

    def release(self, sid: int):
        self._check(self.L.cgpu_scene_release(self.h, sid))
        self._scenes.pop(sid, None)

    def info(self, sid: int) -> cgpu_scene_info:
        out = cgpu_scene_info()
        self._check(self.L.cgpu_scene_info_get(self.h, sid, C.byref(out)))
        return out

    # ----------------------------------------------------------- ray queries
    def trace_closest(self, sid: int, rays: np.ndarray):
        """rays: (n, 8) float32 (org, t_min, dir, t_max) -> (prim, t, u, v)."""
        r = np.ascontiguousarray(rays, dtype=np.float32)
        n = r.shape[0]
        out = np.zeros(n, dtype=[("t", "<f4"), ("prim", "<i4"), ("u", "<f4"), ("v", "<f4")])
        self._check(self.L.cgpu_trace_closest(self.h, sid, _p(r), n, _p(out)))
        return out["prim"].copy(), out["t"].copy(), out["u"].copy(), out["v"].copy()

    def trace_any(self, sid: int, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, dtype=np.float32)
        occ = np.zeros(r.shape[0], dtype=np.uint8)
        self._check(self.L.cgpu_trace_any(self.h, sid, _p(r), r.shape[0], _p(occ)))
        return occ

    def camera_rays(self, sid: int, film_xy: np.ndarray) -> np.ndarray:
        xy = np.ascontiguousarray(film_xy, dtype=np.float64)
        out = np.zeros((xy.shape[0], 6), dtype=np.float32)
        self._check(self.L.cgpu_camera_rays(self.h, sid, _p(xy), xy.shape[0], _p(out)))
        return out

    # ---------------------------------------------------------------- render
    def path_radiance(self, sid: int, film_xy: np.ndarray, keys: np.ndarray, mode: int = CGPU_MODE_MEGAKERNEL):
        xy = np.ascontiguousarray(film_xy, dtype=np.float64)
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros((xy.shape[0], 3), dtype=np.float32)
        self._check(self.L.cgpu_path_radiance(self.h, sid, mode, _p(xy), _p(k), xy.shape[0], _p(out)))
        return out

    def render_paths(self, sid: int, first: int, count: int, seed: int, mode: int = CGPU_MODE_WAVEFRONT):
        flat = self._scenes[sid]
        w, h = flat.desc.width, flat.desc.height
        out = np.zeros((count, h, w, 3), dtype=np.float32)
        self._check(self.L.cgpu_render_paths(self.h, sid, mode, first, count, seed, _p(out)))
        return out

    def render(self, sids: Sequence[int], first: int, count, seed: int,
               mode: int = CGPU_MODE_WAVEFRONT, graph: bool = True, sync: bool = True):
        """Samples [first, first + count) of every scene; `count` may be a
        sequence with one sample count per scene."""
        arr = (C.c_int32 * len(sids))(*sids)
        per = None
        if not isinstance(count, int):
            per = (C.c_uint32 * len(sids))(*[int(c) for c in count])
            count = 0
        p = cgpu_render_params(scenes=arr, num_scenes=len(sids), first_sample=first, num_samples=count,
                               seed=seed, mode=mode, use_graph=1 if graph else 0, scene_samples=per)
        self._check(self.L.cgpu_render(self.h, C.byref(p)))
        if sync:
            self.synchronize()

    def render_noalloc(self, sid: int, first: int, count: int, seed: int, sync: bool = True):
        """cgpu_render_noalloc: the wavefront render with every device buffer
        of the call in the library's static scratch (frames up to 262144
        pixels, max depth 62, scene ids below 64)."""
        self._check(self.L.cgpu_render_noalloc(self.h, sid, first, count, seed))
        if sync:
            self.synchronize()

    def film_clear(self, sid: int):
        self._check(self.L.cgpu_film_clear(self.h, sid))

    def film_read(self, sid: int):
        flat = self._scenes[sid]
        w, h = flat.desc.width, flat.desc.height
        s = np.zeros((h, w, 3))
        q = np.zeros((h, w, 3))
        n = np.zeros((h, w))
        self._check(self.L.cgpu_film_read(self.h, sid, _p(s), _p(q), _p(n)))
        return s, q, n

    def film_read_into(self, sid: int, sum_rgb: np.ndarray, sum_sq_rgb: np.ndarray, count: np.ndarray):
        """Film read-back into caller buffers (e.g. pinned host memory)."""
        flat = self._scenes[sid]
        n = flat.desc.width * flat.desc.height
        for a, k in ((sum_rgb, 3), (sum_sq_rgb, 3), (count, 1)):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != n * k:
                raise ValueError("film_read_into: need contiguous float64 buffers of the film size")
        self._check(self.L.cgpu_film_read(self.h, sid, _p(sum_rgb), _p(sum_sq_rgb), _p(count)))

    def stats(self) -> cgpu_render_stats:
        out = cgpu_render_stats()
        self._check(self.L.cgpu_render_stats_get(self.h, C.byref(out)))
        return out

    def synchronize(self):
        """Wait for the context stream; raises CgpuError (CGPU_ERR_TIMEOUT) if a
        traversal ran out of its device-side visit budget since the last check."""
        self._check(self.L.cgpu_synchronize(self.h))

    def set_visit_budget(self, visits: int):
        """Node and leaf visits per ray before a traversal stops (0: automatic)."""
        self._check(self.L.cgpu_set_visit_budget(self.h, visits))

    def set_tie_order(self, order: int):
        """Exact-tie rule of closest hits for scenes uploaded afterwards:
        CGPU_TIE_ORDER_REFERENCE (default; the reference BVH's visiting
        order, built at upload) or CGPU_TIE_ORDER_INDEX (lower primitive)."""
        self._check(self.L.cgpu_set_tie_order(self.h, order))

    def set_counting(self, on: bool):
        self._check(self.L.cgpu_set_counting(self.h, 1 if on else 0))

    # --------------------------------------------------------------- adjoint
    def param_counts(self, sid: int):
        out = abi.cgpu_param_counts()
        self._check(self.L.cgpu_param_counts_get(self.h, sid, C.byref(out)))
        return int(out.texel_floats), int(out.materials), int(out.lights)

    def get_params(self, sid: int):
        nt, nm, nl = self.param_counts(sid)
        tex = np.zeros(nt, np.float32)
        rough = np.zeros(nm, np.float32)
        rad = np.zeros((nl, 3), np.float32)
        self._check(self.L.cgpu_params_get(self.h, sid, _p(tex) if nt else None, _p(rough), _p(rad)))
        return tex, rough, rad

    def set_params(self, sid: int, texels=None, roughness=None, radiance=None):
        args = []
        keep = []
        for a in (texels, roughness, radiance):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=np.float32)
                keep.append(a)
                args.append(_p(a))
        self._check(self.L.cgpu_params_set(self.h, sid, *args))

    def adjoint_forward(self, sid: int, spp: int, seed: int) -> np.ndarray:
        flat = self._scenes[sid]
        img = np.zeros((flat.desc.height, flat.desc.width, 3), np.float32)
        self._check(self.L.cgpu_adjoint_forward(self.h, sid, spp, seed, _p(img)))
        return img

    def set_bvh_builder(self, builder: int) -> None:
        """abi.CGPU_BVH_BUILDER_AUTO (default), _HOST_SAH or _GPU_PLOC for the following uploads."""
        self._check(self.L.cgpu_set_bvh_builder(self.h, builder))

    def set_adjoint_mode(self, mode: int) -> None:
        """CGPU_MODE_WAVEFRONT (default) or CGPU_MODE_MEGAKERNEL schedule of adjoint_backward."""
        self._check(self.L.cgpu_set_adjoint_mode(self.h, mode))

    def adjoint_backward(self, sid: int, spp: int, seed: int, d_loss_d_image: np.ndarray):
        nt, nm, nl = self.param_counts(sid)
        dl = np.ascontiguousarray(d_loss_d_image, dtype=np.float32)
        gt = np.zeros(max(nt, 1), np.float64)
        gr = np.zeros(max(nm, 1), np.float64)
        gl = np.zeros((max(nl, 1), 3), np.float64)
        self._check(self.L.cgpu_adjoint_backward(self.h, sid, spp, seed, _p(dl), _p(gt), _p(gr), _p(gl)))
        return gt[:nt], gr[:nm], gl[:nl]

    # -------------------------------------------------------------- autotune
    def tuning(self) -> dict:
        t = abi.cgpu_tuning()
        self._check(self.L.cgpu_tuning_get(self.h, C.byref(t)))
        return _tuning_dict(t)

    def set_tuning(self, block_trace: int, block_shade: int, max_paths: int = 0, traversal: int = 0,
                   reorder: int = 0, refill_closest: int = 0, refill_any: int = 0):
        t = abi.cgpu_tuning(block_trace=block_trace, block_shade=block_shade, max_paths=max_paths,
                            traversal=traversal, reorder=reorder, refill_closest=refill_closest,
                            refill_any=refill_any)
        self._check(self.L.cgpu_tuning_set(self.h, C.byref(t)))

    def set_tuning_dict(self, t: dict):
        """set_tuning from a dict as tuning() / autotune() return it."""
        self.set_tuning(t["block_trace"], t["block_shade"], t.get("max_paths", 0), t.get("traversal", 0),
                        t.get("reorder", 0), t.get("refill_closest", 0), t.get("refill_any", 0))

    def autotune(self, sids, samples: int = 1, cache_path: Optional[str] = None) -> dict:
        arr = (C.c_int32 * len(sids))(*sids)
        t = abi.cgpu_tuning()
        self._check(self.L.cgpu_autotune(self.h, arr, len(sids), samples,
                                         cache_path.encode() if cache_path else None, C.byref(t)))
        return _tuning_dict(t)

    def set_profiling(self, on: bool):
        self._check(self.L.cgpu_set_profiling(self.h, 1 if on else 0))

    def kernel_times(self):
        """{class: (total ms, launches)} of the last render with profiling on."""
        out = abi.cgpu_kernel_times()
        self._check(self.L.cgpu_kernel_times_get(self.h, C.byref(out)))
        return {name: (out.ms[i], out.launches[i]) for i, name in enumerate(KERNEL_CLASSES)}


class CrsdScene:
    """A CRSD scene parsed by the library's C++ loader (include/cadise_crsd.h).

    ``desc`` points into memory owned by the loader; it can be handed to
    :meth:`Context.upload` directly."""

    def __init__(self, path: Optional[str] = None, text: Optional[str] = None):
        self.L = load()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        if path is not None:
            st = self.L.cgpu_crsd_load_file(path.encode(), C.byref(h), err, 512)
        else:
            b = text.encode()
            st = self.L.cgpu_crsd_load_text(b, len(b), C.byref(h), err, 512)
        if st != 0:
            raise CgpuError(st, err.value.decode())
        self.h = h
        self.desc = self.L.cgpu_crsd_desc(h).contents

    def settings(self) -> "abi.cgpu_crsd_settings":
        out = abi.cgpu_crsd_settings()
        st = self.L.cgpu_crsd_settings_get(self.h, C.byref(out))
        if st != 0:
            raise CgpuError(st, "settings")
        return out

    def primitive_index(self, name: str) -> int:
        return self.L.cgpu_crsd_primitive_index(self.h, name.encode())

    def arrays(self):
        """numpy views of the flat primitive arrays (kind, vertices, material)."""
        d = self.desc
        n = d.num_primitives
        kind = np.ctypeslib.as_array(d.prim_kind, shape=(n,)).copy()
        verts = np.ctypeslib.as_array(d.prim_vertices, shape=(n, 9)).copy()
        mat = np.ctypeslib.as_array(d.prim_material, shape=(n,)).copy()
        return kind, verts, mat

    def close(self):
        if getattr(self, "h", None):
            self.L.cgpu_crsd_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
