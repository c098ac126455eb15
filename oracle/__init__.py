"""The oracle: test infrastructure only.

* ``oracle/port/cadise_port.cpp`` - CPU restatement of the reference's path
  tracer (camera, BVH, primitives, BSDFs, lights, NEE+MIS estimator, film),
  pinned bit-for-bit against the reference itself through the golden vectors
  in ``tests/golden/``.
* ``oracle/ref_harness.cpp`` + ``oracle/Makefile`` - the reference's own
  objects with a seeded RNG, built only where the reference checkout exists,
  used to make those golden vectors.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker or the timed CPU
baseline; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
PORT_SO = os.path.join(BUILD, "libcadise_port.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")


def reference_dir() -> Optional[str]:
    """Where the reference checkout is: $CADISE_REFERENCE_DIR, else a checkout
    named ``reference`` next to this repository.  None when neither holds the
    reference's ``source/`` tree (the oracle's pinned restatement and the
    golden vectors need no checkout; only the harness build does)."""
    cand = os.environ.get("CADISE_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                   "reference")
    return cand if os.path.isdir(os.path.join(cand, "source")) else None


def build_port(force: bool = False) -> str:
    src = os.path.join(HERE, "port", "cadise_port.cpp")
    deps = [src, os.path.join(HERE, "oracle_rng.h"),
            os.path.join(HERE, "..", "include", "cadise_gpu.h")]
    if not force and os.path.exists(PORT_SO) and all(
            os.path.getmtime(PORT_SO) >= os.path.getmtime(d) for d in deps):
        return PORT_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = PORT_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                           src, "-o", tmp])
    os.replace(tmp, PORT_SO)
    return PORT_SO


def build_reference_harness(ref_root: Optional[str] = None, jobs: int = 8) -> Optional[str]:
    """Compile the reference harness from the reference sources (only where
    they exist; returns None elsewhere)."""
    ref_root = ref_root or reference_dir()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "source")):
        return None
    subprocess.check_call(["make", "-s", "-C", HERE, "-j%d" % jobs, "REF=" + ref_root])
    return REF_HARNESS


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_port())
        L = _lib
        L.port_scene_create.restype = C.c_void_p
        L.port_scene_create.argtypes = [C.c_void_p]
        L.port_scene_destroy.argtypes = [C.c_void_p]
        L.port_num_bvh_nodes.argtypes = [C.c_void_p]
        L.port_camera_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        L.port_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.port_visit_ranks.argtypes = [C.c_void_p, C.c_void_p]
        L.port_paths.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.port_render.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                  C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
        L.port_adjoint_fp64.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                        C.c_int32, C.c_int32, C.c_void_p]
        L.port_filter_splat.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        L.port_sample_positions.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
    return _lib


def filter_splat(film_filter, width: int, height: int, xy: np.ndarray, rgb: np.ndarray) -> np.ndarray:
    """FilmTile::addSample restated: samples (N x 2 positions, N x 3 radiance,
    in this order) through `film_filter` (a cadise_gb300.abi.cgpu_film_filter)
    into an H x W x 7 FP64 film {sum w rgb, sum w rgb^2, sum w}."""
    xy = np.ascontiguousarray(xy, dtype=np.float32).reshape(-1, 2)
    rgb = np.ascontiguousarray(rgb, dtype=np.float32).reshape(-1, 3)
    film = np.zeros((height, width, 7), np.float64)
    lib().port_filter_splat(C.byref(film_filter), width, height, xy.shape[0], _p(xy), _p(rgb), _p(film))
    return film


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class PortScene:
    """The CPU restatement over one flattened scene (see cadise_gb300.abi)."""

    def __init__(self, flat):
        self.flat = flat  # keeps the arrays alive
        self.handle = lib().port_scene_create(C.addressof(flat.desc))
        self.width = flat.desc.width
        self.height = flat.desc.height

    def close(self):
        if self.handle:
            lib().port_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def camera_rays(self, film_xy: np.ndarray) -> np.ndarray:
        xy = np.ascontiguousarray(film_xy, dtype=np.float64)
        out = np.zeros((xy.shape[0], 6), dtype=np.float32)
        lib().port_camera_rays(self.handle, _p(xy), xy.shape[0], _p(out))
        return out

    def trace(self, rays: np.ndarray):
        r = np.ascontiguousarray(rays, dtype=np.float32)
        n = r.shape[0]
        prim = np.zeros(n, dtype=np.int32)
        t = np.zeros(n, dtype=np.float32)
        occ = np.zeros(n, dtype=np.int32)
        lib().port_trace(self.handle, _p(r), n, _p(prim), _p(t), _p(occ))
        return prim, t, occ

    def visit_ranks(self) -> np.ndarray:
        """(num_primitives, 8) leaf-order position of every primitive per
        ray-direction octant in the reference tree's traversal."""
        n = int(self.flat.desc.num_primitives)
        out = np.zeros((n, 8), dtype=np.uint32)
        lib().port_visit_ranks(self.handle, _p(out))
        return out

    def paths(self, film_xy: np.ndarray, keys: np.ndarray):
        xy = np.ascontiguousarray(film_xy, dtype=np.float64)
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        n = xy.shape[0]
        rgb = np.zeros((n, 3), dtype=np.float32)
        draws = np.zeros(n, dtype=np.uint32)
        lib().port_paths(self.handle, _p(xy), _p(k), n, _p(rgb), _p(draws))
        return rgb, draws

    def render(self, seed: int, first: int, count: int, rows=None, threads: int = 1,
               want_paths: bool = False, scene_index: int = 0):
        r0, r1 = rows if rows is not None else (0, self.height)
        film = np.zeros((self.height, self.width, 7), dtype=np.float64)
        paths = np.zeros((count, self.height, self.width, 3), dtype=np.float32) if want_paths else None
        lib().port_render(self.handle, seed, scene_index, first, count, r0, r1, threads, _p(film), _p(paths))
        return film, paths


    def sample_positions(self, seed: int, first: int, count: int, scene_index: int = 0) -> np.ndarray:
        """Film positions (count x H x W x 2, float32) of samples [first, first + count)."""
        xy = np.zeros((count, self.height, self.width, 2), np.float32)
        lib().port_sample_positions(self.handle, seed, scene_index, first, count, _p(xy))
        return xy

    def adjoint_fp64(self, seed: int, spp: int, d_loss_d_image: np.ndarray, params, threads: int = 8,
                     scene_index: int = 0) -> np.ndarray:
        """FP64 forward-mode reference gradient for up to 16 parameters
        [(kind, index, channel)], kind 0 texel float, 1 roughness, 2 radiance."""
        dl = np.ascontiguousarray(d_loss_d_image, dtype=np.float32)
        pr = np.ascontiguousarray(np.asarray(params, dtype=np.int32).reshape(-1, 3))
        if pr.shape[0] > 16:
            raise ValueError("at most 16 parameters per call")
        g = np.zeros(pr.shape[0], np.float64)
        lib().port_adjoint_fp64(self.handle, seed, scene_index, spp, _p(dl), _p(pr), pr.shape[0], threads, _p(g))
        return g


# ---------------------------------------------------------------------------
# the per-path stream of oracle_rng.h, in numpy (for building path keys)
# ---------------------------------------------------------------------------
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def path_key(seed, scene, pixel, sample):
    with np.errstate(over="ignore"):
        s = mix64(np.uint64(seed) ^ (np.uint64(0xD1B54A32D192ED03) * (np.uint64(scene) + np.uint64(1))))
        pk = (np.asarray(sample, dtype=np.uint64) << np.uint64(32)) | np.asarray(pixel, dtype=np.uint64)
        return mix64(s ^ pk)
