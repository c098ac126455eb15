"""Generate the golden vectors from the reference renderer itself.

Run where the reference checkout exists (it is not needed anywhere else):

    python tests/golden/make_golden.py [--ref /root/reference]

It builds ``oracle/_ref/ref_harness`` (the reference's own objects plus a
seeded RNG, see oracle/ref_harness.cpp), writes each test scene as CRSD text
next to this script, and records what the reference computes for it:

* ``<scene>_vectors.npz``
    - camera:  film positions -> primary ray (Camera::spawnPrimaryRay)
    - trace:   seeded rays -> BVH closest hit (primitive, t), brute-force
               closest hit, BVH occlusion
    - paths:   (film position, path key) -> PtEstimator radiance and the
               number of random draws the path consumed
* ``<scene>_image.npz`` - an FP64 box-filtered film rendered with the
  reference tile loop (reference StratifiedSampler + PtEstimator): per-pixel
  sum, sum of squares and sample count, for statistical image parity (for a
  scene with another film filter: sums of w L and of w through the
  reference's FilmTile, sum_sq zero).
* ``filter_vectors.npz`` - the reference's FilmTile::addSample with each
  filter of FILTER_CASES on one set of samples: per-pixel sensor sums.

Primitive indices are the reference's intersector creation order.  Path keys
follow oracle/oracle_rng.h.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from cadise_gb300 import scenes  # noqa: E402
import oracle  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests"))
from golden_scenes import FILTER_CASES, filtered_scene  # noqa: E402

TRACE_SEED = 1234
PATH_SEED = 77


def golden_scenes():
    """name -> (SceneSpec, image spp or 0)."""
    return {
        "cornell": (scenes.cornell_box(64, 64, 16, 6), 4096),
        "field": (scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48,
                                         height=36, spp=16, max_depth=8, dielectric=scenes.GLASS,
                                         box=30.0, radius_range=(2.0, 6.0)), 2048),
        "features": (scenes.feature_scene(), 32768),
        "power": (scenes.power_field(), 131072),
        "spheres": (scenes.sphere_box(), 16384),
        "filtered": (filtered_scene(), 32768),
    }


def make_filter_vectors(harness, work, n=4000):
    """FilmTile::addSample of the reference with each filter on the same
    samples (uniform positions over a 40 x 30 film, some on exact pixel
    edges, a few NaN / Inf radiances)."""
    rng = np.random.default_rng(99)
    W, H = 40, 30
    xy = rng.uniform(0, 1, (n, 2)) * [W, H]
    xy[:100] = np.floor(xy[:100])          # exactly on a pixel corner
    xy = np.minimum(xy, [W - 1e-3, H - 1e-3]).astype(np.float32)
    rgb = rng.uniform(0, 2, (n, 3)).astype(np.float32)
    rgb[200, 0] = np.nan
    rgb[201, 2] = np.inf
    samples = np.concatenate([xy, rgb], 1).astype(np.float32)
    samples.tofile(os.path.join(work, "samples.bin"))
    out = {"xy": xy, "rgb": rgb, "width": W, "height": H}
    for name, f in FILTER_CASES:
        spec = scenes.cornell_box(W, H, 1, 2)
        spec.film_filter = f
        crsd = os.path.join(work, "filter.crsd")
        with open(crsd, "w") as fh:
            fh.write(spec.to_crsd())
        run(harness, ["filmtile", crsd, os.path.join(work, "samples.bin"), os.path.join(work, "ft.bin")])
        out["sensor_" + name] = np.fromfile(os.path.join(work, "ft.bin"), dtype=np.float64).reshape(H, W, 4)
    np.savez_compressed(os.path.join(HERE, "filter_vectors.npz"), **out)


def trace_rays(lo, hi, n, rng):
    """Half the rays start inside the scene bounds in uniform directions, half
    have a finite t_max (shadow-ray style)."""
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = o
    rays[:, 3] = 1e-3
    rays[:, 4:7] = d
    finite = rng.uniform(size=n) < 0.5
    rays[:, 7] = np.where(finite, rng.uniform(0.5, 1.0, n) * np.linalg.norm(hi - lo), 3.4028235e38)
    # renormalise in float32 exactly like the reference Ray constructor would
    return rays


def run(harness, args):
    subprocess.check_call([harness] + [str(a) for a in args])


def make_vectors(name, spec, harness, work, n_camera=512, n_trace=3000, n_paths=2000):
    crsd = os.path.join(HERE, name + ".crsd")
    with open(crsd, "w") as f:
        f.write("# golden scene %s - generated by tests/golden/make_golden.py\n" % name)
        f.write(spec.to_crsd())
    rng = np.random.default_rng(TRACE_SEED)
    out = {}
    # camera
    xy = np.stack([rng.uniform(0, spec.width, n_camera), rng.uniform(0, spec.height, n_camera)], 1)
    xy = xy.astype(np.float64)
    xy.tofile(os.path.join(work, "xy.bin"))
    run(harness, ["camera", crsd, os.path.join(work, "xy.bin"), os.path.join(work, "cam.bin")])
    out["camera_xy"] = xy
    out["camera_rays"] = np.fromfile(os.path.join(work, "cam.bin"), dtype=np.float32).reshape(-1, 6)
    # trace
    from cadise_gb300 import abi
    flat = abi.flatten(spec)
    v = flat.vertices.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    rays = trace_rays(lo, hi, n_trace, rng)
    rays.tofile(os.path.join(work, "rays.bin"))
    run(harness, ["trace", crsd, os.path.join(work, "rays.bin"), os.path.join(work, "trace.bin")])
    t = np.fromfile(os.path.join(work, "trace.bin"),
                    dtype=[("bp", "<i4"), ("bt", "<f4"), ("fp", "<i4"), ("ft", "<f4"), ("oc", "<i4")])
    out["trace_rays"] = rays
    out["trace_bvh_prim"] = t["bp"]
    out["trace_bvh_t"] = t["bt"]
    out["trace_bf_prim"] = t["fp"]
    out["trace_bf_t"] = t["ft"]
    out["trace_occluded"] = t["oc"]
    # paths
    pxy = np.stack([rng.uniform(0, spec.width, n_paths), rng.uniform(0, spec.height, n_paths)], 1)
    keys = oracle.path_key(PATH_SEED, 0, np.arange(n_paths), 5)
    q = np.zeros(n_paths, dtype=[("x", "<f8"), ("y", "<f8"), ("k", "<u8")])
    q["x"], q["y"], q["k"] = pxy[:, 0], pxy[:, 1], keys
    q.tofile(os.path.join(work, "paths.bin"))
    run(harness, ["paths", crsd, os.path.join(work, "paths.bin"), os.path.join(work, "pout.bin")])
    r = np.fromfile(os.path.join(work, "pout.bin"), dtype=[("rgb", "<f4", 3), ("d", "<u4")])
    out["paths_xy"] = pxy.astype(np.float64)
    out["paths_keys"] = keys
    out["paths_rgb"] = r["rgb"]
    out["paths_draws"] = r["d"]
    np.savez_compressed(os.path.join(HERE, name + "_vectors.npz"), **out)
    return crsd


def make_image(name, spec, harness, work, spp, seed=2024, threads=8):
    crsd = os.path.join(HERE, name + ".crsd")
    path = os.path.join(work, "film.bin")
    # a filtered film goes through the reference's FilmTile (no sums of squares)
    cmd = "render" if spec.film_filter is None else "render-tiles"
    run(harness, [cmd, crsd, path, spp, seed, threads])
    film = np.fromfile(path, dtype=np.float64).reshape(spec.height, spec.width, 7)
    np.savez_compressed(os.path.join(HERE, name + "_image.npz"), sum=film[..., :3], sum_sq=film[..., 3:6],
                        count=film[..., 6], spp=spp, seed=seed)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default=None)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 8)
    args = ap.parse_args()
    harness = oracle.build_reference_harness(args.ref)
    if harness is None:
        sys.exit("reference sources not found at %s" % args.ref)
    with tempfile.TemporaryDirectory() as work:
        if args.only in (None, "filters"):
            make_filter_vectors(harness, work)
            print("golden filters done")
        for name, (spec, spp) in golden_scenes().items():
            if args.only and name != args.only:
                continue
            make_vectors(name, spec, harness, work)
            if spp:
                make_image(name, spec, harness, work, spp, threads=args.threads)
            print("golden", name, "done")


if __name__ == "__main__":
    main()
