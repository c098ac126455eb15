"""Generate the golden vectors from the reference renderer itself.

Run where the reference checkout exists (it is not needed anywhere else):

    python tests/golden/make_golden.py [--ref <reference checkout>]

(default: $CADISE_REFERENCE_DIR, else a checkout named ``reference`` next to
this repository)

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
* ``coplanar`` - quad lights in the ceiling's plane overlapping one another
  and tiles overlapping on the floor's plane: its closest hits are decided by
  the order in which the reference's BVH traversal meets the tied primitives.
* ``texel_vectors.npz`` - RgbImageTexture::evaluate (nearest, repeat) of the
  textured scene's texture at uvws on texel borders, below 0, above 1 and
  far outside.

The BASELINE-size scenes:

* ``cornell256`` - the Cornell box of the first configuration itself
  (256 x 256, 16 spp, depth 6), converged image at 16,384 spp.
* ``field1m`` - the full 1,024,000-triangle icosphere field of the second
  configuration (200 icospheres at subdivision 4 + ground + 8 quad lights,
  1920 x 1080, depth 12) with the GGX dielectric replaced by the reference's
  smooth ``glass`` (the reference has no rough dielectric): 100,000 seeded
  rays through the reference BVH (closest hit and occlusion; no brute-force
  pass at this size), 10,000 path radiances at full-resolution film
  positions, and a converged render of the same geometry and camera at
  96 x 54 (262,144 spp).  Its CRSD (100 MB of text) is not committed: the tests rebuild
  the scene with cadise_gb300.scenes and check it against the SHA-1 of its
  flattened arrays stored here; the rays are regenerated from their seed with
  exactly rounded operations only and checked against a stored SHA-1 too.

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
from golden_scenes import FILTER_CASES, exact_rays, field1m_spec, filtered_scene, scene_digest  # noqa: E402

TRACE_SEED = 1234
PATH_SEED = 77


def big_scenes():
    """name -> (vector SceneSpec, image SceneSpec, image spp, trace rays,
    paths, brute force): the BASELINE-size goldens."""
    return {
        "cornell256": (scenes.cornell_box(), None, 16384, 3000, 4000, True),
        # the image: the frame's camera and geometry at 96 x 54 (same aspect); its glass caustics and
        # small bright lights need 262,144 spp for the reference's own noise to fall to relMSE ~1.5e-4
        "field1m": (field1m_spec(), field1m_spec(96, 54), 262144, 100000, 10000, False),
    }


def golden_scenes():
    """name -> (SceneSpec, image spp or 0)."""
    return {
        "textured": (scenes.texture_scene(), 32768),
        "cornell": (scenes.cornell_box(64, 64, 16, 6), 4096),
        "field": (scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48,
                                         height=36, spp=16, max_depth=8, dielectric=scenes.GLASS,
                                         box=30.0, radius_range=(2.0, 6.0)), 2048),
        "features": (scenes.feature_scene(), 32768),
        "power": (scenes.power_field(), 131072),
        "spheres": (scenes.sphere_box(), 16384),
        "filtered": (filtered_scene(), 32768),
        "coplanar": (scenes.coplanar_scene(), 16384),
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


def make_texel_vectors(spec, harness, work):
    """RgbImageTexture::evaluate of the textured scene's texture at uvws on
    texel borders (k / width, k / height exactly), just inside them, below
    0, at 1 and beyond, and far outside."""
    crsd = os.path.join(HERE, "textured.crsd")
    t = spec.textures[0]
    h, w, _ = t.texels.shape
    rng = np.random.default_rng(5)
    us = [k / w for k in range(-2 * w, 3 * w + 1)] + [np.nextafter(np.float32(k / w), np.float32(-9)) for k in range(w + 1)]
    vs = [k / h for k in range(-2 * h, 3 * h + 1)] + [np.nextafter(np.float32(k / h), np.float32(-9)) for k in range(h + 1)]
    uv = [(u, v) for u in us[::3] for v in vs[::2]]
    uv += [(-0.0, 0.0), (1.0, 1.0), (0.999999, 0.999999), (-1e-7, -1e-7), (1e6 + 0.25, -1e6 - 0.75),
           (-3.5, 7.25), (123.456, -98.765)]
    uv += list(map(tuple, rng.uniform(-5.0, 5.0, (400, 2))))
    uvw = np.zeros((len(uv), 3), np.float32)
    uvw[:, :2] = np.asarray(uv, np.float64)
    uvw.tofile(os.path.join(work, "uvw.bin"))
    run(harness, ["texel", crsd, t.name, os.path.join(work, "uvw.bin"), os.path.join(work, "texel.bin")])
    rgb = np.fromfile(os.path.join(work, "texel.bin"), dtype=np.float32).reshape(-1, 3)
    np.savez_compressed(os.path.join(HERE, "texel_vectors.npz"), uvw=uvw, rgb=rgb)


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


def make_vectors(name, spec, harness, work, n_camera=512, n_trace=3000, n_paths=2000, crsd_dir=HERE,
                 brute_force=True, rays=None, extra=None):
    crsd = os.path.join(crsd_dir, name + ".crsd")
    spec.write_crsd(crsd, sidecar_min_triangles=1 << 62,
                    header="# golden scene %s - generated by tests/golden/make_golden.py\n" % name)
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
    if rays is None:
        rays = trace_rays(lo, hi, n_trace, rng)
        out["trace_rays"] = rays
    rays.tofile(os.path.join(work, "rays.bin"))
    run(harness, ["trace" if brute_force else "trace-bvh", crsd, os.path.join(work, "rays.bin"),
                  os.path.join(work, "trace.bin")])
    t = np.fromfile(os.path.join(work, "trace.bin"),
                    dtype=[("bp", "<i4"), ("bt", "<f4"), ("fp", "<i4"), ("ft", "<f4"), ("oc", "<i4")])
    out["trace_bvh_prim"] = t["bp"]
    out["trace_bvh_t"] = t["bt"]
    if brute_force:
        out["trace_bf_prim"] = t["fp"]
        out["trace_bf_t"] = t["ft"]
    out["trace_occluded"] = t["oc"].astype(np.int8)
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
    out.update(extra or {})
    np.savez_compressed(os.path.join(HERE, name + "_vectors.npz"), **out)
    return crsd


def make_image(name, spec, harness, work, spp, seed=2024, threads=8, crsd=None, compact=False):
    """compact: per pixel the FP32 mean and the FP32 variance of one sample
    (the tests form the standard error from them and the sample count)
    instead of FP64 sums, for the large films."""
    crsd = crsd or os.path.join(HERE, name + ".crsd")
    path = os.path.join(work, "film.bin")
    # a filtered film goes through the reference's FilmTile (no sums of squares)
    cmd = "render" if spec.film_filter is None else "render-tiles"
    run(harness, [cmd, crsd, path, spp, seed, threads])
    film = np.fromfile(path, dtype=np.float64).reshape(spec.height, spec.width, 7)
    if compact:
        n = film[..., 6:7]
        mean = film[..., :3] / n
        var = np.maximum(film[..., 3:6] / n - mean * mean, 0.0) * n / np.maximum(n - 1, 1)
        np.savez_compressed(os.path.join(HERE, name + "_image.npz"), mean=mean.astype(np.float32),
                            var=var.astype(np.float32), count=film[..., 6].astype(np.float32), spp=spp, seed=seed)
        return
    np.savez_compressed(os.path.join(HERE, name + "_image.npz"), sum=film[..., :3], sum_sq=film[..., 3:6],
                        count=film[..., 6], spp=spp, seed=seed)


def make_big(name, harness, work, threads, image_only=False):
    """The BASELINE-size goldens (see the module docstring)."""
    from cadise_gb300 import abi
    spec, image_spec, spp, n_trace, n_paths, bf = big_scenes()[name]
    if image_only and image_spec is not None:
        crsd = os.path.join(work, name + "_image.crsd")
        image_spec.write_crsd(crsd, sidecar_min_triangles=1 << 62)
        make_image(name, image_spec, harness, work, spp, threads=threads, crsd=crsd, compact=True)
        return
    extra = {"scene_sha1": scene_digest(abi.flatten(spec))}
    rays = None
    crsd_dir = HERE
    if not bf:
        rays = exact_rays(spec, n_trace, TRACE_SEED)
        import hashlib
        extra["rays_seed"] = TRACE_SEED
        extra["rays_n"] = n_trace
        extra["rays_sha1"] = hashlib.sha1(rays.tobytes()).hexdigest()
        crsd_dir = work
    make_vectors(name, spec, harness, work, n_trace=n_trace, n_paths=n_paths, crsd_dir=crsd_dir, brute_force=bf,
                 rays=rays, extra=extra)
    img = image_spec or spec
    crsd = os.path.join(crsd_dir, name + ".crsd")
    if image_spec is not None:
        crsd = os.path.join(work, name + "_image.crsd")
        image_spec.write_crsd(crsd, sidecar_min_triangles=1 << 62)
    make_image(name, img, harness, work, spp, threads=threads, crsd=crsd, compact=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--only", default=None)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 8)
    ap.add_argument("--image-only", action="store_true", help="a large scene's converged image alone")
    args = ap.parse_args()
    harness = oracle.build_reference_harness(args.ref)
    if harness is None:
        sys.exit("reference sources not found (--ref, $CADISE_REFERENCE_DIR or ../reference)")
    with tempfile.TemporaryDirectory() as work:
        if args.only in (None, "filters"):
            make_filter_vectors(harness, work)
            print("golden filters done")
        for name, (spec, spp) in golden_scenes().items():
            if args.only and name != args.only:
                continue
            make_vectors(name, spec, harness, work)
            if name == "textured":
                make_texel_vectors(spec, harness, work)
            if spp:
                make_image(name, spec, harness, work, spp, threads=args.threads)
            print("golden", name, "done")
        for name in big_scenes():
            if args.only and name != args.only:
                continue
            make_big(name, harness, work, args.threads, image_only=args.image_only)
            print("golden", name, "done")


if __name__ == "__main__":
    main()
