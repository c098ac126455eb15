"""The GPU BVH builds (PLOC clustering, bvh_gpu.cu; the host's binned SAH on
the GPU, bvh_sah_gpu.cu) against the host binned-SAH build.  Closest hits keep, on an exact tie of
distance, the lower primitive index, so every query and every render must
come out bit for bit the same whichever builder made the tree; a tree that
lost, duplicated or mis-bounded a triangle would change hits."""
import numpy as np
import pytest

from cadise_gb300 import CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT, CgpuError, abi, scenes
from golden_scenes import specs, vectors

pytestmark = pytest.mark.gpu

HOST, GPU, GPU_SAH = abi.CGPU_BVH_BUILDER_HOST_SAH, abi.CGPU_BVH_BUILDER_GPU_PLOC, abi.CGPU_BVH_BUILDER_GPU_SAH


def upload_with(ctx, flat, builder):
    ctx.set_bvh_builder(builder)
    try:
        sid = ctx.upload(flat)
    finally:
        ctx.set_bvh_builder(abi.CGPU_BVH_BUILDER_AUTO)
    assert ctx.info(sid).bvh_builder == builder
    return sid


def coincident_scene(n=3000):
    """Many triangles with one centroid (equal Morton codes, equal merge costs)."""
    s = scenes.cornell_box(32, 32, 4, 4)
    rng = np.random.default_rng(1)
    base = np.array([[200.0, 100.0, 200.0], [350.0, 100.0, 250.0], [275.0, 260.0, 225.0]])
    tris = np.repeat(base[None], n, 0) + rng.normal(0, 1e-3, (n, 3, 3))
    tris -= tris.mean(1, keepdims=True) - base.mean(0)  # same centroid, slightly different shapes
    s.primitives.append(scenes.TriangleMesh(name="stack", material=s.materials[0].name,
                                            positions=tris.astype(np.float32)))
    return s


def small_scenes():
    out = dict(specs())
    out["coincident"] = coincident_scene()
    return out


@pytest.mark.parametrize("name", ["cornell", "field", "features", "power", "spheres", "coincident"])
def test_renders_identical_with_either_builder(gpu_ctx, name):
    spec = small_scenes()[name]
    flat = abi.flatten(spec)
    films = []
    for b in (HOST, GPU, GPU_SAH):
        sid = upload_with(gpu_ctx, flat, b)
        for mode in (CGPU_MODE_WAVEFRONT, CGPU_MODE_MEGAKERNEL):
            gpu_ctx.film_clear(sid)
            gpu_ctx.render([sid], 0, 8, seed=31, mode=mode)
            films.append(gpu_ctx.film_read(sid))
        gpu_ctx.release(sid)
    for f in films[1:]:
        for x, y in zip(films[0], f):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["cornell", "field", "features", "power", "spheres"])
def test_ray_queries_identical_with_either_builder(gpu_ctx, name):
    flat = abi.flatten(specs()[name])
    rays = vectors(name)["trace_rays"]
    out = []
    for b in (HOST, GPU, GPU_SAH):
        sid = upload_with(gpu_ctx, flat, b)
        out.append((gpu_ctx.trace_closest(sid, rays), gpu_ctx.trace_any(sid, rays)))
        gpu_ctx.release(sid)
    (h0, o0) = out[0]
    for h1, o1 in out[1:]:
        for x, y in zip(h0, h1):  # primitive, t, u, v
            assert np.array_equal(x, y)
        assert np.array_equal(o0, o1)


def test_tiny_scenes_build_on_the_gpu(gpu_ctx):
    """Two to five primitives: a root that is itself a leaf, and a root with
    fewer than four children."""
    for extra in range(0, 4):
        s = scenes.cornell_box(16, 16, 2, 3)
        s.primitives = s.primitives[:1 + extra] + [p for p in s.primitives if getattr(p, "name", "") == "light"]
        s.lights = s.lights[:1]
        flat = abi.flatten(s)
        films = []
        for b in (HOST, GPU, GPU_SAH):
            sid = upload_with(gpu_ctx, flat, b)
            gpu_ctx.film_clear(sid)
            gpu_ctx.render([sid], 0, 4, seed=2)
            films.append(gpu_ctx.film_read(sid))
            gpu_ctx.release(sid)
        for f in films[1:]:
            for x, y in zip(films[0], f):
                assert np.array_equal(x, y)


def test_million_triangle_field_identical_and_faster_to_build(gpu_ctx):
    """Films bit-identical with every tree; both GPU builds faster than the
    host's; the GPU SAH tree is the host's (same node count, the same node
    visits to 0.01 %: they differ only below median splits of coincident
    centroids, where the host's partition is not stable)."""
    spec = scenes.icosphere_field()
    flat = abi.flatten(spec)
    films, ms, nodes, visits = [], [], [], []
    for b in (HOST, GPU, GPU_SAH):
        sid = upload_with(gpu_ctx, flat, b)
        info = gpu_ctx.info(sid)
        ms.append(info.bvh_ms)
        nodes.append(info.num_bvh_nodes)
        gpu_ctx.set_counting(True)
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 0, 1, seed=3)
        visits.append(gpu_ctx.stats().node_visits)
        gpu_ctx.set_counting(False)
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 0, 1, seed=3)
        films.append(gpu_ctx.film_read(sid))
        gpu_ctx.release(sid)
    for f in films[1:]:
        for x, y in zip(films[0], f):
            assert np.array_equal(x, y)
    assert ms[1] < ms[0] and ms[2] < ms[0], ms
    assert nodes[2] == nodes[0], nodes
    assert abs(visits[2] - visits[0]) <= 1e-4 * visits[0], visits


def test_auto_builder_picks_by_size(gpu_ctx):
    """AUTO: the host build for small scenes, the GPU SAH build for large ones
    rendered with many samples, the PLOC build for a large scene with few
    samples per primitive."""
    small = gpu_ctx.upload(scenes.cornell_box(8, 8, 1, 2))
    assert gpu_ctx.info(small).bvh_builder == HOST
    gpu_ctx.release(small)
    for (w, h, spp), want in (((1920, 1080, 64), GPU_SAH), ((64, 64, 1), GPU)):
        sid = gpu_ctx.upload(scenes.icosphere_field(width=w, height=h, spp=spp))
        assert gpu_ctx.info(sid).bvh_builder == want, (w, h, spp)
        gpu_ctx.release(sid)
    with pytest.raises(CgpuError) as e:
        gpu_ctx.set_bvh_builder(4)
    assert e.value.status == 1
