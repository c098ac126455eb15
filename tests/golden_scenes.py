"""The golden scenes, rebuilt from the same generator calls as
tests/golden/make_golden.py (the committed CRSD files must match them)."""
import os

import numpy as np

from cadise_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def filtered_scene():
    """The sphere box with the reference's default Gaussian film filter
    (4 x 4 pixels, sigma 0.5) on 16 x 16 tiles."""
    s = scenes.sphere_box()
    s.film_filter = scenes.FilmFilter("gaussian")
    return s


# Film filter cases of filter_vectors.npz: (name, FilmFilter).
FILTER_CASES = [
    ("box1", scenes.FilmFilter("box")),
    ("box2_5", scenes.FilmFilter("box", width=2.5, height=1.5)),
    ("gauss", scenes.FilmFilter("gaussian")),
    ("gauss_wide", scenes.FilmFilter("gaussian", width=3.0, height=5.0, sigma_x=0.8, sigma_y=1.3, amplitude=2.0)),
    ("mitchell", scenes.FilmFilter("mitchell")),
    ("catmull_rom", scenes.FilmFilter("mitchell", b=0.0, c=0.5, tile=(8, 12))),
    ("cone", scenes.FilmFilter("cone")),
    ("cone_small_tiles", scenes.FilmFilter("cone", width=3.0, height=3.0, tile=(5, 7))),
]


def specs():
    return {
        "cornell": scenes.cornell_box(64, 64, 16, 6),
        # the first configuration itself: 256 x 256, 16 spp, depth 6
        "cornell256": scenes.cornell_box(),
        "textured": scenes.texture_scene(),
        "field": scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48, height=36,
                                        spp=16, max_depth=8, dielectric=scenes.GLASS, box=30.0,
                                        radius_range=(2.0, 6.0)),
        "features": scenes.feature_scene(),
        "power": scenes.power_field(),
        "spheres": scenes.sphere_box(),
        "filtered": filtered_scene(),
        # coplanar, overlapping primitives: the reference's tie order
        "coplanar": scenes.coplanar_scene(),
    }


def field1m_spec(width=1920, height=1080):
    """The second configuration's 1,024,000-triangle field with the GGX
    dielectric replaced by the reference's smooth glass (the reference has no
    rough dielectric); same geometry, lights and camera."""
    return scenes.icosphere_field(dielectric=scenes.GLASS, width=width, height=height)


# Fraction of the golden paths whose radiance must match the reference's to
# 1e-3: 99 %, except in the coplanar scene, where a rectangle and a triangle
# mesh share a plane: their reference distances come from two different
# formulas and differ by a rounding, so a bounce perturbed by an ulp upstream
# (a transcendental of another libm) meets them in either order - about 1 %
# of its paths end on the other tile.  Its exact rays (the trace vectors) tie
# bit for bit.
def path_close_fraction(name):
    return 0.98 if name == "coplanar" else 0.99


def vectors(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_vectors.npz")))


def image(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_image.npz")))


def image_mean_var(name):
    """Per pixel the reference render's mean and the variance of that mean,
    from either golden film layout (FP64 sums, or FP32 mean / sample variance)."""
    ref = image(name)
    if "mean" in ref:
        n = ref["count"][..., None].astype(np.float64)
        return ref["mean"].astype(np.float64), ref["var"].astype(np.float64) / n
    n = ref["count"][..., None]
    mean = ref["sum"] / n
    return mean, (ref["sum_sq"] / n - mean ** 2) / n


def scene_digest(flat) -> str:
    """SHA-1 of a flattened scene's arrays (geometry, materials, lights,
    textures), as tests/golden/make_golden.py records it for a large golden
    scene that is rebuilt rather than committed."""
    import hashlib
    h = hashlib.sha1()
    for a in (flat.kind, flat.vertices, flat.material):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(bytes(flat.materials))
    h.update(bytes(flat.lights))
    for t in flat.texture_arrays:
        h.update(t.tobytes())
    return h.hexdigest()


def exact_rays(spec, n, seed):
    """Seeded rays from exactly rounded operations only (uniform draws,
    +, *, /, sqrt), so that every platform regenerates the same bits: 40 %
    from the camera towards points in the sphere cube, 60 % from points in
    the cube in uniform directions (half of those with a finite t_max)."""
    rng = np.random.default_rng(seed)
    box = 100.0
    o = rng.random((n, 3)) * box
    nc = (2 * n) // 5
    cam = np.array(spec.cam_position, np.float64)
    o[:nc] = cam
    tgt = rng.random((nc, 3)) * box
    d = np.empty((n, 3))
    d[:nc] = tgt - cam
    m = n - nc
    got = 0
    while got < m:
        c = rng.random((2 * m, 3)) * 2.0 - 1.0
        r2 = c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1] + c[:, 2] * c[:, 2]
        c = c[(r2 > 1e-4) & (r2 <= 1.0)][:m - got]
        d[nc + got:nc + got + len(c)] = c
        got += len(c)
    d /= np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])[:, None]
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = o
    rays[:, 3] = 1e-3
    rays[:, 4:7] = d
    finite = rng.random(n) < 0.5
    finite[:nc] = False
    rays[:, 7] = np.where(finite, (0.1 + 0.9 * rng.random(n)) * box, 3.4028235e38)
    return rays


def crsd_text(name):
    with open(os.path.join(GOLDEN, name + ".crsd")) as f:
        return f.read()
