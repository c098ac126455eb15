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
        "field": scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48, height=36,
                                        spp=16, max_depth=8, dielectric=scenes.GLASS, box=30.0,
                                        radius_range=(2.0, 6.0)),
        "features": scenes.feature_scene(),
        "power": scenes.power_field(),
        "spheres": scenes.sphere_box(),
        "filtered": filtered_scene(),
    }


def vectors(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_vectors.npz")))


def image(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_image.npz")))


def crsd_text(name):
    with open(os.path.join(GOLDEN, name + ".crsd")) as f:
        return f.read()
