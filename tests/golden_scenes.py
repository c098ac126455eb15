"""The golden scenes, rebuilt from the same generator calls as
tests/golden/make_golden.py (the committed CRSD files must match them)."""
import os

import numpy as np

from cadise_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def specs():
    return {
        "cornell": scenes.cornell_box(64, 64, 16, 6),
        "field": scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48, height=36,
                                        spp=16, max_depth=8, dielectric=scenes.GLASS, box=30.0,
                                        radius_range=(2.0, 6.0)),
        "features": scenes.feature_scene(),
        "power": scenes.power_field(),
        "spheres": scenes.sphere_box(),
    }


def vectors(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_vectors.npz")))


def image(name):
    return dict(np.load(os.path.join(GOLDEN, name + "_image.npz")))


def crsd_text(name):
    with open(os.path.join(GOLDEN, name + ".crsd")) as f:
        return f.read()
