"""Film reconstruction filters: the oracle's restatement of
FilmTile::addSample (core/film/filmTile.cpp:36-66) with the box, Gaussian,
Mitchell and cone filters (core/film/filter/) against the reference's own
FilmTile on the same samples, and the CRSD film block keys.  No GPU needed."""
import os

import numpy as np
import pytest

import cadise_gb300 as cg
import oracle
from cadise_gb300 import abi, scenes
from golden_scenes import FILTER_CASES, GOLDEN

_REF = oracle.reference_dir()
SHIPPED = os.path.join(_REF, "scene", "cornell-box.crsd") if _REF else None


@pytest.fixture(scope="module")
def vec():
    return dict(np.load(os.path.join(GOLDEN, "filter_vectors.npz")))


@pytest.mark.parametrize("case", [c[0] for c in FILTER_CASES])
def test_oracle_filter_matches_reference_filmtile(vec, case):
    """Reference sensors are FP32 sums; the oracle's FP64.  Same pixels, same
    weights: agreement to FP32 summation error."""
    f = abi.film_filter_struct(dict(FILTER_CASES)[case])
    W, H = int(vec["width"]), int(vec["height"])
    film = oracle.filter_splat(f, W, H, vec["xy"], vec["rgb"])
    ref = vec["sensor_" + case]
    mine = np.concatenate([film[..., :3], film[..., 6:7]], -1)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(mine, ref, rtol=1e-5, atol=1e-6 * scale)
    # pixels the footprint never reaches stay exactly zero on both sides
    assert np.array_equal(mine[..., 3] == 0, ref[..., 3] == 0)


@pytest.mark.parametrize("case", [c[0] for c in FILTER_CASES])
def test_crsd_film_block_round_trips(case):
    f = dict(FILTER_CASES)[case]
    spec = scenes.cornell_box(16, 12, 1, 2)
    spec.film_filter = f
    got = cg.CrsdScene(text=spec.to_crsd()).desc.filter
    want = abi.film_filter_struct(f)
    for name, _ in abi.cgpu_film_filter._fields_:
        assert getattr(got, name) == pytest.approx(getattr(want, name), rel=1e-7), name


def test_crsd_filter_defaults_are_the_reference_defaults():
    """filterInstantiator.cpp:16-57: size 1 for the box, 4 for the others;
    sigma 0.5, amplitude 1; Mitchell b = c = 1/3; 16 x 16 tiles."""
    base = scenes.cornell_box(16, 12, 1, 2).to_crsd()
    for name, typ in (("gaussian", abi.CGPU_FILTER_GAUSSIAN), ("mitchell", abi.CGPU_FILTER_MITCHELL),
                      ("cone", abi.CGPU_FILTER_CONE)):
        f = cg.CrsdScene(text=base.replace('[filter string "box"]', '[filter string "%s"]' % name)).desc.filter
        assert (f.type, f.width, f.height, f.tile_width, f.tile_height) == (typ, 4.0, 4.0, 16, 16)
        assert (f.sigma_x, f.sigma_y, f.amplitude) == (0.5, 0.5, 1.0)
        assert f.b == pytest.approx(1 / 3) and f.c == pytest.approx(1 / 3)
    with pytest.raises(cg.CgpuError) as e:
        cg.CrsdScene(text=base.replace('[filter string "box"]', '[filter string "lanczos"]'))
    assert e.value.status == 5


@pytest.mark.skipif(not SHIPPED or not os.path.exists(SHIPPED), reason="reference checkout not present")
def test_shipped_reference_scene_loads():
    """The reference's own scene file (Gaussian filter, plastic, GGX conductor,
    spheres, rectangles) loads without an unsupported feature."""
    sc = cg.CrsdScene(path=SHIPPED)
    d = sc.desc
    assert d.filter.type == abi.CGPU_FILTER_GAUSSIAN and (d.width, d.height) == (640, 480)
    kind, _, _ = sc.arrays()
    assert (kind == abi.CGPU_PRIM_SPHERE).sum() == 2
    types = {d.materials[i].type for i in range(d.num_materials)}
    assert abi.CGPU_BSDF_PLASTIC in types and abi.CGPU_BSDF_CONDUCTOR_GGX in types
