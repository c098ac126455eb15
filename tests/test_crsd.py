"""The library's CRSD loader (host C++, include/cadise_crsd.h) against the
scene generator's own flattening, the reference's format rules and its
error handling.  No GPU needed."""
import numpy as np
import pytest

import cadise_gb300 as cg
from cadise_gb300 import CgpuError, abi, scenes
from golden_scenes import GOLDEN, specs

import os


@pytest.fixture(scope="module", autouse=True)
def built():
    cg.build()


@pytest.mark.parametrize("name", ["cornell", "field", "features", "power", "spheres", "filtered"])
def test_golden_crsd_loads_to_the_generator_arrays(name):
    sc = cg.CrsdScene(path=os.path.join(GOLDEN, name + ".crsd"))
    flat = abi.flatten(specs()[name])
    kind, verts, mat = sc.arrays()
    assert np.array_equal(kind, flat.kind)
    assert np.array_equal(verts, flat.vertices)
    assert np.array_equal(mat, flat.material)
    d, f = sc.desc, flat.desc
    assert (d.width, d.height, d.max_depth, d.spp) == (f.width, f.height, f.max_depth, f.spp)
    assert list(d.cam_position) == list(f.cam_position) and d.fov_degrees == f.fov_degrees
    assert d.num_lights == f.num_lights and d.num_materials == f.num_materials
    for i in range(d.num_lights):
        a, b = d.lights[i], f.lights[i]
        assert (a.primitive, list(a.color), a.watt, a.back_face_emit) == (b.primitive, list(b.color), b.watt, b.back_face_emit)
    for i in range(d.num_materials):
        a, b = d.materials[i], f.materials[i]
        assert a.type == b.type
        if a.type == abi.CGPU_BSDF_CONDUCTOR_GGX:
            assert list(a.f0) == list(b.f0) and a.roughness == b.roughness
        elif a.type != abi.CGPU_BSDF_PHONG:  # phong has no albedo
            assert list(a.albedo) == list(b.albedo)
        if a.type in (abi.CGPU_BSDF_GLASS, abi.CGPU_BSDF_DIELECTRIC_GGX) or \
                (a.type == abi.CGPU_BSDF_MIRROR and a.fresnel == 1):
            assert a.ior_inner == b.ior_inner and a.ior_outer == b.ior_outer
        if a.type == abi.CGPU_BSDF_MIRROR:
            assert a.fresnel == b.fresnel and (a.fresnel == 1 or list(a.f0) == list(b.f0))
        if a.type in (abi.CGPU_BSDF_PHONG, abi.CGPU_BSDF_PLASTIC):
            assert a.exponent == b.exponent
        if a.type == abi.CGPU_BSDF_PLASTIC:
            assert a.diffuse_ratio == b.diffuse_ratio
    if flat.normals is not None:
        n = np.ctypeslib.as_array(d.prim_normals, shape=(d.num_primitives, 9))
        assert np.array_equal(n, flat.normals)
    st = sc.settings()
    assert st.renderer_type == b"sampling" and st.estimator == b"pt" and st.spp == f.spp


def test_comments_and_first_match_wins():
    text = """
    # a comment with [brackets] and {braces
    film { [image-width int32 "8"] [image-height int32 "6"] [filter string "box"] }
    camera { [type string "perspective-pinhole"] [position vector3r "0 0 -5"]
             [direction vector3r "0 0 1"] [up vector3r "0 1 0"] [fov real "40"] [fov real "90"] }
    renderer { [type string "cuda-sampling"] [sample-number int32 "3"] [estimator string "pt"]
               [mode string "megakernel"] [seed int32 "17"] }
    material { [type string "matte-lambertian"] [name string "m"] [albedo rgb "0.1 0.2 0.3"] }
    primitive { [type string "rectangle"] [name string "q"] [bsdf material "m"]
                [v1 vector3r "1 0 0"] [v2 vector3r "0 0 0"] [v3 vector3r "0 1 0"] }
    light { [type string "area"] [primitive primitive "q"] [color rgb "1 1 1"] [watt real "10"] }
    """
    sc = cg.CrsdScene(text=text)
    assert sc.desc.fov_degrees == 40.0
    assert sc.desc.max_depth == 10000  # the reference's default max-depth
    st = sc.settings()
    assert st.mode == cg.CGPU_MODE_MEGAKERNEL and st.seed == 17 and st.spp == 3
    assert sc.primitive_index("q") == 0


def test_mesh_name_maps_to_its_first_triangle():
    s = scenes.cornell_box(8, 8, 1, 2)
    sc = cg.CrsdScene(text=s.to_crsd())
    assert sc.primitive_index("shortBox") == 5
    assert sc.primitive_index("tallBox") == 17
    assert sc.primitive_index("light") == 29
    assert sc.primitive_index("nope") == -1


@pytest.mark.parametrize("bad,status", [
    ("film { [image-width int32 \"4\"] }", 7),                                   # no camera / renderer
    ("material { [type string \"cloth\"] [name string \"x\"] }", 5),              # unsupported BSDF
    ("camera { [fov real \"abc\"] }", 7),                                         # not a number
])
def test_errors_are_status_codes(bad, status):
    with pytest.raises(CgpuError) as e:
        cg.CrsdScene(text=bad)
    assert e.value.status == status


def test_missing_file_is_not_found():
    with pytest.raises(CgpuError) as e:
        cg.CrsdScene(path="/nonexistent/scene.crsd")
    assert e.value.status == 6


def test_binary_mesh_sidecars_load_like_text(tmp_path):
    """Large meshes written as float32 sidecars load to the same arrays as
    the text vector3r-array form (and much faster)."""
    import time
    spec = scenes.icosphere_field(n_spheres=20, subdivision=3, width=32, height=32, spp=1)
    path = str(tmp_path / "field.crsd")
    spec.write_crsd(path, sidecar_min_triangles=100)
    t0 = time.perf_counter()
    sc = cg.CrsdScene(path=path)
    t_bin = time.perf_counter() - t0
    t0 = time.perf_counter()
    txt = cg.CrsdScene(text=spec.to_crsd())
    t_txt = time.perf_counter() - t0
    a, b = sc.arrays(), txt.arrays()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert t_bin < t_txt
