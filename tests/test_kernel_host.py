"""The CUDA library's device code, compiled as host C++ (tests/native/), run on
the CPU against the reference's golden vectors and the oracle: traversal
(both the per-ray loop and the resumable stepper of the persistent kernels),
the per-path estimator, the per-path adjoint, scene construction.  Catches logic errors - wrong
hits, endless loops, wrong random-number order - before GPU time is spent.
Same tolerances as the GPU parity tests.  The host build does not contract
multiply-adds either (-ffp-contract=off), like the kernels (-fmad=false)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle
from cadise_gb300 import abi, scenes
from golden_scenes import FILTER_CASES, field1m_spec, path_close_fraction, specs, vectors
from parity_util import check_hits

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
BUILD = os.path.join(ROOT, "tests", "native", "_build")
LIB = os.path.join(BUILD, "libkhc.so")
SRCS = [os.path.join(ROOT, "tests", "native", "kernel_host_check.cpp"),
        os.path.join(ROOT, "cadise_gb300", "csrc", "scene_build.cpp"),
        os.path.join(ROOT, "cadise_gb300", "csrc", "bvh_build.cpp"),
        os.path.join(ROOT, "cadise_gb300", "csrc", "tie_order.cpp")]


def _cuda_include():
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


@pytest.fixture(scope="module")
def khc():
    deps = SRCS + [os.path.join(ROOT, "cadise_gb300", "csrc", f) for f in os.listdir(os.path.join(ROOT, "cadise_gb300", "csrc"))
                   if f.endswith((".cuh", ".h"))]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        os.makedirs(BUILD, exist_ok=True)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                               "-I", os.path.join(ROOT, "include"), "-I", _cuda_include()] + SRCS + ["-o", LIB])
    L = C.CDLL(LIB)
    L.khc_create.restype = C.c_void_p
    L.khc_create.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.khc_destroy.argtypes = [C.c_void_p]
    L.khc_set_budget.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    L.khc_ranks.argtypes = [C.c_void_p, C.c_void_p]
    L.khc_texel.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_uint32, C.c_void_p]
    L.khc_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int] + [C.c_void_p] * 5
    L.khc_paths.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    L.khc_render_paths.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
    L.khc_adjoint.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32] + [C.c_void_p] * 4
    L.khc_wf_layout_check.argtypes = [C.c_uint64, C.c_int]
    L.khc_filter_gather.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.khc_quantize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.khc_noalloc_layout_bytes.restype = C.c_uint64
    L.khc_noalloc_scratch_bytes.restype = C.c_uint64
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Host:
    def __init__(self, L, flat):
        self.L, self.flat = L, flat
        err = C.create_string_buffer(256)
        self.h = L.khc_create(C.addressof(flat.desc), err, 256)
        assert self.h, err.value

    def trace(self, rays, dyn=0):
        r = np.ascontiguousarray(rays, np.float32)
        n = r.shape[0]
        prim, occ = np.zeros(n, np.int32), np.zeros(n, np.int32)
        t, u, v = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
        self.L.khc_trace(self.h, _p(r), n, dyn, _p(prim), _p(t), _p(u), _p(v), _p(occ))
        return prim, t, occ

    def paths(self, xy, keys):
        xy = np.ascontiguousarray(xy, np.float64)
        k = np.ascontiguousarray(keys, np.uint64)
        out = np.zeros((xy.shape[0], 3), np.float32)
        self.L.khc_paths(self.h, _p(xy), _p(k), xy.shape[0], _p(out))
        return out

    def render_paths(self, seed, first, count, scene_index=0):
        d = self.flat.desc
        out = np.zeros((count, d.height, d.width, 3), np.float32)
        self.L.khc_render_paths(self.h, seed, scene_index, first, count, _p(out))
        return out

    def close(self):
        self.L.khc_destroy(self.h)


NAMES = ["cornell", "cornell256", "textured", "field", "features", "power", "spheres", "coplanar"]


@pytest.mark.parametrize("name", NAMES)
def test_kernel_traversal_matches_reference_hits(khc, name):
    v = vectors(name)
    flat = abi.flatten(specs()[name])
    h = Host(khc, flat)
    rays = v["trace_rays"]
    prim, t, occ = h.trace(rays)
    ref_p, ref_t = v["trace_bvh_prim"], v["trace_bvh_t"]
    check_hits(flat, rays, prim, t, ref_p, ref_t, name)
    both = (prim == ref_p) & (prim >= 0)
    assert np.array_equal(t[both], ref_t[both])  # the reference's own distance formula
    # the resumable stepper of the persistent kernels and the warp traversal
    # of the extend pass find the same hits
    for variant in (1, 2):
        p2, t2, occ2 = h.trace(rays, dyn=variant)
        assert np.array_equal(p2, prim) and np.array_equal(t2, t) and np.array_equal(occ2, occ)
    h.close()


@pytest.mark.parametrize("name", NAMES + ["field1m"])
def test_tie_ranks_follow_the_reference_tree(khc, name):
    """The library's exact-tie ranks (its own build of the reference's binary
    BVH, tie_order.cpp) equal the leaf order of the oracle's tree, which
    reproduces the reference's hits, ties included, on the golden rays."""
    flat = abi.flatten(field1m_spec() if name == "field1m" else specs()[name])
    h = Host(khc, flat)
    n = int(flat.desc.num_primitives)
    got = np.zeros((n, 8), np.uint32)
    khc.khc_ranks(h.h, _p(got))
    h.close()
    want = oracle.PortScene(flat).visit_ranks()
    assert np.array_equal(got, want)
    # each octant's ranks are a permutation, and the octants differ
    assert all(np.array_equal(np.sort(got[:, o]), np.arange(n)) for o in range(8))
    assert n < 3 or len({got[:, o].tobytes() for o in range(8)}) > 1


@pytest.mark.parametrize("name", NAMES)
def test_kernel_paths_match_reference(khc, name):
    v = vectors(name)
    h = Host(khc, abi.flatten(specs()[name]))
    rgb = h.paths(v["paths_xy"], v["paths_keys"])
    ref = v["paths_rgb"]
    close = np.all(np.abs(rgb - ref) <= 1e-3 * np.abs(ref) + 1e-5, axis=1)
    assert close.mean() >= path_close_fraction(name), close.mean()
    h.close()


@pytest.mark.parametrize("name", ["field", "features"])
def test_kernel_render_paths_match_oracle(khc, name):
    flat = abi.flatten(specs()[name])
    h = Host(khc, flat)
    got = h.render_paths(11, 3, 2)
    _, port = oracle.PortScene(flat).render(seed=11, first=3, count=2, threads=8, want_paths=True)
    close = np.all(np.abs(got - port) <= 1e-3 * np.abs(port) + 1e-5, axis=-1)
    assert close.mean() >= 0.99, close.mean()
    h.close()


def test_kernel_rough_dielectric_and_sky_match_oracle(khc):
    for spec in (scenes.icosphere_field(n_spheres=12, subdivision=2, n_lights=3, seed=9, width=40, height=30,
                                        spp=4, max_depth=8, dielectric=scenes.ROUGH_DIELECTRIC, box=30.0,
                                        radius_range=(2.0, 6.0)),
                 scenes.env_field(n_spheres=10, subdivision=2, n_lights=2, width=32, height=24, spp=4,
                                  max_depth=6, sky=(64, 32))):
        flat = abi.flatten(spec)
        h = Host(khc, flat)
        got = h.render_paths(3, 0, 4)
        _, port = oracle.PortScene(flat).render(seed=3, first=0, count=4, threads=8, want_paths=True)
        close = np.all(np.abs(got - port) <= 1e-3 * np.abs(port) + 1e-5, axis=-1)
        assert close.mean() >= 0.99, close.mean()
        h.close()


def test_kernel_adjoint_matches_fp64_reference(khc):
    """The adjoint's per-path replay (the kernel's own code, run on the CPU)
    against the oracle's FP64 forward-mode gradient of the same detached
    estimator: texels, GGX roughness and emitter radiance."""
    spec = scenes.diff_scene(width=32, height=32, spp=16, max_depth=3, n_spheres=10, subdivision=2,
                             tex_size=16, n_conductors=3, n_lights=2, seed=5)
    flat = abi.flatten(spec)
    h = Host(khc, flat)
    W = np.random.default_rng(5).normal(size=(spec.height, spec.width, 3)).astype(np.float32)
    spp, seed, scene_index = 16, 23, 1
    gt, gr, gl = np.zeros(16 * 16 * 3), np.zeros(len(spec.materials)), np.zeros((2, 3))
    khc.khc_adjoint(h.h, seed, scene_index, spp, _p(W), _p(gt), _p(gr), _p(gl))
    h.close()
    metals = [i for i, m in enumerate(spec.materials) if m.type == scenes.CONDUCTOR]
    top = list(np.argsort(-np.abs(gt))[:6])
    params = [(0, int(i), 0) for i in top] + [(1, i, 0) for i in metals] + [(2, 0, c) for c in range(3)] + \
             [(2, 1, c) for c in range(3)]
    ref = oracle.PortScene(flat).adjoint_fp64(seed, spp, W, params, scene_index=scene_index)
    got = np.concatenate([gt[top], gr[metals], gl[0], gl[1]])
    assert np.all(ref[:6] != 0) and np.all(ref[6:9] != 0)
    assert np.all(np.abs(got - ref) <= 1e-3 * np.abs(ref) + 1e-4 * np.abs(ref).max()), np.stack([got, ref])


def test_kernel_adjoint_roughness_of_every_ggx_bsdf_matches_fp64_reference(khc):
    """The same on the close-up of two GGX conductors and a GGX (rough)
    dielectric: d loss / d roughness of each, reflection and refraction
    half vectors, against the oracle's FP64 forward mode."""
    spec = scenes.roughness_scene(width=32, height=24)
    flat = abi.flatten(spec)
    h = Host(khc, flat)
    W = np.random.default_rng(8).normal(size=(spec.height, spec.width, 3)).astype(np.float32)
    spp, seed, scene_index = 16, 31, 0
    gt, gr, gl = np.zeros(1), np.zeros(len(spec.materials)), np.zeros((len(spec.lights), 3))
    khc.khc_adjoint(h.h, seed, scene_index, spp, _p(W), _p(gt), _p(gr), _p(gl))
    h.close()
    ggx = [i for i, m in enumerate(spec.materials) if m.type in (scenes.CONDUCTOR, scenes.ROUGH_DIELECTRIC)]
    assert any(spec.materials[i].type == scenes.ROUGH_DIELECTRIC for i in ggx)
    ref = oracle.PortScene(flat).adjoint_fp64(seed, spp, W, [(1, i, 0) for i in ggx], scene_index=scene_index)
    got = gr[ggx]
    assert np.all(ref != 0)
    assert np.all(np.abs(got - ref) <= 1e-3 * np.abs(ref) + 1e-4 * np.abs(ref).max()), np.stack([got, ref])


@pytest.mark.parametrize("cap", [1, 63, 20000, 1 << 14, 2073600, (1 << 21) + 5])
def test_wavefront_buffer_layout_fits(khc, cap):
    """The path-state arrays of the wavefront stay inside the block they are
    carved from, for capacities that are not multiples of the alignment."""
    for rows in (3, 34, 66):
        assert khc.khc_wf_layout_check(cap, rows) == 0


def test_noalloc_scratch_holds_its_layout(khc):
    """Header, batch tables and the path state of 262144 paths fit the 80 MiB
    static array of cgpu_render_noalloc."""
    need, have = khc.khc_noalloc_layout_bytes(), khc.khc_noalloc_scratch_bytes()
    assert have == 80 << 20
    assert 0 < need <= have, (need, have)


@pytest.mark.parametrize("case", [c[0] for c in FILTER_CASES])
def test_kernel_filter_gather_matches_oracle(khc, case):
    """The splat kernel's gather over the pixels of each tile (film.cuh) and
    the oracle's scatter restatement of FilmTile::addSample add the same
    weights to the same pixels: equal up to the order of the FP64 sums.
    Samples include positions on exact pixel edges (where the footprint
    reaches one pixel further) and NaN / Inf radiance."""
    import oracle
    f = abi.film_filter_struct(dict(FILTER_CASES)[case])
    W, H, count = 37, 29, 3
    rng = np.random.default_rng(5)
    pix = np.stack(np.meshgrid(np.arange(W), np.arange(H)), -1).astype(np.float32)  # H x W x 2 (x, y)
    jit = rng.uniform(0, 1, (count, H, W, 2)).astype(np.float32)
    jit[0, ::3, ::2] = 0.0  # exact pixel corners
    xy = (pix[None] + jit).astype(np.float32)
    rgb = rng.uniform(0, 3, (count, H, W, 3)).astype(np.float32)
    rgb[1, 4, 5, 0] = np.nan
    rgb[2, 10, 11, 1] = np.inf
    film = np.zeros((H, W, 7), np.float64)
    assert khc.khc_filter_gather(C.byref(f), W, H, count, _p(xy), _p(rgb), _p(film)) == 0
    ref = oracle.filter_splat(f, W, H, xy.reshape(-1, 2), rgb.reshape(-1, 3))
    scale = np.abs(ref).max(axis=(0, 1))
    np.testing.assert_allclose(film, ref, rtol=1e-12, atol=1e-12 * scale.max())
    assert ref[..., 6].min() != ref[..., 6].max()


def test_invalid_film_filter_is_rejected(khc):
    spec = scenes.cornell_box(8, 8, 1, 2)
    flat = abi.flatten(spec)
    for bad in (dict(type=7), dict(type=abi.CGPU_FILTER_GAUSSIAN, width=4.0, height=4.0, sigma_x=0.0, sigma_y=0.5),
                dict(type=abi.CGPU_FILTER_CONE, width=-1.0, height=2.0), dict(type=0, tile_width=-3)):
        flat.desc.filter = abi.cgpu_film_filter(**bad)
        err = C.create_string_buffer(256)
        assert not khc.khc_create(C.addressof(flat.desc), err, 256)
        assert b"filter" in err.value or b"tile" in err.value, err.value


def decode_node(raw):
    """The 64-byte quantized node (scene_device.cuh) to FP64 child boxes."""
    org = np.frombuffer(raw[0:12], np.float32).astype(np.float64)
    exps = np.frombuffer(raw[12:16], np.uint8)[:3].astype(int) - 127
    planes = np.frombuffer(raw[32:56], np.uint8).reshape(6, 4).astype(np.float64)  # lox hix loy hiy loz hiz
    step = np.ldexp(1.0, exps)
    lo = org[None, :] + planes[0::2].T * step[None, :]
    hi = org[None, :] + planes[1::2].T * step[None, :]
    child = np.frombuffer(raw[16:32], np.uint32)
    return lo, hi, step, child


@pytest.mark.parametrize("scale", [1e-3, 1.0, 37.5, 1e4])
def test_quantized_nodes_are_conservative_and_tight(khc, scale):
    """Every decoded child box contains its box and exceeds it by less than
    one step per plane; the union spans at most 254 steps; the steps are
    powers of two no finer than the float spacing of the coordinates.
    Boxes far from the origin, flat boxes and identical boxes included."""
    rng = np.random.default_rng(int(scale * 7) + 1)
    for trial in range(300):
        nk = int(rng.integers(1, 5))
        centre = rng.normal(0, 50 * scale, 3) if trial % 3 else rng.normal(0, 1e4 * scale, 3)
        lo = centre + rng.uniform(-scale, scale, (nk, 3))
        ext = rng.uniform(0, scale, (nk, 3)) * (rng.uniform(size=(nk, 3)) > 0.1)  # some flat axes
        hi = lo + ext
        if trial % 17 == 0:
            lo[:] = lo[0]
            hi[:] = hi[0]
        lo32, hi32 = lo.astype(np.float32), hi.astype(np.float32)
        hi32 = np.maximum(hi32, lo32)
        raw = np.zeros(64, np.uint8)
        khc.khc_quantize(_p(np.ascontiguousarray(lo32)), _p(np.ascontiguousarray(hi32)), nk, _p(raw))
        dlo, dhi, step, child = decode_node(raw.tobytes())
        assert list(child[:nk]) == [1, 2, 3, 4][:nk] and not child[nk:].any()
        assert np.all(dlo[:nk] <= lo32) and np.all(dhi[:nk] >= hi32)
        assert np.all(lo32 - dlo[:nk] < step) and np.all(dhi[:nk] - hi32 < step)
        span = (hi32.max(0) - lo32.min(0)) / step
        assert np.all(span <= 254.0)
        mag = np.maximum(np.abs(lo32).max(0), np.abs(hi32).max(0))
        assert np.all(step >= mag * 2.0 ** -22 * 0.999)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_visit_budget_stops_traversals_and_counts_them(khc, variant):
    """The device-side iteration budget, on the CPU: with 3 node and leaf
    visits per ray every traversal variant (per-ray loop, resumable stepper
    of the persistent kernels, warp traversal) stops early and counts its
    rays; with the automatic budget (5 x nodes + 64) none runs out and the
    hits are the reference's again."""
    v = vectors("field")
    flat = abi.flatten(specs()["field"])
    h = Host(khc, flat)
    status = np.zeros(1, np.uint32)
    rays = v["trace_rays"]
    khc.khc_set_budget(h.h, 3, _p(status))
    prim_cut, _, _ = h.trace(rays, dyn=variant)
    assert status[0] > 0
    assert not np.array_equal(prim_cut, v["trace_bvh_prim"])
    status[0] = 0
    khc.khc_set_budget(h.h, 0, _p(status))
    prim, t, occ = h.trace(rays, dyn=variant)
    assert status[0] == 0
    assert np.array_equal(prim, v["trace_bvh_prim"])
    h.close()


def test_kernel_texel_lookup_matches_reference_texture(khc):
    """The kernels' nearest / repeat texel lookup (texture_rgb) against the
    reference's RgbImageTexture::evaluate (rgbImageTexture.cpp:8-15,
    tNearestPixelSampler.ipp:14-31, repeatUvwWrapper.cpp:9-15) on uvws on
    texel borders, just below them, negative, at 1 and far outside:
    bit-identical texels."""
    v = dict(np.load(os.path.join(ROOT, "tests", "golden", "texel_vectors.npz")))
    h = Host(khc, abi.flatten(specs()["textured"]))
    uvw = np.ascontiguousarray(v["uvw"], np.float32)
    out = np.zeros_like(uvw)
    khc.khc_texel(h.h, 0, _p(uvw), uvw.shape[0], _p(out))
    assert np.array_equal(out, v["rgb"]), np.where(np.any(out != v["rgb"], axis=1))[0][:10]
    # the border cases are there: u = k / width exactly, negative and >= 1
    w = specs()["textured"].textures[0].texels.shape[1]
    borders = np.arange(-2 * w, 3 * w + 1, dtype=np.float64) / w
    assert np.isin(uvw[:, 0], borders.astype(np.float32)).sum() >= 20
    assert (uvw[:, 0] < 0).any() and (uvw[:, 0] >= 1).any()
    h.close()
