"""The FP64 reference gradient of the oracle (forward-mode dual numbers,
detached sampling) against central finite differences of the oracle's own
renders with common random numbers.  Roulette is off (max depth 3), so for
emitter radiance and albedo texels the same-seed estimator is smooth and the
two must agree to FP32 rounding of the finite-difference renders."""
import copy

import numpy as np
import pytest

import oracle
from cadise_gb300 import abi, scenes

SEED, SPP = 21, 32


@pytest.fixture(scope="module")
def spec():
    return scenes.diff_scene(width=20, height=16, spp=SPP, max_depth=3, n_spheres=8, subdivision=1,
                             tex_size=8, n_conductors=2, n_lights=2, seed=6)


def loss_of(s, W):
    film, _ = oracle.PortScene(abi.flatten(s)).render(seed=SEED, first=0, count=SPP, threads=8)
    img = film[..., :3] / film[..., 6:7]
    return float((W * img).sum())


def test_radiance_gradient_against_finite_differences(spec):
    W = np.random.default_rng(1).normal(size=(spec.height, spec.width, 3))
    ps = oracle.PortScene(abi.flatten(spec))
    for l in range(len(spec.lights)):
        g = ps.adjoint_fp64(SEED, SPP, W.astype(np.float32), [(2, l, c) for c in range(3)])
        rad = ps_radiance(spec, l)
        h = 1e-3
        sp, sm = copy.deepcopy(spec), copy.deepcopy(spec)
        sp.lights[l].watt *= 1 + h
        sm.lights[l].watt *= 1 - h
        fd = (loss_of(sp, W) - loss_of(sm, W)) / (2 * h)  # d loss / d log(watt)
        pred = float((g * rad).sum())
        assert abs(fd - pred) <= 2e-3 * abs(fd) + 1e-9, (l, fd, pred)


def ps_radiance(spec, l):
    lt = spec.lights[l]
    prim = next(p for p in spec.primitives if getattr(p, "name", None) == lt.primitive)
    v1, v2, v3 = (np.array(x, np.float64) for x in (prim.v1, prim.v2, prim.v3))
    area = np.linalg.norm(v1 - v2) * np.linalg.norm(v3 - v2)
    c = np.array(lt.color, np.float64)
    return c / c.sum() * lt.watt / (area * np.pi)


def test_texel_gradient_against_finite_differences(spec):
    W = np.random.default_rng(2).normal(size=(spec.height, spec.width, 3))
    ps = oracle.PortScene(abi.flatten(spec))
    tex = spec.textures[0].texels
    # texels actually seen: the ones with the largest gradient among a coarse probe
    probe = [(0, i, 0) for i in range(0, tex.size, max(1, tex.size // 16))][:16]
    g = ps.adjoint_fp64(SEED, SPP, W.astype(np.float32), probe)
    order = np.argsort(-np.abs(g))[:3]
    assert abs(g[order[0]]) > 0
    for j in order:
        i = probe[j][1]
        h = 1e-3 * float(tex.reshape(-1)[i])
        sp, sm = copy.deepcopy(spec), copy.deepcopy(spec)
        sp.textures[0].texels.reshape(-1)[i] += h
        sm.textures[0].texels.reshape(-1)[i] -= h
        fd = (loss_of(sp, W) - loss_of(sm, W)) / (2 * h)
        assert abs(fd - g[j]) <= 5e-3 * abs(fd) + 1e-7, (i, fd, g[j])


def test_roughness_gradient_is_finite_and_nonzero(spec):
    W = np.ones((spec.height, spec.width, 3), np.float32)
    ps = oracle.PortScene(abi.flatten(spec))
    metals = [i for i, m in enumerate(spec.materials) if m.type == scenes.CONDUCTOR]
    g = ps.adjoint_fp64(SEED, SPP, W, [(1, i, 0) for i in metals])
    assert np.all(np.isfinite(g)) and np.any(g != 0)
