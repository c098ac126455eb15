"""The path-replay adjoint (cgpu_adjoint_backward) against central finite
differences of the forward renderer (cgpu_adjoint_forward) with common random
numbers (same seed, same samples), FP64 film accumulation.

Loss: linear, loss = sum(W * image) with a fixed weight image W, so
d loss / d image = W.  With roulette off (max depth 3) the same-seed
estimator is polynomial in the albedo texels and linear in the emitter
radiances, so adjoint and finite differences agree to FP32 noise; the GGX
roughness moves the sampled directions (finite differences see that, the
detached adjoint does not), so there the two agree in expectation and the
check is statistical over independent seeds, with enough of them that four
standard errors are at most 1 % of the gradient and the bar is 2 %.  The
differentiable configuration itself (512 x 512, 256^2 texture, 8
roughnesses, 4 lights, roulette on) is checked the same way.
"""
import numpy as np
import pytest

from cadise_gb300 import scenes

pytestmark = pytest.mark.gpu

H = 1e-3


@pytest.fixture(scope="module")
def diff(gpu_ctx):
    spec = scenes.diff_scene(width=48, height=48, spp=64, max_depth=3, n_spheres=10, subdivision=2,
                             tex_size=16, n_conductors=3, n_lights=2, seed=5)
    sid = gpu_ctx.upload(spec)
    yield spec, sid
    gpu_ctx.release(sid)


def weights(spec, seed=3):
    return np.random.default_rng(seed).normal(size=(spec.height, spec.width, 3)).astype(np.float32)


def loss(ctx, sid, W, spp, seed):
    img = ctx.adjoint_forward(sid, spp, seed).astype(np.float64)
    return float((W.astype(np.float64) * img).sum())


def test_params_round_trip(gpu_ctx, diff):
    spec, sid = diff
    tex, rough, rad = gpu_ctx.get_params(sid)
    assert tex.size == 16 * 16 * 3
    np.testing.assert_array_equal(tex, spec.textures[0].texels.reshape(-1))
    assert rough.size == len(spec.materials) and rad.shape == (2, 3)
    gpu_ctx.set_params(sid, texels=tex * 0.5, roughness=rough, radiance=rad)
    t2, _, _ = gpu_ctx.get_params(sid)
    np.testing.assert_array_equal(t2, tex * 0.5)
    gpu_ctx.set_params(sid, texels=tex)


def test_zero_and_linear_in_loss_gradient(gpu_ctx, diff):
    spec, sid = diff
    z = np.zeros((spec.height, spec.width, 3), np.float32)
    gt, gr, gl = gpu_ctx.adjoint_backward(sid, 16, 7, z)
    assert not gt.any() and not gr.any() and not gl.any()
    W1, W2 = weights(spec, 1), weights(spec, 2)
    a = gpu_ctx.adjoint_backward(sid, 16, 7, W1)
    b = gpu_ctx.adjoint_backward(sid, 16, 7, W2)
    c = gpu_ctx.adjoint_backward(sid, 16, 7, W1 + W2)
    for x, y, s in zip(a, b, c):
        np.testing.assert_allclose(x + y, s, rtol=1e-4, atol=1e-9 * (np.abs(s).max() + 1))


def test_radiance_gradient_matches_finite_differences(gpu_ctx, diff):
    spec, sid = diff
    W = weights(spec)
    spp, seed = 256, 11
    _, _, gl = gpu_ctx.adjoint_backward(sid, spp, seed, W)
    tex, rough, rad = gpu_ctx.get_params(sid)
    for l in range(rad.shape[0]):
        for c in range(3):
            h = H * rad[l, c]
            r = rad.copy()
            r[l, c] += h
            gpu_ctx.set_params(sid, radiance=r)
            lp = loss(gpu_ctx, sid, W, spp, seed)
            r[l, c] -= 2 * h
            gpu_ctx.set_params(sid, radiance=r)
            lm = loss(gpu_ctx, sid, W, spp, seed)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - gl[l, c]) <= 2e-3 * abs(fd) + 1e-6, (l, c, fd, gl[l, c])
    gpu_ctx.set_params(sid, radiance=rad)


def test_texel_gradient_matches_finite_differences(gpu_ctx, diff):
    spec, sid = diff
    W = weights(spec)
    spp, seed = 256, 13
    gt, _, _ = gpu_ctx.adjoint_backward(sid, spp, seed, W)
    tex, _, _ = gpu_ctx.get_params(sid)
    top = np.argsort(-np.abs(gt))[:6]
    assert np.abs(gt[top[0]]) > 0
    for i in top:
        h = H * tex[i]
        t = tex.copy()
        t[i] += h
        gpu_ctx.set_params(sid, texels=t)
        lp = loss(gpu_ctx, sid, W, spp, seed)
        t[i] -= 2 * h
        gpu_ctx.set_params(sid, texels=t)
        lm = loss(gpu_ctx, sid, W, spp, seed)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gt[i]) <= 5e-3 * abs(fd) + 1e-6, (i, fd, gt[i])
    gpu_ctx.set_params(sid, texels=tex)


def pixel_masks(ctx, sid, spec, flat, materials):
    """Per material, W = 1 on the pixels whose centre sees it directly."""
    h, w = spec.height, spec.width
    xy = np.stack(np.meshgrid(np.arange(w) + 0.5, np.arange(h) + 0.5), -1).reshape(-1, 2).astype(np.float64)
    cam = ctx.camera_rays(sid, xy)
    rays = np.zeros((len(xy), 8), np.float32)
    rays[:, :3], rays[:, 3], rays[:, 4:7], rays[:, 7] = cam[:, :3], 1e-3, cam[:, 3:6], 3e38
    prim = ctx.trace_closest(sid, rays)[0]
    seen = np.where(prim >= 0, flat.material[np.maximum(prim, 0)], -1).reshape(h, w)
    return {m: np.repeat((seen == m)[..., None], 3, -1).astype(np.float32) for m in materials}


def roughness_fd_check(ctx, spec, materials, nseeds, spp, step, seed0):
    """Per material m: with W the pixels that see m, the adjoint's d loss /
    d roughness_m and the central finite difference (common random
    numbers, FP64 films) over `nseeds` independent seeds.  Both estimate
    the same derivative; per seed they differ by noise (the finite
    difference also sees sampled directions move, and a path whose shadow
    or next ray crosses an edge jumps).  Returns (mean adjoint gradient,
    mean difference, standard error of the difference) per material."""
    from cadise_gb300 import abi
    flat = abi.flatten(spec)
    sid = ctx.upload(flat)
    try:
        tex, rough, rad = ctx.get_params(sid)
        Ws = pixel_masks(ctx, sid, spec, flat, materials)
        adj = np.zeros((nseeds, len(materials)))
        fd = np.zeros((nseeds, len(materials)))
        for k in range(nseeds):
            seed = seed0 + k
            for j, m in enumerate(materials):
                assert Ws[m].sum() > 0
                adj[k, j] = ctx.adjoint_backward(sid, spp, seed, Ws[m])[1][m]
                r = rough.copy()
                r[m] += step
                ctx.set_params(sid, roughness=r)
                lp = loss(ctx, sid, Ws[m], spp, seed)
                r[m] -= 2 * step
                ctx.set_params(sid, roughness=r)
                lm = loss(ctx, sid, Ws[m], spp, seed)
                ctx.set_params(sid, roughness=rough)
                fd[k, j] = (lp - lm) / (2 * step)
        d = fd - adj
        return adj.mean(0), d.mean(0), d.std(0, ddof=1) / np.sqrt(nseeds)
    finally:
        ctx.release(sid)


def test_roughness_gradient_matches_finite_differences(gpu_ctx):
    """GGX conductor roughness within 2 % of central finite differences,
    with enough independent seeds that four standard errors of the
    difference are at most 1 % of the gradient (the check has teeth at 2 %).
    Close-up scene (scenes.roughness_scene: two conductors and a rough
    dielectric), depth 3, 192 seeds x 4,096 spp, step 0.02 (the central
    difference's curvature error at that step is far below the noise)."""
    spec = scenes.roughness_scene()
    conductors = [i for i, m in enumerate(spec.materials) if m.type == scenes.CONDUCTOR]
    g, dm, se = roughness_fd_check(gpu_ctx, spec, conductors, nseeds=192, spp=4096, step=0.02, seed0=1000)
    print("roughness (close-up): gradient %s, (fd - adjoint) / |g| %s, 4 SE / |g| %s"
          % (g, dm / np.abs(g), 4 * se / np.abs(g)))
    assert np.all(4 * se <= 0.01 * np.abs(g)), (g, se)
    assert np.all(np.abs(dm) <= 0.02 * np.abs(g)), (g, dm)


def test_config4_gradients_match_finite_differences(gpu_ctx):
    """The differentiable configuration itself: 102,400-triangle scene,
    512 x 512, 256 x 256 albedo texture, 8 conductor roughnesses, 4 light
    radiances, depth 6 with Russian roulette on; FP64 films of 4,096 spp.
    Radiance (channel 0 of every light) and the four texels with the largest
    gradients: central differences with h = 1e-3 relative, one seed, within
    2 %.  Roughness: with h = 1e-3 a 4,096-spp difference is dominated by
    paths whose sampled directions cross an edge or whose roulette decision
    flips (measured: standard errors of 100 % and more), so the conductor
    with the most pixels of its own among those whose noise allows it is
    checked with step 0.02 over 32 seeds: 4 SE <= 1 % and within 2 %."""
    spec = scenes.diff_scene()
    assert spec.max_depth > 3  # roulette on (after the third bounce)
    sid = gpu_ctx.upload(spec)
    try:
        W = np.random.default_rng(3).normal(size=(spec.height, spec.width, 3)).astype(np.float32)
        spp, seed = 4096, 11
        gt, gr, gl = gpu_ctx.adjoint_backward(sid, spp, seed, W)
        tex, rough, rad = gpu_ctx.get_params(sid)
        assert tex.size == 256 * 256 * 3 and (rad.shape[0], len(rough)) == (4, len(spec.materials))
        for l in range(rad.shape[0]):
            h = H * rad[l, 0]
            r = rad.copy()
            r[l, 0] += h
            gpu_ctx.set_params(sid, radiance=r)
            lp = loss(gpu_ctx, sid, W, spp, seed)
            r[l, 0] -= 2 * h
            gpu_ctx.set_params(sid, radiance=r)
            lm = loss(gpu_ctx, sid, W, spp, seed)
            gpu_ctx.set_params(sid, radiance=rad)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - gl[l, 0]) <= 0.02 * abs(fd), ("radiance", l, fd, gl[l, 0])
        for i in np.argsort(-np.abs(gt))[:4]:
            h = H * tex[i]
            t = tex.copy()
            t[i] += h
            gpu_ctx.set_params(sid, texels=t)
            lp = loss(gpu_ctx, sid, W, spp, seed)
            t[i] -= 2 * h
            gpu_ctx.set_params(sid, texels=t)
            lm = loss(gpu_ctx, sid, W, spp, seed)
            gpu_ctx.set_params(sid, texels=tex)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - gt[i]) <= 0.02 * abs(fd), ("texel", int(i), fd, gt[i])
    finally:
        gpu_ctx.release(sid)
    metal = [i for i, m in enumerate(spec.materials) if m.type == scenes.CONDUCTOR][2]
    g, dm, se = roughness_fd_check(gpu_ctx, spec, [metal], nseeds=32, spp=4096, step=0.02, seed0=500)
    print("roughness (config 4, material %d): gradient %s, (fd - adjoint) / |g| %s, 4 SE / |g| %s"
          % (metal, g, dm / np.abs(g), 4 * se / np.abs(g)))
    assert np.all(4 * se <= 0.01 * np.abs(g)), (g, se)
    assert np.all(np.abs(dm) <= 0.02 * np.abs(g)), (g, dm)


def test_adjoint_matches_fp64_reference_gradient(gpu_ctx, diff):
    """Seed for seed: the GPU's FP32 path replay with FP64 reductions against
    the oracle's FP64 forward-mode gradient of the same detached estimator.
    The paths are the same, so all parameter kinds agree to FP32 rounding
    (1 % allows for the rare path that branches differently on the GPU)."""
    import oracle
    from cadise_gb300 import abi
    spec, sid = diff
    W = weights(spec, 5)
    spp, seed = 64, 23
    gt, gr, gl = gpu_ctx.adjoint_backward(sid, spp, seed, W)
    ps = oracle.PortScene(abi.flatten(spec))
    metals = [i for i, m in enumerate(spec.materials) if m.type == scenes.CONDUCTOR]
    top = list(np.argsort(-np.abs(gt))[:6])
    params = [(0, int(i), 0) for i in top] + [(1, i, 0) for i in metals] + [(2, 0, c) for c in range(3)]
    ref = ps.adjoint_fp64(seed, spp, W, params, scene_index=sid)
    gpu = np.concatenate([gt[top], gr[metals], gl[0]])
    scale = np.abs(ref).max()
    assert np.all(np.abs(gpu - ref) <= 0.01 * np.abs(ref) + 1e-4 * scale), np.stack([gpu, ref])


def test_ggx_roughness_gradients_match_fp64_reference_gradient(gpu_ctx):
    """Seed for seed, the roughness gradients of two GGX conductors and a GGX
    (rough) dielectric - reflection and refraction half vectors - against
    the oracle's FP64 forward-mode gradient of the same detached estimator
    (1 %, as above).  The dielectric's finite difference is dominated by
    caustic paths, so this is its check."""
    import oracle
    from cadise_gb300 import abi
    spec = scenes.roughness_scene()
    sid = gpu_ctx.upload(spec)
    try:
        W = weights(spec, 8)
        spp, seed = 64, 29
        _, gr, _ = gpu_ctx.adjoint_backward(sid, spp, seed, W)
        ggx = [i for i, m in enumerate(spec.materials) if m.type in (scenes.CONDUCTOR, scenes.ROUGH_DIELECTRIC)]
        ref = oracle.PortScene(abi.flatten(spec)).adjoint_fp64(seed, spp, W, [(1, i, 0) for i in ggx],
                                                               scene_index=sid)
        gpu = gr[ggx]
        assert np.all(ref != 0)
        assert np.all(np.abs(gpu - ref) <= 0.01 * np.abs(ref) + 1e-4 * np.abs(ref).max()), np.stack([gpu, ref])
    finally:
        gpu_ctx.release(sid)


@pytest.mark.parametrize("name", ["diff", "features"])
def test_wavefront_and_megakernel_schedules_agree(gpu_ctx, diff, name):
    """The wavefront adjoint (forward pass, then a replay pass by pass) and
    the megakernel adjoint (one thread replays one path twice) run the same
    per-path arithmetic on the same samples: every gradient agrees up to the
    order of the FP64 sums.  The feature scene adds glass, rough dielectric,
    plastic and the environment light (MIS rays that escape)."""
    from cadise_gb300 import CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT
    if name == "diff":
        spec, sid = diff
        release = False
    else:
        spec = scenes.feature_scene()
        sid = gpu_ctx.upload(spec)
        release = True
    try:
        W = weights(spec, 9)
        spp, seed = 32, 41
        gpu_ctx.set_adjoint_mode(CGPU_MODE_MEGAKERNEL)
        mk = gpu_ctx.adjoint_backward(sid, spp, seed, W)
        gpu_ctx.set_adjoint_mode(CGPU_MODE_WAVEFRONT)
        assert sum(np.count_nonzero(g) for g in mk) > 0
        base = gpu_ctx.tuning()
        # per-ray traversal passes, and the persistent while-while passes (traversal 3)
        for traversal in (0, 3):
            gpu_ctx.set_tuning(base["block_trace"], base["block_shade"], base["max_paths"], traversal)
            wf = gpu_ctx.adjoint_backward(sid, spp, seed, W)
            for a, b in zip(wf, mk):
                scale = np.abs(b).max() if b.size else 0.0
                np.testing.assert_allclose(a, b, rtol=1e-7, atol=1e-10 * scale + 1e-30)
        gpu_ctx.set_tuning_dict(base)
    finally:
        gpu_ctx.set_adjoint_mode(CGPU_MODE_WAVEFRONT)
        if release:
            gpu_ctx.release(sid)
