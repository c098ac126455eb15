"""cgpu_render_noalloc (every device buffer of the call in the library's
static scratch) against cgpu_render, through the C ABI.

Collected last on purpose: it must pass alone and after every other GPU test
has used the context.  Same paths (keyed by seed, scene, pixel, sample) and
the same kernels, so the films agree; they may differ in the last FP64 bits
because the two entry points split the samples into batches differently:
rtol 1e-12 on the sums (and on a filtered film's sums of weights)."""
import numpy as np
import pytest

from cadise_gb300 import CgpuError, scenes

pytestmark = pytest.mark.gpu


def films_close(a, b):
    (s1, q1, n1), (s2, q2, n2) = a, b
    # sample counts exactly; a filtered film's sums of weights to FP64 order
    np.testing.assert_allclose(n1, n2, rtol=1e-12, atol=0)
    np.testing.assert_allclose(s1, s2, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(q1, q2, rtol=1e-12, atol=1e-300)


def filtered_spheres():
    s = scenes.sphere_box(64, 48, 16, 8)
    s.film_filter = scenes.FilmFilter("gaussian")
    return s


@pytest.mark.parametrize("traversal", [0, 1, 2, 3])
@pytest.mark.parametrize("make", [
    lambda: scenes.cornell_box(96, 64, 16, 6),
    lambda: scenes.feature_scene(width=48, height=40, spp=16, max_depth=16),
    # analytic spheres (the kernels with the sphere test) and a Gaussian film filter (the gathering splat)
    filtered_spheres,
], ids=["cornell", "features", "spheres_gaussian"])
def test_noalloc_render_matches_render_on_two_calls(gpu_ctx, make, traversal):
    """Each traversal variant of the tuning: the no-alloc call launches its
    own serial list of the same kernels."""
    spec = make()
    sid = gpu_ctx.upload(spec)
    base = gpu_ctx.tuning()
    gpu_ctx.set_tuning(base["block_trace"], base["block_shade"], base["max_paths"], traversal=traversal)
    try:
        npix = spec.width * spec.height
        per = (1 << 18) // npix  # samples per batch of the 262144-path scratch
        # two calls in a row into one film, the first one in several batches
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 0, 300, seed=7)
        gpu_ctx.render([sid], 300, 60, seed=7)
        ref = gpu_ctx.film_read(sid)
        gpu_ctx.film_clear(sid)
        gpu_ctx.render_noalloc(sid, 0, 300, seed=7)
        assert gpu_ctx.stats().batches == -(-300 // per) > 1
        gpu_ctx.render_noalloc(sid, 300, 60, seed=7)
        got = gpu_ctx.film_read(sid)
        if spec.film_filter is None:
            assert got[2].max() == 360  # sample counts (a filtered film holds sums of weights)
        films_close(got, ref)
        # and once more on its own: nothing carried over from the previous call
        gpu_ctx.film_clear(sid)
        gpu_ctx.render_noalloc(sid, 300, 60, seed=7)
        alone = gpu_ctx.film_read(sid)
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 300, 60, seed=7)
        films_close(alone, gpu_ctx.film_read(sid))
    finally:
        gpu_ctx.set_tuning_dict(base)
        gpu_ctx.release(sid)


def test_noalloc_render_rejects_frames_beyond_the_scratch(gpu_ctx):
    big = scenes.cornell_box(640, 480, 1, 4)  # 307200 pixels > 262144
    sid = gpu_ctx.upload(big)
    try:
        with pytest.raises(CgpuError) as e:
            gpu_ctx.render_noalloc(sid, 0, 1, seed=1)
        assert e.value.status == 1  # CGPU_ERR_INVALID_ARGUMENT
        assert "262144" in str(e.value)
    finally:
        gpu_ctx.release(sid)
