"""The device-side iteration budget of the traversals (cgpu_set_visit_budget)
on the GPU: a budget that runs out is a status, not a hang.  With 2 node and
leaf visits per ray every traversal stops early; the rays are counted on the
device and the next synchronising call returns CGPU_ERR_TIMEOUT (status 4).
The wait is bounded by construction (a visit counter per ray), so nothing
here can keep a kernel running; after the error the context renders exactly
as before."""
import numpy as np
import pytest

from cadise_gb300 import CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT, CgpuError, scenes
from golden_scenes import vectors

pytestmark = pytest.mark.gpu

TIMEOUT = 4  # CGPU_ERR_TIMEOUT


@pytest.fixture(scope="module")
def field(gpu_ctx):
    spec = scenes.icosphere_field(n_spheres=10, subdivision=2, n_lights=3, seed=3, width=48, height=36, spp=16,
                                  max_depth=8, dielectric=scenes.GLASS, box=30.0, radius_range=(2.0, 6.0))
    sid = gpu_ctx.upload(spec)
    yield spec, sid
    gpu_ctx.set_visit_budget(0)
    gpu_ctx.release(sid)


def render(ctx, sid, mode):
    ctx.film_clear(sid)
    ctx.render([sid], 0, 2, seed=9, mode=mode)
    return ctx.film_read(sid)


@pytest.mark.parametrize("traversal", [0, 1, 2, 3])
def test_render_reports_an_exhausted_budget(gpu_ctx, field, traversal):
    spec, sid = field
    base = gpu_ctx.tuning()
    try:
        gpu_ctx.set_tuning(base["block_trace"], base["block_shade"], 1 << 16, traversal=traversal)
        ref = render(gpu_ctx, sid, CGPU_MODE_WAVEFRONT)
        gpu_ctx.set_visit_budget(2)
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 0, 2, seed=9, mode=CGPU_MODE_WAVEFRONT, sync=False)  # asynchronous: no status yet
        with pytest.raises(CgpuError) as e:
            gpu_ctx.film_read(sid)
        assert e.value.status == TIMEOUT
        assert "budget" in str(e.value)
        gpu_ctx.synchronize()  # the count was reset by the report
        gpu_ctx.set_visit_budget(0)
        again = render(gpu_ctx, sid, CGPU_MODE_WAVEFRONT)
        for x, y in zip(ref, again):
            assert np.array_equal(x, y)
    finally:
        gpu_ctx.set_visit_budget(0)
        gpu_ctx.set_tuning_dict(base)


def test_megakernel_and_queries_report_an_exhausted_budget(gpu_ctx, field):
    spec, sid = field
    rays = vectors("field")["trace_rays"]
    ref_prim = gpu_ctx.trace_closest(sid, rays)[0]
    gpu_ctx.set_visit_budget(2)
    try:
        gpu_ctx.film_clear(sid)
        gpu_ctx.render([sid], 0, 1, seed=9, mode=CGPU_MODE_MEGAKERNEL, sync=False)
        with pytest.raises(CgpuError) as e:
            gpu_ctx.synchronize()
        assert e.value.status == TIMEOUT
        with pytest.raises(CgpuError) as e:
            gpu_ctx.trace_closest(sid, rays)
        assert e.value.status == TIMEOUT
        with pytest.raises(CgpuError) as e:
            gpu_ctx.trace_any(sid, rays)
        assert e.value.status == TIMEOUT
    finally:
        gpu_ctx.set_visit_budget(0)
    gpu_ctx.synchronize()
    assert np.array_equal(gpu_ctx.trace_closest(sid, rays)[0], ref_prim)


def test_automatic_budget_is_never_reached(gpu_ctx, field):
    """The automatic budget bounds a correct traversal: the golden scene's
    renders and queries under it report nothing."""
    spec, sid = field
    gpu_ctx.set_visit_budget(0)
    render(gpu_ctx, sid, CGPU_MODE_WAVEFRONT)
    render(gpu_ctx, sid, CGPU_MODE_MEGAKERNEL)
    gpu_ctx.trace_closest(sid, vectors("field")["trace_rays"])
    gpu_ctx.synchronize()
