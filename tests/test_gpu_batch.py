"""Batched uneven scenes in one launch sequence, and the autotuner.

Paths are keyed by (seed, scene id, pixel, sample), so a scene rendered in a
batch with others, with any block size or batch capacity, accumulates the
same film bit for bit as when rendered alone."""
import os

import numpy as np
import pytest

import cadise_gb300 as cg
from cadise_gb300 import CGPU_MODE_MEGAKERNEL, CGPU_MODE_WAVEFRONT, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def uneven(gpu_ctx):
    specs = [
        scenes.cornell_box(40, 24, 8, 4),
        scenes.icosphere_field(n_spheres=6, subdivision=2, n_lights=2, seed=31, width=64, height=48, spp=16,
                               max_depth=8, box=30.0, radius_range=(2, 6)),
        scenes.feature_scene(width=24, height=24, spp=4, max_depth=16),
    ]
    sids = [gpu_ctx.upload(s) for s in specs]
    yield specs, sids
    for s in sids:
        gpu_ctx.release(s)


def films(ctx, sids):
    return [ctx.film_read(s) for s in sids]


def test_batch_equals_individual_renders(gpu_ctx, uneven):
    specs, sids = uneven
    for s in sids:
        gpu_ctx.film_clear(s)
    gpu_ctx.render(sids, 0, 8, seed=77, mode=CGPU_MODE_WAVEFRONT)
    together = films(gpu_ctx, sids)
    for s in sids:
        gpu_ctx.film_clear(s)
        gpu_ctx.render([s], 0, 8, seed=77, mode=CGPU_MODE_WAVEFRONT)
    alone = films(gpu_ctx, sids)
    for a, b in zip(together, alone):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    for s in sids:
        gpu_ctx.film_clear(s)
    gpu_ctx.render(sids, 0, 8, seed=77, mode=CGPU_MODE_MEGAKERNEL)
    mk = films(gpu_ctx, sids)
    for a, b in zip(together, mk):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_per_scene_sample_counts(gpu_ctx, uneven):
    """One call, a different sample range per scene (cgpu_render_params.scene_samples)."""
    specs, sids = uneven
    counts = [3, 8, 5]
    for s in sids:
        gpu_ctx.film_clear(s)
    gpu_ctx.render(sids, 2, counts, seed=19, mode=CGPU_MODE_WAVEFRONT)
    together = films(gpu_ctx, sids)
    for s, c in zip(sids, counts):
        gpu_ctx.film_clear(s)
        gpu_ctx.render([s], 2, c, seed=19, mode=CGPU_MODE_WAVEFRONT)
    alone = films(gpu_ctx, sids)
    for a, b, c in zip(together, alone, counts):
        assert a[2].max() == c
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_tuning_does_not_change_results(gpu_ctx, uneven):
    specs, sids = uneven
    base = gpu_ctx.tuning()
    for s in sids:
        gpu_ctx.film_clear(s)
    gpu_ctx.render(sids, 0, 4, seed=5)
    ref = films(gpu_ctx, sids)
    # small batches; persistent ray replacement (1) and persistent while-while (2);
    # closest-hit queues sorted by direction octant and origin (reorder) with traversals 0 and 2;
    # the queue-compaction (refill) thresholds of the persistent passes at their extremes
    for traversal, reorder, rc, ra in ((1, 0, 0, 0), (2, 0, 0, 0), (3, 0, 0, 0), (0, 1, 0, 0), (2, 2, 0, 0),
                                       (3, 3, 0, 0), (3, 4, 0, 0), (3, 0, 1, 32), (3, 0, 32, 1), (2, 0, 20, 0), (3, 0, 6, 24)):
        gpu_ctx.set_tuning(64, 256, 1 << 14, traversal=traversal, reorder=reorder, refill_closest=rc,
                           refill_any=ra)
        for s in sids:
            gpu_ctx.film_clear(s)
        gpu_ctx.render(sids, 0, 4, seed=5)
        got = films(gpu_ctx, sids)
        assert gpu_ctx.stats().batches > 1
        for a, b in zip(ref, got):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
    gpu_ctx.set_tuning_dict(base)


def test_autotune_picks_and_caches(gpu_ctx, uneven, tmp_path):
    specs, sids = uneven
    cache = str(tmp_path / "tune.jsonl")
    t1 = gpu_ctx.autotune(sids, samples=1, cache_path=cache)
    assert t1["block_trace"] in (64, 128, 256) and t1["block_shade"] in (64, 128, 256)
    assert os.path.getsize(cache) > 0
    lines = open(cache).read().strip().splitlines()
    t2 = gpu_ctx.autotune(sids, samples=1, cache_path=cache)
    assert t2 == t1
    assert open(cache).read().strip().splitlines() == lines  # served from the cache
    assert gpu_ctx.tuning() == t1
    with pytest.raises(cg.CgpuError):
        gpu_ctx.set_tuning(100, 128)
    with pytest.raises(cg.CgpuError):
        gpu_ctx.set_tuning(128, 128, refill_closest=33)
