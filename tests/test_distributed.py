"""Multi-process host logic of multi-GPU rendering, on CPU with gloo ranks.

The renderer itself needs a GPU; here each rank renders its share of the
samples with the oracle (a stand-in with the same sample keying) and the
films are merged with the same all-reduce the GPU path uses."""
import os
import socket

import numpy as np
import pytest

from cadise_gb300 import distributed


def test_sample_ranges_partition_the_frame():
    for spp in (1, 7, 64, 1024):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                first, count = distributed.sample_range(spp, r, world)
                seen.extend(range(first, first + count))
            assert seen == list(range(spp))
    with pytest.raises(ValueError):
        distributed.sample_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    import oracle
    from cadise_gb300 import abi, scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = scenes.cornell_box(16, 12, 8, 4)
    first, count = distributed.sample_range(spec.spp, rank, world)
    film, _ = oracle.PortScene(abi.flatten(spec)).render(seed=3, first=first, count=count, threads=2)
    s, q, n = film[..., :3].copy(), film[..., 3:6].copy(), film[..., 6].copy()
    distributed.merge_films(s, q, n)
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), np.concatenate([s.ravel(), q.ravel(), n.ravel()]))
    dist.destroy_process_group()


def test_two_gloo_ranks_merge_to_the_single_process_film(tmp_path):
    import multiprocessing as mp

    import oracle
    from cadise_gb300 import abi, scenes
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    a = np.load(tmp_path / "rank0.npy")
    b = np.load(tmp_path / "rank1.npy")
    assert np.array_equal(a, b)  # every rank holds the merged film
    spec = scenes.cornell_box(16, 12, 8, 4)
    film, _ = oracle.PortScene(abi.flatten(spec)).render(seed=3, first=0, count=spec.spp, threads=2)
    ref = np.concatenate([film[..., :3].ravel(), film[..., 3:6].ravel(), film[..., 6].ravel()])
    np.testing.assert_allclose(a, ref, rtol=1e-12, atol=1e-12)
