"""Multi-rank partitioning on CPU with gloo (world size 2): bands, shards, film gather, gradient sum."""
import os
import socket

import numpy as np
import pytest


def test_row_band_covers_image():
    from dfpt.parallel import row_band

    for h in (0, 1, 7, 1080):
        for world in (1, 2, 3, 8):
            bands = [row_band(h, world, r) for r in range(world)]
            assert bands[0][0] == 0 and bands[-1][1] == h
            assert all(bands[i][1] == bands[i + 1][0] for i in range(world - 1))
            assert max(b - a for a, b in bands) - min(b - a for a, b in bands) <= 1
    with pytest.raises(ValueError):
        row_band(10, 2, 2)


def test_scene_shard_is_a_partition():
    from dfpt.parallel import scene_shard

    costs = np.random.default_rng(0).uniform(1, 100, 64)
    shards = [scene_shard(costs, 4, r) for r in range(4)]
    assert sorted(i for s in shards for i in s) == list(range(64))
    loads = [costs[s].sum() for s in shards]
    assert max(loads) / min(loads) < 1.1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, queue):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root / "dayflower-path-tracer_gb300"), str(root)]
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from dfpt import synthetic
        from dfpt.kernel import default_params
        from dfpt.parallel import allreduce_sum, gather_film, row_band
        from oracle import oracle

        scene, sky, params, _ = synthetic.sphere_scene(0, 24, 17)
        w, h = 24, 17
        p = default_params()
        for k, v in params.items():
            setattr(p, k, v)
        r0, r1 = row_band(h, world, rank)
        out = oracle.render(scene, sky, p, w, h, passes=2, precision=64, rows=(r0, r1), threads=1)
        band = out["film"].reshape(h, w, 3)[r0:r1]
        full = gather_film(band, h, w)
        g = allreduce_sum(np.full(5, rank + 1.0))
        if rank == 0:
            ref = oracle.render(scene, sky, p, w, h, passes=2, precision=64, threads=1)["film"].reshape(h, w, 3)
            queue.put((np.abs(full - ref.astype(np.float32)).max(), g.tolist()))
    finally:
        dist.destroy_process_group()


def test_gloo_band_render_and_gradient_sum():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    err, g = q.get(timeout=10)
    assert err == 0.0
    assert g == [3.0] * 5
