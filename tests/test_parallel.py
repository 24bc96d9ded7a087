"""Multi-rank host logic with world_size-2 gloo process groups on CPU: sample passes split across
ranks, one film reduction, same image as a single film over all passes."""
import os
import socket

import numpy as np
import pytest

from milton_gb300.parallel import film_partials, kahan_film, pass_range, reduce_films


def test_pass_ranges_cover_every_pass_once():
    for spp in (1, 7, 16, 64, 255):
        for world in (1, 2, 3, 8):
            got = []
            for r in range(world):
                b, n = pass_range(spp, world, r)
                got.extend(range(b, b + n))
            assert got == list(range(spp))
    with pytest.raises(ValueError):
        pass_range(16, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, paths, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, n = pass_range(paths.shape[2], world, rank)
    raw = kahan_film(paths[:, :, b:b + n])
    mean = reduce_films(raw)
    out_q.put((rank, mean))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_film_reduction_matches_single_film(oracle):
    import multiprocessing as mp
    from milton_gb300 import scenegen
    s = scenegen.plain(0)
    tree = oracle.Tree(s.tri_v)
    _, paths, _ = oracle.render(s, tree, 16, 12, 16, max_depth=5, rr_start=3, seed=7, per_path=True, threads=2)
    single = film_partials(kahan_film(paths))
    want = single[..., :3] / single[..., 3:4]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, paths, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert np.allclose(results[r], want, rtol=1e-6, atol=1e-7)
        assert np.allclose(results[r], paths.mean(axis=2), rtol=1e-5, atol=1e-6)


def test_single_process_reduce_is_the_film_mean():
    rng = np.random.default_rng(0)
    paths = rng.random((4, 5, 9, 3)) * 3
    mean = reduce_films(kahan_film(paths))
    assert np.allclose(mean, paths.mean(axis=2), rtol=1e-6)
