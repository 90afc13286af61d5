"""The multi-GPU path is replicas only: a pixel list is split into contiguous
shards, each rank solves its shard, results are concatenated in order and
timings reduced with max.  Exercised here with world_size 2 on the gloo
backend on CPU, with a host-side stand-in for the per-shard solve."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _fake_solve(cases, opts, aers):
    # per-pixel result depending only on the pixel's own input (like a real solve)
    dt = np.dtype([("rho_I", np.float64), ("idx", np.int32)])
    out = np.zeros(len(cases), dtype=dt)
    out["rho_I"] = [0.01 * c for c in cases]
    out["idx"] = cases
    return out


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from ocrt_gb300.replicas import max_over_ranks, solve_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cases = list(range(11))
        res = solve_sharded(_fake_solve, cases, None, None)
        t = max_over_ranks(1.0 + rank)
        q.put((rank, res["idx"].tolist(), float(res["rho_I"].sum()), t))
    finally:
        dist.destroy_process_group()


def test_shard_bounds_cover_exactly_once():
    from ocrt_gb300.replicas import shard_bounds
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_bounds(n, r, world)
                seen.extend(range(lo, hi))
                assert hi - lo in (n // world, n // world + 1)
            assert seen == list(range(n))


def test_sharded_solve_and_max_timing_world2_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, idx, s, t in out:
        assert idx == list(range(11))          # every pixel once, in order, on every rank
        assert abs(s - 0.01 * sum(range(11))) < 1e-12
        assert t == 2.0                        # max over ranks
