"""Ensemble sharding across processes (one GPU each in production): members
are split by largest-processing-time-first, each rank propagates its own
members with no data-path collective, and the host gathers the results.
Checked here with two gloo ranks on the CPU, the oracle standing in for the
per-rank engine."""
import os

import numpy as np
import pytest

from tests import cases


def test_lpt_partition_balances_and_covers():
    costs = [10, 9, 8, 7, 6, 5, 4, 3, 2, 1]
    parts, loads = cases.lpt_partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(10))
    assert max(loads) - min(loads) <= max(costs)


def _worker(rank, world, port, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    O.threads(1)
    ens = cases.cfg4_ensemble(n=6, seed=3, sizes_1d=[256, 384], sides_2d=[32], nt=8)
    costs = [m["grid"].npts for m in ens]
    parts, _ = cases.lpt_partition(costs, world)
    mine = {}
    for i in parts[rank]:
        S = O.System(cases.member_hplan(ens[i]))
        P = O.Propagator(S, "Cheby", "", dt=10.0)
        x = ens[i]["psi"].copy()
        for s in range(2):
            P.apply(x, s)
        mine[i] = x
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)   # host-side gather of finished members
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        np.savez(result_path, **{str(k): v for k, v in merged.items()})
    dist.destroy_process_group()


def test_two_rank_sharding_matches_single_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "res.npz")
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    res = np.load(out)
    from oracle import oracle as O
    ens = cases.cfg4_ensemble(n=6, seed=3, sizes_1d=[256, 384], sides_2d=[32], nt=8)
    assert sorted(int(k) for k in res.files) == list(range(6))
    for i, m in enumerate(ens):
        S = O.System(cases.member_hplan(m))
        P = O.Propagator(S, "Cheby", "", dt=10.0)
        x = m["psi"].copy()
        for s in range(2):
            P.apply(x, s)
        assert np.array_equal(res[str(i)], x)
