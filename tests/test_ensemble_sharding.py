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


def _store_worker(rank, world, port, result_path, fail_rank, timeout):
    """One rank of a sharded ensemble on a TCPStore; fail_rank claims its
    first member and then raises (a crash between steps: nothing of its is
    left in flight)."""
    import torch.distributed as dist
    from qdng_gb300.sharding import ShardedEnsemble
    from oracle import oracle as O
    O.threads(1)
    store = dist.TCPStore("127.0.0.1", port, world, rank == 0, timeout=__import__("datetime").timedelta(seconds=60))
    ens = cases.cfg4_ensemble(n=7, seed=5, sizes_1d=[256, 384], sides_2d=[32], nt=8)
    costs = [m["grid"].npts for m in ens]
    sh = ShardedEnsemble(store, rank, world, costs, timeout=timeout)

    def work(i):
        if rank == fail_rank:
            raise RuntimeError("rank failed")
        S = O.System(cases.member_hplan(ens[i]))
        P = O.Propagator(S, "Cheby", "", dt=10.0)
        x = ens[i]["psi"].copy()
        for s in range(2):
            P.apply(x, s)
        return x

    ran = sh.run(work)
    store.set(f"ran/{rank}", ",".join(map(str, ran)))
    if rank == 0:
        while not all(store.check([f"ran/{r}"]) for r in range(world) if r != fail_rank):
            __import__("time").sleep(0.05)
        res = sh.gather()
        np.savez(result_path, **{str(k): v for k, v in res.items()})


def test_failed_rank_members_run_by_survivors(tmp_path):
    """Three ranks, rank 2 fails after claiming its first member: ranks 0
    and 1 see its heartbeat stop, claim its members and finish the ensemble;
    every result equals the single-process one."""
    pytest.importorskip("torch")
    import multiprocessing as mpc
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "res.npz")
    ctx = mpc.get_context("spawn")
    procs = [ctx.Process(target=_store_worker, args=(r, 3, port, out, 2, 1.0)) for r in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert procs[0].exitcode == 0 and procs[1].exitcode == 0
    assert procs[2].exitcode != 0
    res = np.load(out)
    from oracle import oracle as O
    ens = cases.cfg4_ensemble(n=7, seed=5, sizes_1d=[256, 384], sides_2d=[32], nt=8)
    assert sorted(int(k) for k in res.files) == list(range(7))
    for i, m in enumerate(ens):
        S = O.System(cases.member_hplan(m))
        P = O.Propagator(S, "Cheby", "", dt=10.0)
        x = m["psi"].copy()
        for s in range(2):
            P.apply(x, s)
        assert np.array_equal(res[str(i)], x)
