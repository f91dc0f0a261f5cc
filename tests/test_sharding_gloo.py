"""Sharded runs on CPU ranks (gloo): the host logic of the multi-GPU path.

Each rank steps its column range (climaland_gb300.sharding) with the oracle
standing in for its GPU; the state gathered on rank 0 must equal the
unsharded run bit for bit (columns are independent and the rain-pulse hash
uses global column indices), and the all-reduced budget totals must equal
the unsharded totals."""
import multiprocessing
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def _paths():
    for p in (REPO / "climaland.jl_gb300", REPO / "oracle", REPO / "tests"):
        if str(p) not in sys.path:
            sys.path.insert(0, str(p))


def _workload(name):
    _paths()
    from climaland_gb300 import workloads as WL
    if name == "full_scale":  # rain pulses hashed per column
        return WL.full_scale_c4(ncol=96, seed=5)
    if name == "uneven":
        return WL.uneven_c2(ncol=262144, seed=2).subset(120)
    if name == "atmos_topmodel":  # per-column drivers and TOPMODEL rows travel with the shard
        from climaland_gb300 import _abi as A
        return WL.with_atmos(WL.full_scale_c4(ncol=96, seed=5), runoff=A.CLM_RUNOFF_TOPMODEL)
    return WL.richards_c0(ncol=64, seed=1)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, name, nsteps, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    _paths()
    import torch.distributed as dist

    import oracle as O
    from climaland_gb300 import sharding as S

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = _workload(name)
        part = S.shard(w, rank, world)
        o = O.Oracle(part, nthreads=1)
        st = part.copy_state()
        rc, _, _ = o.step(st, part.t0, part.dt, nsteps)
        W, E = o.budgets(st)
        totals = S.reduce_totals([float(W.sum()), float(E.sum())])
        got = S.gather_state(w, st, rank, world)
        if rank == 0:
            q.put((rc, got, totals))
    finally:
        dist.destroy_process_group()


def _run_sharded(name, world, nsteps):
    ctx = multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, name, nsteps, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def test_partition_is_contiguous_and_balanced():
    _paths()
    from climaland_gb300 import sharding as S
    w = _workload("uneven")
    for world in (1, 2, 3, 5):
        ranges = S.partition(w.nlayers, world)
        assert ranges[0][0] == 0 and ranges[-1][1] == w.ncol
        assert all(a < b for a, b in ranges)
        assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
        cells = [int(w.offsets[b] - w.offsets[a]) for a, b in ranges]
        assert max(cells) - min(cells) <= 2 * int(w.nlayers.max())
    with pytest.raises(ValueError):
        S.partition(np.ones(3), 4)


@pytest.mark.parametrize("name,world", [("full_scale", 2), ("uneven", 3), ("richards", 2),
                                        ("atmos_topmodel", 2)])
def test_sharded_run_equals_unsharded(name, world):
    _paths()
    import oracle as O
    nsteps = 12
    rc, got, totals = _run_sharded(name, world, nsteps)
    assert rc == 0
    w = _workload(name)
    ref = w.copy_state()
    O.Oracle(w, nthreads=1).step(ref, w.t0, w.dt, nsteps)
    for a, b in zip(ref, got):
        if a is None:
            assert b is None
        else:
            assert np.array_equal(a, b)
    W, E = O.Oracle(w).budgets(ref)
    assert np.isclose(totals[0], W.sum(), rtol=1e-14, atol=0.0)
    assert np.isclose(totals[1], E.sum(), rtol=1e-14, atol=1e-300)
