"""Multi-rank host logic on CPU (gloo, world size 2): runs of a sweep are
dealt whole to ranks, each rank advances its share (here with the oracle, no
GPU), and the timing / zone counts are reduced over ranks."""
import os
import socket
import sys

import numpy as np
import pytest

from binary2d.distributed import deal_runs


def test_deal_runs_partition_and_balance():
    zones = [256 ** 2, 512 ** 2, 768 ** 2, 1024 ** 2, 512 ** 2, 256 ** 2, 768 ** 2]
    for ws in (1, 2, 3, 4):
        parts = [deal_runs(zones, ws, r) for r in range(ws)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(zones)))
        loads = [sum(zones[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(zones)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "app-binary2d_gb300"), os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import binary2d as b2
    from binary2d.distributed import deal_runs, max_over_ranks, sum_over_ranks
    from helpers import make_case
    from oracle import binding
    cases = [b2.presets.iso_disk(nb, 16, seed=50 + k) for k, nb in enumerate([2, 4, 3, 2, 4])]
    mine = deal_runs([c[0].total_zones() for c in cases], world, rank)
    out = {}
    done = 0
    for k in mine:
        mesh, hydro, physics, model = cases[k]
        cons, cfg = make_case(mesh, hydro, physics, model, run=k)
        st = binding.OracleState(cfg, cons)
        st.advance(2, nthreads=1)
        out[k] = st.cons[..., 0].sum()
        done += mesh.total_zones() * 2
    total = sum_over_ranks(done)
    slowest = max_over_ranks(float(rank + 1))
    q.put((rank, out, total, slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_share_a_sweep():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    merged = {}
    for rank, out, total, slowest in res:
        assert slowest == 2.0
        assert set(out).isdisjoint(merged)
        merged.update(out)
    assert sorted(merged) == list(range(5))
    import binary2d as b2
    expect = sum(c[0].total_zones() * 2 for c in [b2.presets.iso_disk(nb, 16) for nb in [2, 4, 3, 2, 4]])
    assert res[0][2] == expect
    # the ranks' results equal a single-process run of the same cases
    from helpers import make_case
    from oracle import binding
    for k, nb in enumerate([2, 4, 3, 2, 4]):
        mesh, hydro, physics, model = b2.presets.iso_disk(nb, 16, seed=50 + k)
        cons, cfg = make_case(mesh, hydro, physics, model, run=k)
        st = binding.OracleState(cfg, cons)
        st.advance(2, nthreads=3)
        assert st.cons[..., 0].sum() == merged[k]
