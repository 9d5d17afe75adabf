"""A single run split across ranks in row slabs (CPU, gloo).

The reference advances every block of a run in one process; its only
parallel decomposition is the block dataflow, in which each block's flux task
joins its 3x3 neighbours' primitives and extends a 2-zone halo
(src/scheme.rs:119-133; periodic neighbours, src/mesh.rs:101-110).  Across
ranks that becomes a split of the block rows into slabs, one per rank:

  * once per advance, the maximum signal speed of each slab, reduced with max
    over the ranks, gives the global dt (scheme.rs:336-340);
  * before every RK stage each rank sends its slab's first and last two zone
    rows (whole rows, so the depth-1 corners come along) and receives its
    neighbours' into its halo rows (periodic: the first slab's upper
    neighbour is the last slab);
  * each rank runs the stage on its own blocks (the oracle's per-slab stage,
    oracle_stage_rows) and the RK average on them;
  * the per-block ledgers are summed over the ranks (each block has one owner).

The test runs this with two and three gloo ranks on the oracle and checks the
gathered state, the ledgers, every dt and the time against a whole-mesh oracle
run of the same steps, bit for bit."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADVANCES = 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case(variant):
    import dataclasses
    import binary2d as b2
    mesh, hydro, physics, model = b2.presets.iso_disk(6, 16, seed=77)
    if variant == "alpha_rk3":
        physics = dataclasses.replace(physics, viscosity=("alpha", 0.1), rk_order="RK3")
    return mesh, hydro, physics, model


def slab_rows(nb, world, rank):
    return rank * nb // world, (rank + 1) * nb // world


def exchange_halo(dist, torch, u, lo, hi, world, rank):
    """Send this slab's first and last two zone rows; receive the neighbours'
    edge rows into the halo rows above and below the slab."""
    nb = u.shape[0]
    edges = torch.from_numpy(np.ascontiguousarray(np.stack([u[lo, :, 0:2], u[hi - 1, :, -2:]])))
    got = [torch.empty_like(edges) for _ in range(world)]
    dist.all_gather(got, edges)
    up, down = (rank - 1) % world, (rank + 1) % world
    u[(lo - 1) % nb, :, -2:] = got[up][1].numpy()      # the upper slab's last two rows
    u[hi % nb, :, 0:2] = got[down][0].numpy()           # the lower slab's first two rows


def _worker(rank, world, port, variant, q):
    for p in (ROOT, os.path.join(ROOT, "app-binary2d_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import binding
    mesh, hydro, physics, model = _case(variant)
    u, cfg = binding.disk_initial_state(mesh, hydro, physics, model)
    nb, nf = mesh.num_blocks, u.shape[-1]
    lo, hi = slab_rows(nb, world, rank)
    bg = u.copy()
    led = np.zeros((nb, nb, 7, nf))
    t = 0.0
    dx = mesh.cell_spacing()
    dts = []
    rk = {"RK1": 1, "RK2": 2, "RK3": 3}[physics.rk_order]
    for _ in range(ADVANCES):
        amax = torch.tensor([binding.max_signal_speed_rows(cfg, u, lo, hi)], dtype=torch.float64)
        dist.all_reduce(amax, op=dist.ReduceOp.MAX)
        dt = physics.cfl * dx / float(amax.item())
        dts.append(dt)
        u0, led0, t0 = u.copy(), led.copy(), t
        # the RK stages (godunov-core's SSP forms, as the oracle runs them):
        # stage k reads the previous stage's output, averaged with u0 at weight bf
        weights = {1: [None], 2: [None, 0.5], 3: [None, 0.75, 1.0 / 3.0]}[rk]
        cur, cur_led, ts = u0, led0, t0
        for bf in weights:
            exchange_halo(dist, torch, cur, lo, hi, world, rank)
            out, out_led = cur.copy(), cur_led.copy()
            if bf is None:
                binding.stage_rows(cfg, cur, out, bg, cur_led, out_led, ts, dt, lo, hi)
            else:
                binding.stage_rows(cfg, cur, out, bg, cur_led, out_led, ts, dt, lo, hi, base=u0, led_base=led0,
                                   bf=bf)
            t_stage = ts + dt
            ts = t_stage if bf is None else t_stage * (-bf + 1.0) + t0 * bf
            cur, cur_led = out, out_led
        u, led, t = cur, cur_led, ts
    mine = np.zeros_like(u)
    mine[lo:hi] = u[lo:hi]
    full = torch.from_numpy(mine)
    dist.all_reduce(full, op=dist.ReduceOp.SUM)
    mled = np.zeros_like(led)
    mled[lo:hi] = led[lo:hi]
    fled = torch.from_numpy(mled)
    dist.all_reduce(fled, op=dist.ReduceOp.SUM)
    if rank == 0:
        q.put((full.numpy(), fled.numpy(), t, dts))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,variant", [(2, "iso"), (3, "iso"), (2, "alpha_rk3")])
def test_row_slabs_match_the_whole_mesh(world, variant):
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "app-binary2d_gb300"))
    from oracle import binding
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, variant, q)) for r in range(world)]
    for p in procs:
        p.start()
    state, ledger, t, dts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    mesh, hydro, physics, model = _case(variant)
    cons, cfg = binding.disk_initial_state(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    ref_dts = [ref.advance(1, nthreads=2) for _ in range(ADVANCES)]
    assert dts == ref_dts
    assert np.array_equal(state, ref.cons)
    assert np.array_equal(ledger, ref.ledger)
    assert t == ref.time.value
