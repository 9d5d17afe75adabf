"""One run split into row slabs across contexts on one GPU, against the
unsplit run with the same block-aligned tiles: bit-identical states,
per-block ledgers and orbital-element changes, and the same dt every advance,
on the FP64 kernel and on the FP32 kernels (compensated and FP64 state).

Each context owns a slab of block rows (b2d_set_slab).  Per advance: the
slabs' maximum signal speeds are reduced with max and passed to
b2d_slab_begin; before every RK stage each slab sends its first and last two
zone rows to its neighbours, which write them into the two rows above and
below their own slab (periodically, src/mesh.rs:101-110); then every context
runs the stage on its blocks.  The exchange here goes through host memory, as
it would between processes; the split run equals the whole one because the
reference's block dataflow reads a block's 3x3 neighbours only through a
2-zone halo (src/scheme.rs:119-133)."""
import numpy as np
import pytest

import binary2d as b2
from helpers import make_case

pytestmark = pytest.mark.gpu


def slabs_of(nb, k):
    return [(r * nb // k, (r + 1) * nb // k) for r in range(k)]


def split_run(mesh, hydro, physics, cons, nslab, fold, advances, tile, precision="fp64"):
    bs, N = mesh.block_size, mesh.zones_per_side()
    parts = slabs_of(mesh.num_blocks, nslab)
    rts = []
    for lo, hi in parts:
        rt = b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision)
        rt.set_tile(*tile)
        rt.upload(0, cons)
        rt.set_slab(0, lo, hi)
        rts.append(rt)
    dts = []
    for _ in range(advances):
        amax = max(rt.max_signal_speed(0) for rt in rts)
        for rt in rts:
            rt.slab_begin(fold, [amax])
        rk = {"RK1": 1, "RK2": 2, "RK3": 3}[physics.rk_order]
        for _ in range(fold * rk):
            edges = [(rt.slab_rows(0, lo * bs, 2), rt.slab_rows(0, hi * bs - 2, 2)) for rt, (lo, hi) in zip(rts, parts)]
            for k, (rt, (lo, hi)) in enumerate(zip(rts, parts)):
                up, down = (k - 1) % nslab, (k + 1) % nslab
                rt.put_slab_rows(0, lo * bs - 2, edges[up][1])     # the upper slab's last two rows
                rt.put_slab_rows(0, hi * bs, edges[down][0])       # the lower slab's first two rows
            for rt in rts:
                rt.slab_stage()
        d = [rt.slab_end()[0] for rt in rts]
        assert len(set(d)) == 1
        dts.append(d[0])
    state = np.empty_like(cons)
    led = np.empty((mesh.num_blocks, mesh.num_blocks, 7, cons.shape[-1]))
    el = np.empty((mesh.num_blocks, mesh.num_blocks, 7, 4))
    t_end = []
    for rt, (lo, hi) in zip(rts, parts):
        s, t, it = rt.download(0)
        state[lo:hi] = s[lo:hi]
        led[lo:hi] = rt.ledger(0)[lo:hi]
        el[lo:hi] = rt.elements(0)[lo:hi]
        t_end.append((t, it))
        rt.close()
    assert len(set(t_end)) == 1
    return state, led, el, dts, t_end[0]


@pytest.mark.parametrize("nb,bs,nslab,tile,variant,precision", [
    (4, 32, 2, (32, 16), "iso", "fp64"),
    (6, 32, 3, (32, 32), "iso", "fp64"),
    (4, 64, 2, (64, 32), "alpha_rk3", "fp64"),
    (4, 32, 2, (32, 16), "euler", "fp64"),
    # the FP32 kernels on slabs: paired isothermal (64- and 512-column tiles),
    # paired Euler, the one-column kernel on compensated and on FP64 state
    (4, 64, 2, (64, 32), "iso", "fp32_comp"),
    (4, 128, 2, (512, 32), "iso", "fp32_comp"),
    (6, 64, 3, (128, 16), "alpha_rk3", "fp32_comp"),
    (4, 64, 2, (64, 32), "euler", "fp32_comp"),
    (4, 128, 2, (512, 64), "euler", "fp32_comp"),
    (4, 32, 2, (32, 16), "iso", "fp32_comp"),
    (4, 64, 2, (64, 32), "euler", "fp32_state64"),
])
def test_slabs_match_the_whole_run(nb, bs, nslab, tile, variant, precision):
    import dataclasses
    mesh, hydro, physics, model = b2.presets.iso_disk(nb, bs, seed=96)
    if variant == "alpha_rk3":
        physics = dataclasses.replace(physics, viscosity=("alpha", 0.1), rk_order="RK3")
    elif variant == "euler":
        hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
        physics = dataclasses.replace(b2.presets.iso_physics(q=0.5, e=0.3), sink_radius=0.3, softening_length=0.2)
        model = b2.DiskModel(surface_density=1.0, mach_number=5.0, noise=1e-3, seed=5)
    cons = make_case(mesh, hydro, physics, model)[0]
    fold, advances = 2, 3
    state, led, el, dts, (t, it) = split_run(mesh, hydro, physics, cons, nslab, fold, advances, tile, precision)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
        rt.set_tile(*tile)
        rt.upload(0, cons)
        ref_dts = [rt.advance(fold)[0] for _ in range(advances)]
        ref, t_ref, it_ref = rt.download(0)
        ref_led, ref_el = rt.ledger(0), rt.elements(0)
    assert dts == ref_dts
    assert np.array_equal(state, ref)
    assert np.array_equal(led, ref_led)
    assert np.array_equal(el, ref_el)
    assert t == t_ref and it == it_ref


def test_slab_arguments():
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=97)
    cons = make_case(mesh, hydro, physics, model)[0]
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        for lo, hi in ((-1, 2), (2, 2), (3, 5)):
            with pytest.raises(b2.B2DException):
                rt.set_slab(0, lo, hi)
        with pytest.raises(b2.B2DException):
            rt.slab_stage()                 # no advance begun
        rt.set_slab(0, 0, 2)
        whole_max = None
        rt.set_slab(0, 0, 0)
        whole_max = rt.max_signal_speed(0)
        rt.set_slab(0, 1, 3)
        assert rt.max_signal_speed(0) <= whole_max
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp32_comp") as rt:
        rt.upload(0, cons)
        rt.set_slab(0, 0, 2)             # every precision takes slabs
        got = rt.slab_rows(0, 62, 4)     # the compensated state's hi and lo words
        assert got.dtype == np.float32 and got.shape == (3, 2, 4, 128)
        rt.put_slab_rows(0, 62, got)
