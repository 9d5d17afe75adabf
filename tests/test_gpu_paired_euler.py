"""The paired-column Euler kernel (compensated FP32 state, tiles 64, 128, 256
or 512 wide) against the CPU oracle: the Euler physics variants of the FP64
parity tests, every tile width, row chunks across block rows and tiles across
block columns, and batched runs; and the tiling independence of its states."""
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from helpers import ledger_err, make_case, rel_err, run_pair
from oracle import binding

pytestmark = pytest.mark.gpu

BUFFER = 4
TOL, L1_TOL, LED_TOL = 2e-4, 1e-5, 1e-4


def euler_case(nb=4, bs=64, variant="t4"):
    """An Euler disk without a cavity (T^4 cooling of a near-vacuum cavity
    reaches pow(negative, -1/3) in the reference's own arithmetic)."""
    mesh = b2.Mesh(num_blocks=nb, block_size=bs, domain_radius=8.0)
    hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
    physics = b2.presets.iso_physics(q=0.5, e=0.3)
    physics = dataclasses.replace(physics, sink_radius=0.3, softening_length=0.2)
    model = b2.DiskModel(surface_density=1.0, mach_number=5.0, noise=1e-3, seed=5, cavity_radius=0.0)
    if variant == "t4_ceiling_slow":
        hydro = dataclasses.replace(hydro, cooling_slow_start=True, density_index=1)
        physics = dataclasses.replace(physics, mach_ceiling=12.0)
    elif variant == "beta_alpha":
        hydro = dataclasses.replace(hydro, cooling_beta=10.0)
        physics = dataclasses.replace(physics, viscosity=("alpha", 0.1))
    elif variant == "torque_free":
        physics = dataclasses.replace(physics, sink_model="torque_free")
        hydro = dataclasses.replace(hydro, pressure_floor=1e-8)
    elif variant == "floors":
        hydro = dataclasses.replace(hydro, density_floor=1e-3, pressure_floor=1e-8)
    elif variant == "lambda_rk3":
        physics = dataclasses.replace(physics, lambda_multiplier=0.7, rk_order="RK3")
    elif variant == "eccentric":
        physics = dataclasses.replace(physics, binary_eccentricity=0.6, binary_mass_ratio=0.3)
    return mesh, hydro, physics, model


def item_errors(led, ref):
    """Per ledger item, the largest |GPU - oracle| over blocks and fields
    against the item's largest |oracle|.  Items the oracle leaves at zero up
    to rounding are judged against the largest item: the FP32 cooling item's
    mass and momentum are zero, and the oracle's cooling item (uc - u of a
    prim -> cons round trip) is rounding alone where no cooling acts, e.g.
    under the T^4 law's slow start (exp(-2 pi / t) = 0 at t << 1)."""
    scale = np.abs(ref).max(axis=(0, 1, 3))
    diff = np.abs(led - ref).max(axis=(0, 1, 3))
    big = scale.max()
    rounding = scale <= 1e-12 * big
    err = np.where(rounding, 0.0, diff / np.maximum(scale, 1e-300))
    zero = float((diff[rounding] / big).max()) if rounding.any() else 0.0
    return err, zero


def check(r):
    assert np.all(np.isfinite(r["gpu"]))
    assert rel_err(r["gpu"], r["ref"]) <= TOL
    l1 = np.abs(r["gpu"][..., 0] - r["ref"][..., 0]).sum() / np.abs(r["ref"][..., 0]).sum()
    assert l1 <= L1_TOL, l1
    err, zero = item_errors(r["led"], r["led_ref"])
    # the buffer item is formed from the FP32 high words of u and u_bg (see
    # test_gpu_paired.py); the other items are held to the FP32 tolerance
    assert all(err[k] <= LED_TOL for k in range(7) if k != BUFFER), err
    assert err[BUFFER] <= 5e-3, err
    assert zero <= 1e-6, zero
    assert abs(r["t"] - r["t_ref"]) <= 1e-5 * abs(r["t_ref"])
    assert r["it"] == r["it_ref"]


@pytest.mark.parametrize("variant", ["t4", "t4_ceiling_slow", "beta_alpha", "torque_free", "floors", "lambda_rk3",
                                     "eccentric"])
def test_euler_paired_physics_variants(variant):
    mesh, hydro, physics, model = euler_case(variant=variant)
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=3, precision="fp32_comp", tile=(64, 32))
    check(r)


@pytest.mark.parametrize("nb,bs,tw,rows", [
    (2, 128, 128, 0),      # block-aligned 128 x 32
    (2, 128, 128, 100),    # 3 chunks of 85-86 rows, the middle one across row 128
    (2, 128, 256, 100),    # 256-column tiles over both block columns
    (4, 64, 128, 50),      # 128-column tiles over two 64-column blocks, 6 chunks
    (4, 128, 512, 100),    # 512-column tiles over four block columns
])
def test_euler_paired_tiles_and_chunks(nb, bs, tw, rows):
    mesh, hydro, physics, model = euler_case(nb, bs, variant="beta_alpha")
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=3, precision="fp32_comp", tile=(tw, 32),
                 strip_rows=rows)
    check(r)


TILINGS = [
    (64, "beta_alpha", [(64, 32, 0), (64, 16, 30), (128, 32, 50), (256, 32, 0), (256, 32, 40)]),
    (64, "torque_free", [(64, 32, 0), (128, 32, 50), (256, 32, 40)]),
    (128, "beta_alpha", [(128, 32, 0), (256, 32, 60), (512, 32, 0), (512, 32, 100)]),
]


@pytest.mark.parametrize("bs,variant,tilings", TILINGS)
def test_euler_paired_tilings_match(bs, variant, tilings):
    """Block-aligned tiles, row chunks and tiles over several block columns
    (the kernel's 128-, 256- and 512-column instantiations) give the same
    state bit for bit; ledgers and orbital elements to FP32 summation order."""
    mesh, hydro, physics, model = euler_case(4, bs, variant=variant)
    cons = make_case(mesh, hydro, physics, model)[0]
    out = []
    for tw, th, rows in tilings:
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp32_comp") as rt:
            rt.set_tile(tw, th)
            rt.set_strip_rows(rows)
            assert rt.tile() == (tw, th) and rt.strip_rows() == rows
            rt.upload(0, cons)
            dts = [rt.advance(3)[0] for _ in range(3)]
            s, t, it = rt.download(0)
            out.append((s, t, dts, rt.ledger(0), rt.elements(0)))
    s0, t0, dts0, led0, el0 = out[0]
    for s, t, dts, led, el in out[1:]:
        assert np.array_equal(s, s0)
        assert t == t0 and dts == dts0
        assert ledger_err(led, led0) <= 1e-5
        escale = np.maximum(np.abs(el0).max(axis=(0, 1)), 1e-300)
        assert (np.abs(el - el0).max(axis=(0, 1)) / escale).max() <= 1e-5


def test_euler_paired_batched_runs():
    """Euler runs of different sizes and physics in one launch (parameters
    from shared memory) against the oracle."""
    cases = [euler_case(2, 64, "t4"), euler_case(3, 64, "beta_alpha")]
    runs = [b2.Run(m, h, p) for m, h, p, _ in cases]
    cons = [make_case(m, h, p, md)[0] for m, h, p, md in cases]
    with b2.Runtime(runs, precision="fp32_comp") as rt:
        rt.set_tile(64, 32)
        rt.set_strip_rows(50)
        for k, c in enumerate(cons):
            rt.upload(k, c)
        for _ in range(3):
            rt.advance(3)
        batched = [rt.download(k)[0] for k in range(len(runs))]
    for k, (m, h, p, md) in enumerate(cases):
        ref = binding.OracleState(b2.to_c(m, h, p), cons[k])
        for _ in range(3):
            ref.advance(3)
        assert rel_err(batched[k], ref.cons) <= TOL


def test_euler_preset_block_on_the_paired_kernel():
    """The 4096^2 preset's physics (beta-cooling, alpha viscosity, the
    cavity, sinks, the buffer) on 4 x 4 blocks of 128^2 with the bench's tile
    shape family (512-column tiles, row chunks): the oracle within FP32
    tolerance after 20 RK2 steps."""
    mesh, hydro, physics, model = b2.presets.euler_beta_disk(4, 128)
    r = run_pair(mesh, hydro, physics, model, fold=10, advances=2, precision="fp32_comp", tile=(512, 32),
                 strip_rows=100)
    check(r)


@pytest.mark.parametrize("kind", ["NegativePressure", "NegativeDensity"])
def test_euler_paired_failure_reports_the_zone(kind):
    """Euler::try_to_primitive's errors (physics.rs:631-660) from the paired
    kernel: the advance fails with the zone and the kind, and the context
    keeps the pre-advance state (main.rs:159-205)."""
    mesh, hydro, physics, model = euler_case(4, 64, variant="t4")
    cons, cfg = make_case(mesh, hydro, physics, model)
    bad = cons.copy()
    z = bad[2, 3, 17, 40]
    if kind == "NegativePressure":
        z[3] = 0.5 * (z[1] ** 2 + z[2] ** 2) / z[0] - 1.0     # E below the kinetic energy
    else:
        z[0] = -1e-3
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp32_comp") as rt:
        rt.set_tile(128, 32)
        rt.set_strip_rows(50)
        rt.upload(0, bad, background=cons, time=0.5, iteration=3)
        with pytest.raises(b2.HydroError) as ei:
            rt.advance(2)
        e = ei.value
        assert e.kind == kind
        assert e.block == (2, 3) and e.zone == (17, 40)
        out, t, it = rt.download(0)
        assert np.allclose(out, bad, rtol=1e-14, atol=0) and t == 0.5 and it == 3
        ref = binding.OracleState(cfg, bad, background=cons)
        with pytest.raises(binding.OracleHydroError):
            ref.advance(2)
