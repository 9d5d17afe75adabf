"""FP64 GPU path vs the CPU oracle, through the C ABI.

Tolerance: 1e-12 relative (max-norm per conserved field) after N steps; dt,
time and iteration to 1e-12 / exactly.  The per-block source ledger is
summed in a different order on the GPU and is compared to 1e-12 of each
item's total magnitude.
"""
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from helpers import ledger_err, make_case, rel_err, run_pair
from oracle import binding

pytestmark = pytest.mark.gpu

TOL = 1e-12


def check(r, tol=TOL, led_tol=TOL):
    assert np.all(np.isfinite(r["gpu"]))
    assert rel_err(r["gpu"], r["ref"]) <= tol, rel_err(r["gpu"], r["ref"])
    assert np.allclose(r["dt"], r["dt_ref"], rtol=tol, atol=0)
    assert r["it"] == r["it_ref"]
    assert abs(r["t"] - r["t_ref"]) <= tol * abs(r["t_ref"])
    assert ledger_err(r["led"], r["led_ref"]) <= led_tol


def test_disk_512_100_steps():
    """Plain FP64 isothermal run, 8x8 blocks of 64^2, 100 steps (fold 10)."""
    mesh, hydro, physics, model = b2.presets.disk_512(seed=1)
    r = run_pair(mesh, hydro, physics, model, fold=10, advances=10)
    check(r)


@pytest.mark.parametrize("rk", ["RK1", "RK2", "RK3"])
def test_rk_orders(rk):
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=2)
    physics = dataclasses.replace(physics, rk_order=rk)
    r = run_pair(mesh, hydro, physics, model, fold=4, advances=3)
    check(r)


@pytest.mark.parametrize("variant", ["alpha", "torque_free", "floor_trigger", "one_body", "eccentric", "lambda"])
def test_iso_physics_variants(variant):
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=3)
    if variant == "alpha":
        physics = dataclasses.replace(physics, viscosity=("alpha", 0.1))
    elif variant == "torque_free":
        physics = dataclasses.replace(physics, sink_model="torque_free", sink_radius=0.3)
    elif variant == "floor_trigger":
        hydro = b2.Isothermal(mach_number=10.0, density_floor=1e-3)
        physics = dataclasses.replace(physics, plm_density_trigger=1e-2, fake_mass_threshold=0.5,
                                      fake_mass_rate=1e-3, dt_min=1e-4)
    elif variant == "one_body":
        physics = dataclasses.replace(physics, one_body=True, sink_radius=0.2)
    elif variant == "eccentric":
        physics = dataclasses.replace(physics, binary_eccentricity=0.6, binary_mass_ratio=0.3, sink_radius=0.3)
    elif variant == "lambda":
        physics = dataclasses.replace(physics, lambda_multiplier=0.7)
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=3)
    check(r)


@pytest.mark.parametrize("variant", ["t4", "t4_ceiling_slow", "beta_alpha", "torque_free", "floors"])
def test_euler_variants(variant):
    mesh = b2.Mesh(num_blocks=4, block_size=32, domain_radius=8.0)
    hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
    physics = b2.presets.iso_physics(q=0.5, e=0.3)
    physics = dataclasses.replace(physics, sink_radius=0.3, softening_length=0.2)
    # no cavity: Euler::source_terms converts without floors (physics.rs:696), and
    # T^4 cooling of a near-vacuum cavity reaches pow(negative, -1/3) = NaN in the
    # reference's own arithmetic
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
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=3)
    check(r)


@pytest.mark.parametrize("tile", [(32, 32), (32, 8), (32, 16), (64, 64), (64, 16)])
def test_tile_shapes_bitwise(tile):
    """The decomposition into CTA tiles changes nothing: bitwise equal states."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 64, seed=4)
    base = run_pair(mesh, hydro, physics, model, fold=2, advances=2, tile=(64, 32))
    other = run_pair(mesh, hydro, physics, model, fold=2, advances=2, tile=tile)
    assert np.array_equal(base["gpu"], other["gpu"])
    check(other)


def test_graphs_bitwise():
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=6)
    a = run_pair(mesh, hydro, physics, model, fold=3, advances=3, graphs=True)
    b = run_pair(mesh, hydro, physics, model, fold=3, advances=3, graphs=False)
    assert np.array_equal(a["gpu"], b["gpu"])


def test_tiny_blocks_and_small_tiles():
    """Blocks smaller than a warp (4x4 blocks of 8^2) exercise the periodic
    halo across many block edges."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 8, seed=8)
    physics = dataclasses.replace(physics, buffer_rate=10.0)
    r = run_pair(mesh, hydro, physics, model, fold=5, advances=2)
    check(r)


def test_failure_is_the_reference_error():
    """At dx = 0.5 the explicit buffer (rate 1000) drives a zone negative.
    Both sides reject the step, and the GPU names the zone the reference
    would: first block in index order with a failing 3x3 neighbour, its
    first failing neighbour, that block's first failing zone."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 8, seed=8)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    with b2.Runtime([b2.Run(mesh, hydro, physics)]) as rt:
        rt.upload(0, cons)
        gpu_err = None
        for _ in range(4):
            try:
                rt.advance(5)
            except b2.HydroError as e:
                gpu_err = e
                break
        assert gpu_err is not None
        out, t, it = rt.download(0)
    ref_err = None
    for _ in range(4):
        try:
            ref.advance(5)
        except binding.OracleHydroError as e:
            ref_err = e.err
            break
    assert ref_err is not None
    assert gpu_err.code == ref_err.code
    assert gpu_err.block == (ref_err.block_i, ref_err.block_j)
    assert gpu_err.zone == (ref_err.zone_i, ref_err.zone_j)
    assert gpu_err.position == (ref_err.x, ref_err.y)
    assert abs(gpu_err.value - ref_err.value) <= 1e-12 * abs(ref_err.value)
    assert abs(gpu_err.time - ref_err.time) <= 1e-12 * abs(ref_err.time)
    # the GPU context is left at the state before the failing advance
    assert rel_err(out, ref.cons) <= TOL and it == ref.iteration.value


def test_background_differs_from_state():
    """BlockData::initial_conserved is an independent input (scheme.rs:36-58)."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=9)
    bg, _ = make_case(mesh, hydro, physics, dataclasses.replace(model, seed=99, noise=0.05))
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=2, background=bg)
    check(r)
