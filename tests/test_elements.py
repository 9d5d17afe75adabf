"""Orbital-element change ledger (BlockState::orbital_elements_change,
src/state.rs:44-49; ItemizedChange::perturbation, state.rs:258-281;
scheme.rs:307-314): GPU against the oracle, and the unbound-orbit error."""
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from binary2d import presets
from oracle import binding

from helpers import make_case


def _dense_case(sigma, rk="RK2"):
    """A small mesh around the binary with no cavity: the sinks and the
    gas's gravity act on every step."""
    mesh, hydro, physics, model = presets.iso_disk(4, 32, domain_radius=2.0, q=0.5, e=0.3)
    physics = dataclasses.replace(physics, rk_order=rk)
    model = dataclasses.replace(model, surface_density=sigma, cavity_radius=0.0)
    return mesh, hydro, physics, model


def _element_err(el, el_ref):
    """The per-item change is a difference of two elements near (1, 1, q, e):
    its rounding is absolute, about one ulp of the element per stage."""
    scale = np.abs(el_ref).max(axis=(0, 1))
    return np.abs(el - el_ref).max(axis=(0, 1)), scale


def test_oracle_elements_cpu():
    """The oracle's element ledger: gas items only, zero where nothing is
    accreted or pulled, averaged like the state."""
    mesh, hydro, physics, model = _dense_case(1.0)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    ref.advance(2, nthreads=4)
    e = ref.elements
    assert np.all(e[:, :, 4:] == 0.0)            # buffer, cooling, fake mass
    assert np.abs(e[:, :, :4]).max() > 1e-6
    assert np.isfinite(e).all()
    # gravity moves the bodies but adds no mass: M is unchanged by grav1/grav2
    assert np.abs(e[:, :, 2:4, 1]).max() == 0.0


def test_oracle_unbound_is_an_error_cpu():
    mesh, hydro, physics, model = _dense_case(1e4)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    with pytest.raises(binding.OracleHydroError) as ei:
        ref.advance(1, nthreads=4)
    assert ei.value.err.code == 3
    assert (ei.value.err.x, ei.value.err.y) == (0.0, 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("rk", ["RK1", "RK2", "RK3"])
def test_elements_match_oracle(rk):
    mesh, hydro, physics, model = _dense_case(1.0, rk)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        for _ in range(3):
            rt.advance(2)
            ref.advance(2)
        el = rt.elements(0)
        out, _, _ = rt.download(0)
    assert np.abs(out - ref.cons).max() <= 1e-12 * np.abs(ref.cons).max()
    diff, scale = _element_err(el, ref.elements)
    # 3 advances x 2 steps x up to 3 stages, each adding an absolute rounding
    # of a few ulp of O(1) elements; relative part from the reordered sums
    assert np.all(diff <= 1e-12 * scale + 1e-13), (diff, scale)
    assert np.all(el[:, :, 4:] == 0.0)


@pytest.mark.gpu
def test_elements_fp32_paths():
    mesh, hydro, physics, model = _dense_case(1.0)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    ref.advance(4)
    for precision in ("fp32_state64", "fp32_comp"):
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
            rt.upload(0, cons)
            rt.advance(4)
            el = rt.elements(0)
        tot, tot_ref = el.sum(axis=(0, 1)), ref.elements.sum(axis=(0, 1))
        assert np.abs(tot - tot_ref).max() <= 1e-4 * np.abs(tot_ref).max(), precision


@pytest.mark.gpu
def test_elements_roundtrip_and_reset():
    mesh, hydro, physics, model = _dense_case(1.0)
    cons, _ = make_case(mesh, hydro, physics, model)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        assert np.all(rt.elements(0) == 0.0)
        e = np.random.default_rng(5).normal(size=(4, 4, 7, 4))
        rt.upload_elements(0, e)
        assert np.array_equal(rt.elements(0), e)
        rt.upload(0, cons)
        assert np.all(rt.elements(0) == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32_comp"])
def test_unbound_orbit_is_the_reference_error(precision):
    """A gas mass far above the binary's makes the perturbed orbit unbound:
    OrbitalEvolutionError at (0, 0) with the binary's state, and the state
    is left as it was."""
    mesh, hydro, physics, model = _dense_case(1e4)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    with pytest.raises(binding.OracleHydroError) as ei:
        ref.advance(1)
    want = ei.value.err
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
        rt.upload(0, cons)
        with pytest.raises(b2.HydroError) as gi:
            rt.advance(1)
        got = gi.value
        after, t, it = rt.download(0)
    assert got.code == want.code == 3
    assert got.kind == "OrbitalEvolutionError"
    assert got.position == (0.0, 0.0)
    assert got.block == (want.block_i, want.block_j)
    assert got.time == want.time
    assert np.allclose(got.binary, list(want.binary), rtol=0, atol=1e-14)
    assert t == 0.0 and it == 0
    assert np.array_equal(after, cons) or precision != "fp64"
