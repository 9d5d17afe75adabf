"""CPU tests: the oracle's analytic identities, the C ABI's exports, and the
host-side initial state against the oracle's."""
import ctypes
import math
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import binary2d as b2
from binary2d import _lib
from helpers import make_case
from oracle import binding

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cfg(hydro=None, **kw):
    mesh, h, physics, model = b2.presets.iso_disk(2, 8)
    return b2.to_c(mesh, hydro or h, physics)


def _dp(a):
    return a.ctypes.data_as(binding.c_dp)


# ----------------------------------------------------------------------------
# C ABI


def test_library_exports_every_declared_symbol(b2d_lib):
    text = open(os.path.join(ROOT, "include", "b2d.h")).read()
    declared = set(re.findall(r"\b(b2d_[a-z_0-9]+)\s*\(", text))
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (b2d_[a-z_0-9]+)", out))
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        assert hasattr(b2d_lib, name)


def test_config_struct_layout_matches_oracle():
    # both sides of the ctypes struct are the same C layout; a field count check
    # guards against the headers drifting apart
    hdr = open(os.path.join(ROOT, "oracle", "oracle.h")).read()
    body = hdr[hdr.index("typedef struct oracle_config"):hdr.index("} oracle_config;")]
    fields = re.findall(r"\b(?:int32_t|double)\s+(\w+);", body)
    assert fields == [f for f, _ in _lib.B2DConfig._fields_]


def test_host_initial_state_matches_oracle_bitwise():
    for hydro in (b2.Isothermal(mach_number=10.0), b2.Euler(gamma_law_index=5 / 3)):
        mesh, _, physics, model = b2.presets.iso_disk(3, 16, seed=42)
        model.mach_number = 10.0
        cons = b2.initial_state(mesh, hydro, physics, model, run=3)
        cfg = b2.to_c(mesh, hydro, physics)
        m = _lib.B2DDiskModel(surface_density=1.0, mach_number=10.0, cavity_radius=model.cavity_radius,
                              cavity_floor=model.cavity_floor, noise=model.noise, seed=42, run=3)
        ref = binding.initial_state(cfg, m, cons.shape)
        assert np.array_equal(cons, ref)


@pytest.mark.parametrize("kind", ["infinite_disk", "infinite_alpha_disk", "finite_disk", "residual_test"])
def test_all_initial_models_match_oracle_bitwise(kind):
    mesh = b2.Mesh(num_blocks=3, block_size=16, domain_radius=6.0)
    for hydro in (b2.Isothermal(mach_number=10.0), b2.Euler(gamma_law_index=1.66666666666666)):
        physics = b2.presets.iso_physics()
        model = b2.DiskModel(surface_density=1.0, mach_number=8.0, kind=kind, disk_mass=1e-3, disk_width=3.0,
                             disk_radius=3.0, softening_length=0.05, noise=1e-3, seed=7, cavity_radius=1.0,
                             core_radius=0.7, edge_width=1.5)
        cons = b2.initial_state(mesh, hydro, physics, model)
        cfg = b2.to_c(mesh, hydro, physics)
        m = _lib.B2DDiskModel(surface_density=1.0, mach_number=8.0, cavity_radius=1.0, cavity_floor=1e-4,
                              noise=1e-3, seed=7, run=0, kind=b2.config.MODEL_KINDS[kind], disk_mass=1e-3,
                              disk_width=3.0, disk_radius=3.0, disk_softening=0.05, core_radius=0.7,
                              edge_width=1.5)
        ref = binding.initial_state(cfg, m, cons.shape)
        assert np.array_equal(cons, ref)
        assert np.all(np.isfinite(cons)) and np.all(cons[..., 0] > 0)


def test_initial_state_noise_is_layout_independent():
    """The noise is keyed by global zone index: re-blocking the same mesh
    gives the same field."""
    mesh_a = b2.Mesh(num_blocks=4, block_size=16, domain_radius=8.0)
    mesh_b = b2.Mesh(num_blocks=2, block_size=32, domain_radius=8.0)
    hydro, physics = b2.Isothermal(mach_number=10.0), b2.presets.iso_physics()
    model = b2.DiskModel(noise=1e-3, seed=5)
    a = b2.initial_state(mesh_a, hydro, physics, model)
    b = b2.initial_state(mesh_b, hydro, physics, model)
    ga = a.transpose(0, 2, 1, 3, 4).reshape(64, 64, 3)
    gb = b.transpose(0, 2, 1, 3, 4).reshape(64, 64, 3)
    assert np.allclose(ga, gb, rtol=1e-15, atol=0)
    rel = ga[..., 0] / b2.initial_state(mesh_a, hydro, physics, b2.DiskModel()).transpose(0, 2, 1, 3, 4).reshape(64, 64, 3)[..., 0] - 1
    assert np.abs(rel).max() <= 1e-3 and np.abs(rel).max() > 9e-4


# ----------------------------------------------------------------------------
# oracle identities (self-consistency checks of the restatement)


def test_plm_gradient_properties(oracle_lib):
    g = oracle_lib.oracle_plm_gradient
    assert g(0.0, 1.0, 2.0, 3.0) == 0.0                   # θ = 0 ⇒ no slope
    assert g(1.5, 1.0, 2.0, 3.0) == 1.0                   # smooth: central difference
    assert g(1.5, 1.0, 3.0, 2.0) == 0.0                   # extremum ⇒ zero slope
    assert g(1.0, 0.0, 1.0, 10.0) == 1.0                  # limited by the smaller side
    assert g(2.0, 3.0, 2.0, 1.0) == -1.0
    rng = np.random.default_rng(0)
    for a, b, c in rng.normal(size=(200, 3)):
        s = g(1.5, a, b, c)
        assert abs(s) <= 1.5 * min(abs(b - a), abs(c - b)) + 1e-15
        assert s == 0.0 or np.sign(s) == np.sign(c - a)


@pytest.mark.parametrize("kind", ["iso", "euler"])
def test_hlle_consistency(oracle_lib, kind):
    """HLLE with equal states returns the physical flux."""
    hydro = b2.Isothermal(mach_number=10.0) if kind == "iso" else b2.Euler(gamma_law_index=5 / 3)
    cfg = _cfg(hydro)
    nf = 3 if kind == "iso" else 4
    rng = np.random.default_rng(1)
    for _ in range(50):
        p = np.array([rng.uniform(0.1, 2), rng.normal(), rng.normal(), rng.uniform(0.1, 2)][:nf])
        for axis in (0, 1):
            f = np.zeros(4)
            fh = np.zeros(4)
            oracle_lib.oracle_physical_flux(ctypes.byref(cfg), _dp(p), axis, 0.3, _dp(f))
            oracle_lib.oracle_hlle(ctypes.byref(cfg), _dp(p), _dp(p), axis, 0.3, _dp(fh))
            assert np.allclose(f[:nf], fh[:nf], rtol=1e-13, atol=1e-14)


def test_hlle_supersonic_upwinding(oracle_lib):
    cfg = _cfg()
    pl = np.array([1.0, 5.0, 0.2])
    pr = np.array([0.5, 4.0, -0.1])
    f = np.zeros(3)
    fl = np.zeros(3)
    oracle_lib.oracle_hlle(ctypes.byref(cfg), _dp(pl), _dp(pr), 0, 0.01, _dp(f))
    oracle_lib.oracle_physical_flux(ctypes.byref(cfg), _dp(pl), 0, 0.01, _dp(fl))
    assert np.allclose(f, fl, rtol=1e-14)


def test_kepler_circular_orbit():
    for q in (1.0, 0.5, 0.1):
        mesh, hydro, physics, _ = b2.presets.iso_disk(2, 8, q=q)
        cfg = b2.to_c(mesh, hydro, physics)
        for t in (0.0, 1.0, math.pi, 2 * math.pi):
            p1, p2 = binding.orbital_state(cfg, t)
            assert math.isclose(p1.m, 1 / (1 + q), rel_tol=1e-15) and math.isclose(p2.m, q / (1 + q), rel_tol=1e-15)
            sep = math.hypot(p2.x - p1.x, p2.y - p1.y)
            assert math.isclose(sep, 1.0, rel_tol=1e-14)
            assert math.isclose(math.hypot(p1.x, p1.y), q / (1 + q), rel_tol=1e-14)
            assert abs(p1.m * p1.x + p2.m * p2.x) < 1e-15 and abs(p1.m * p1.vx + p2.m * p2.vx) < 1e-15
        p1, p2 = binding.orbital_state(cfg, 2 * math.pi)   # period 2π (physics.rs:21)
        assert abs(p2.x - 1 / (1 + q)) < 1e-13 and abs(p2.y) < 1e-13


def test_kepler_eccentric_orbit():
    mesh, hydro, physics, _ = b2.presets.iso_disk(2, 8, q=0.5, e=0.6)
    cfg = b2.to_c(mesh, hydro, physics)
    p1, p2 = binding.orbital_state(cfg, 0.0)
    assert math.isclose(p2.x - p1.x, 0.4, rel_tol=1e-14)    # periapsis a(1 - e)
    p1, p2 = binding.orbital_state(cfg, math.pi)
    assert math.isclose(p1.x - p2.x, 1.6, rel_tol=1e-13)    # apoapsis a(1 + e)
    # energy conservation of the relative orbit: v²/2 - M/r = -M/2a
    for t in np.linspace(0, 6, 7):
        p1, p2 = binding.orbital_state(cfg, t)
        r = math.hypot(p2.x - p1.x, p2.y - p1.y)
        v2 = (p2.vx - p1.vx) ** 2 + (p2.vy - p1.vy) ** 2
        assert math.isclose(0.5 * v2 - 1.0 / r, -0.5, rel_tol=1e-12)


def test_mass_conserved_without_sources():
    """Flux telescoping on the periodic block mesh: with sinks and buffer off,
    total mass is conserved to round-off.  Euler is used because its face
    flux does not depend on the face position; the isothermal face sound
    speed comes from the potential at the face (physics.rs:596), so the two
    images of a periodic boundary face (x = -R and x = +R) carry different
    fluxes and the reference itself does not conserve mass there."""
    import dataclasses
    mesh, _, physics, model = b2.presets.iso_disk(4, 16, seed=3)
    hydro = b2.Euler(gamma_law_index=5 / 3, cooling_coefficient=1e-2, pressure_floor=1e-10)
    model.mach_number = 10.0
    model.cavity_radius = 0.0
    physics = dataclasses.replace(physics, sink_rate=0.0, buffer_rate=0.0)
    cons, cfg = make_case(mesh, hydro, physics, model)
    st = binding.OracleState(cfg, cons)
    m0 = cons[..., 0].sum()
    st.advance(5, nthreads=4)
    assert abs(st.cons[..., 0].sum() - m0) <= 1e-13 * m0


def test_point_symmetry_equal_mass_circular():
    """q = 1, e = 0 and a noise-free disk are symmetric under (x, y) → (-x, -y)."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 16, seed=3)
    model.noise = 0.0
    cons, cfg = make_case(mesh, hydro, physics, model)
    st = binding.OracleState(cfg, cons)
    st.advance(4, nthreads=4)
    g = st.cons.transpose(0, 2, 1, 3, 4).reshape(64, 64, 3)
    rot = g[::-1, ::-1]
    assert np.allclose(g[..., 0], rot[..., 0], rtol=1e-12, atol=0)
    assert np.allclose(g[..., 1], -rot[..., 1], rtol=1e-10, atol=1e-13)


def test_oracle_threads_do_not_change_results():
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 16, seed=4)
    cons, cfg = make_case(mesh, hydro, physics, model)
    a = binding.OracleState(cfg, cons)
    b = binding.OracleState(cfg, cons)
    a.advance(3, nthreads=1)
    b.advance(3, nthreads=7)
    assert np.array_equal(a.cons, b.cons) and np.array_equal(a.ledger, b.ledger)


def test_oracle_reports_negative_density():
    mesh, hydro, physics, model = b2.presets.iso_disk(2, 16, seed=4)
    cons, cfg = make_case(mesh, hydro, physics, model)
    cons[1, 1, 3, 2, 0] = -0.5
    st = binding.OracleState(cfg, cons)
    with pytest.raises(binding.OracleHydroError) as e:
        st.advance(1, nthreads=2)
    assert e.value.err.code == 1 and e.value.err.value == -0.5
    assert (e.value.err.block_i, e.value.err.block_j, e.value.err.zone_i, e.value.err.zone_j) == (1, 1, 3, 2)


def _run_geometry_check(tmp_path, *defines):
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "chunk_geometry_check")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "chunk_geometry_check.cu")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", *defines, src, "-o", exe], check=True,
                   capture_output=True, text=True)
    return subprocess.run([exe], capture_output=True, text=True)


def test_tile_geometry_pieces(tmp_path):
    """Row chunks across block rows and tiles across block columns: every row
    lies in its piece's block row, every ledger piece has one slot, and every
    block receives exactly its count of pieces (the real runtime.cuh helpers,
    with the stage kernels' slot formulas, on the host)."""
    r = _run_geometry_check(tmp_path)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


def test_tile_geometry_check_rejects_a_wrong_slot(tmp_path):
    r = _run_geometry_check(tmp_path, "-DPLANT_SLOT_MISTAKE")
    assert r.returncode != 0 and "piece slot" in r.stdout, r.stdout


def test_missing_library_fails_loudly():
    """No CPU fallback: without libb2d.so the product path raises, and says so."""
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from binary2d import _lib\n"
            "try:\n"
            "    _lib.load('/nonexistent/libb2d.so')\n"
            "except RuntimeError as e:\n"
            "    print('raised:', e)\n") % os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                               "app-binary2d_gb300")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "raised:" in r.stdout and "no CPU fallback" in r.stdout, r.stdout + r.stderr
