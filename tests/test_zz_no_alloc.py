"""The allocation-free stage entry point, b2d_stage_noalloc.

For callers that cannot call cudaMalloc (a host code with its own fixed
device memory pool, or an allocator-less runtime): they pass every buffer,
and the stage kernel's scratch comes from a static device array inside the
library.  These tests drive it through the C ABI on buffers the test owns and
compare two calls in a row (one RK2 step: stage 1, then stage 2 with the
average) with the context-based entry point, b2d_advance, to the FP64
tolerance of the parity tests (1e-12, max-norm per field), for the
isothermal and the Euler system; a host-made negative density must be
reported at the same block and zone, with the same value, as b2d_advance
reports it.  Arguments it must refuse are refused before any device work.

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest

import binary2d as b2
from binary2d import _lib

TOL = 1e-12


def planes(cons):
    """Block layout [nb, nb, bs, bs, nf] -> field planes [nf, N, N]."""
    nb, _, bs, _, nf = cons.shape
    return np.ascontiguousarray(cons.transpose(4, 0, 2, 1, 3).reshape(nf, nb * bs, nb * bs))


def call(lib, cfg, a, bg, base, out, led_in, led_base, led_out, time, dt, bf, amax=None):
    err = _lib.B2DError()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    st = lib.b2d_stage_noalloc(ctypes.byref(cfg), ptr(a), ptr(bg), ptr(base), ptr(out), ptr(led_in),
                               ptr(led_base), ptr(led_out), time, dt, bf, ptr(amax), ctypes.byref(err), None)
    assert st == 0, _lib.last_error()


def rk2_step_noalloc(torch, lib, cfg, cons, nf, nb, dt):
    """One RK2 step as two allocation-free stage calls; returns the state
    planes, the ledger and the max signal speed of the result."""
    dev = torch.device("cuda:0")
    a = torch.from_numpy(planes(cons)).to(dev)
    bg = a.clone()
    s1 = torch.full_like(a, float("nan"))
    s2 = torch.full_like(a, float("nan"))
    zeros = torch.zeros(nb * nb * 7 * nf, dtype=torch.float64, device=dev)
    l1 = torch.empty_like(zeros)
    l2 = torch.empty_like(zeros)
    amax = torch.zeros(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    # stage 1: s1 = L(a) at time 0; stage 2: s2 = (L(s1) + a) / 2 at time dt
    call(lib, cfg, a, bg, None, s1, zeros, None, l1, 0.0, dt, 0.0)
    call(lib, cfg, s1, bg, a, s2, l1, zeros, l2, 0.0 + dt, dt, 0.5, amax)
    torch.cuda.synchronize()
    return s2.cpu().numpy(), l2.cpu().numpy(), amax.item()


def compare_with_advance(mesh, hydro, physics, model):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    cfg = b2.to_c(mesh, hydro, physics)
    cons = b2.initial_state(mesh, hydro, physics, model)
    nf, nb = b2.num_fields(hydro), mesh.num_blocks

    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        dt = float(rt.advance(1)[0])          # one RK2 step
        ref, t_ref, _ = rt.download(0)
        led_ref = rt.ledger(0)
        amax_ref = rt.max_signal_speed(0)

    for repeat in range(2):  # the shared scratch must serve consecutive calls
        got, led, amax = rk2_step_noalloc(torch, lib, cfg, cons, nf, nb, dt)
        want = planes(ref)
        scale = np.abs(want).reshape(nf, -1).max(axis=1)
        err = (np.abs(got - want).reshape(nf, -1).max(axis=1) / scale).max()
        assert err <= TOL, (repeat, err)
        led = led.reshape(led_ref.shape)
        lscale = np.maximum(np.abs(led_ref).sum(axis=(0, 1)), 1e-300)
        assert (np.abs(led - led_ref).sum(axis=(0, 1)) / lscale).max() <= TOL
        assert abs(amax - amax_ref) <= TOL * amax_ref
    assert abs(t_ref - dt) <= TOL * dt


@pytest.mark.gpu
def test_stage_noalloc_matches_advance():
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=31)
    compare_with_advance(mesh, hydro, physics, model)


@pytest.mark.gpu
def test_stage_noalloc_euler_matches_advance():
    """Four conserved fields (Euler, T^4 cooling, alpha viscosity): another
    scratch size and another stage kernel instantiation."""
    import dataclasses
    mesh = b2.Mesh(num_blocks=4, block_size=32, domain_radius=8.0)
    hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
    physics = dataclasses.replace(b2.presets.iso_physics(q=0.5, e=0.3), sink_radius=0.3, softening_length=0.2,
                                  viscosity=("alpha", 0.1))
    model = b2.DiskModel(surface_density=1.0, mach_number=5.0, noise=1e-3, seed=5, cavity_radius=0.0)
    compare_with_advance(mesh, hydro, physics, model)


@pytest.mark.gpu
def test_stage_noalloc_reports_the_failing_zone():
    """A negative density planted in the input: the error code, block, zone,
    value and position match what b2d_advance reports for the same state."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=33)
    cfg = b2.to_c(mesh, hydro, physics)
    cons = b2.initial_state(mesh, hydro, physics, model)
    cons[2, 1, 5, 17, 0] = -1e-3           # block (2, 1), zone (5, 17)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        with pytest.raises(b2.HydroError) as info:
            rt.advance(1)
    want = info.value
    dev = torch.device("cuda:0")
    a = torch.from_numpy(planes(cons)).to(dev)
    out = torch.empty_like(a)
    nf, nb = 3, mesh.num_blocks
    zeros = torch.zeros(nb * nb * 7 * nf, dtype=torch.float64, device=dev)
    led = torch.empty_like(zeros)
    for repeat in range(2):  # a failed call leaves the scratch ready for the next
        err = _lib.B2DError()
        ptr = lambda t: ctypes.c_void_p(t.data_ptr())
        st = lib.b2d_stage_noalloc(ctypes.byref(cfg), ptr(a), ptr(a), None, ptr(out), ptr(zeros), None, ptr(led),
                                   0.0, 1e-3, 0.0, None, ctypes.byref(err), None)
        assert st == 1, (repeat, st, _lib.last_error())
        assert err.code == want.code == 1
        assert (err.block_i, err.block_j) == want.block == (2, 1)
        assert (err.zone_i, err.zone_j) == want.zone == (5, 17)
        assert err.value == want.value == -1e-3
        assert (err.x, err.y) == want.position
        assert tuple(err.binary) == want.binary


@pytest.mark.gpu
def test_stage_noalloc_rejects_oversize_mesh():
    lib = _lib.load()
    mesh, hydro, physics, _ = b2.presets.iso_disk(256, 64)     # 16384^2: too many tiles for the scratch
    cfg = b2.to_c(mesh, hydro, physics)
    err = _lib.B2DError()
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.b2d_stage_noalloc(ctypes.byref(cfg), dummy, dummy, None, dummy, dummy, None, dummy, 0.0, 1e-3, 0.0,
                               None, ctypes.byref(err), None)
    assert st == 6 and "scratch" in _lib.last_error()


def test_stage_noalloc_rejects_unlaunchable_block_width():
    """A block width that is neither a multiple of 32 nor at most 256 would be
    one tile wider than the FP64 kernel's 256 threads: refused as an invalid
    argument before any device work (so this runs without a GPU)."""
    lib = _lib.load()
    mesh, hydro, physics, _ = b2.presets.iso_disk(1, 300)
    cfg = b2.to_c(mesh, hydro, physics)
    err = _lib.B2DError()
    dummy = ctypes.c_void_p(16)   # never dereferenced: the check comes first
    st = lib.b2d_stage_noalloc(ctypes.byref(cfg), dummy, dummy, None, dummy, dummy, None, dummy, 0.0, 1e-3, 0.0,
                               None, ctypes.byref(err), None)
    assert st == 6 and "multiple of 32" in _lib.last_error()
