"""The allocation-free stage entry point, b2d_stage_noalloc.

For callers that cannot call cudaMalloc (a host code with its own fixed
device memory pool, an allocator-less runtime, code running under another
framework's stream capture): they pass every buffer, and the stage kernel's
scratch comes from a static device array inside the library.  This test
drives it through the C ABI on buffers the test owns and compares two calls
in a row (one RK2 step: stage 1, then stage 2 with the average) with the
context-based entry point, b2d_advance, to the FP64 tolerance of the parity
tests (1e-12, max-norm per field).

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest

import binary2d as b2
from binary2d import _lib

pytestmark = pytest.mark.gpu

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


def test_stage_noalloc_matches_advance():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=31)
    cfg = b2.to_c(mesh, hydro, physics)
    cons = b2.initial_state(mesh, hydro, physics, model)
    nf, nb = 3, mesh.num_blocks

    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp64") as rt:
        rt.upload(0, cons)
        dt = float(rt.advance(1)[0])          # one RK2 step
        ref, t_ref, _ = rt.download(0)
        led_ref = rt.ledger(0)
        amax_ref = rt.max_signal_speed(0)

    dev = torch.device("cuda:0")
    a = torch.from_numpy(planes(cons)).to(dev)
    bg = a.clone()
    s1 = torch.empty_like(a)
    s2 = torch.empty_like(a)
    zeros = torch.zeros(nb * nb * 7 * nf, dtype=torch.float64, device=dev)
    l1 = torch.empty_like(zeros)
    l2 = torch.empty_like(zeros)
    amax = torch.zeros(1, dtype=torch.float64, device=dev)

    for repeat in range(2):  # the shared scratch must serve consecutive calls
        s1.fill_(float("nan"))
        s2.fill_(float("nan"))
        torch.cuda.synchronize()
        # stage 1: s1 = L(a) at time 0; stage 2: s2 = (L(s1) + a) / 2 at time dt
        call(lib, cfg, a, bg, None, s1, zeros, None, l1, 0.0, dt, 0.0)
        call(lib, cfg, s1, bg, a, s2, l1, zeros, l2, 0.0 + dt, dt, 0.5, amax)
        torch.cuda.synchronize()
        got = s2.cpu().numpy()
        want = planes(ref)
        scale = np.abs(want).reshape(nf, -1).max(axis=1)
        err = (np.abs(got - want).reshape(nf, -1).max(axis=1) / scale).max()
        assert err <= TOL, (repeat, err)
        led = l2.cpu().numpy().reshape(led_ref.shape)
        lscale = np.maximum(np.abs(led_ref).sum(axis=(0, 1)), 1e-300)
        assert (np.abs(led - led_ref).sum(axis=(0, 1)) / lscale).max() <= TOL
        assert abs(amax.item() - amax_ref) <= TOL * amax_ref
    assert abs(t_ref - dt) <= TOL * dt


def test_stage_noalloc_rejects_oversize_mesh():
    lib = _lib.load()
    mesh, hydro, physics, _ = b2.presets.iso_disk(256, 64)     # 16384^2: too many tiles for the scratch
    cfg = b2.to_c(mesh, hydro, physics)
    err = _lib.B2DError()
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.b2d_stage_noalloc(ctypes.byref(cfg), dummy, dummy, None, dummy, dummy, None, dummy, 0.0, 1e-3, 0.0,
                               None, ctypes.byref(err), None)
    assert st == 6 and "scratch" in _lib.last_error()
