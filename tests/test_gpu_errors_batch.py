"""Failure path, batched runs and the mixed-precision variants on the GPU."""
import ctypes
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from helpers import ledger_err, make_case, rel_err, run_pair
from oracle import binding

pytestmark = pytest.mark.gpu


def test_negative_density_reports_and_keeps_state():
    """HydroErrorType::NegativeDensity (physics.rs:499-501): the advance fails
    with the zone's position and the context keeps the pre-advance state,
    as the caller's copy of State does in main.rs:159-205."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=11)
    cons, cfg = make_case(mesh, hydro, physics, model)
    bad = cons.copy()
    bad[2, 1, 5, 7, 0] = -1e-3          # block (2,1), zone (5,7)
    with b2.Runtime([b2.Run(mesh, hydro, physics)]) as rt:
        rt.upload(0, bad, background=cons, time=1.5, iteration=4)
        with pytest.raises(b2.HydroError) as ei:
            rt.advance(2)
        e = ei.value
        assert e.kind == "NegativeDensity"
        assert e.block == (2, 1) and e.zone == (5, 7)
        assert e.value == -1e-3
        xc = np.empty(32)
        binding.load().oracle_cell_centers(ctypes.byref(cfg), 2, xc.ctypes.data_as(binding.c_dp))
        assert e.position[0] == xc[5]
        out, t, it = rt.download(0)
        assert np.array_equal(out, bad) and t == 1.5 and it == 4
        # the oracle agrees that the step fails
        ref = binding.OracleState(cfg, bad, background=cons)
        with pytest.raises(binding.OracleHydroError) as eo:
            ref.advance(2)
        assert eo.value.err.code == 1
        # the context recovers once the state is repaired
        rt.upload_conserved(0, cons)
        rt.advance(1)


def test_negative_pressure_euler():
    mesh = b2.Mesh(num_blocks=2, block_size=32, domain_radius=8.0)
    hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=0.0)
    physics = b2.presets.iso_physics()
    model = b2.DiskModel(surface_density=1.0, mach_number=10.0)
    cons, cfg = make_case(mesh, hydro, physics, model)
    bad = cons.copy()
    bad[1, 0, 3, 4, 3] = 0.5 * (bad[1, 0, 3, 4, 1] ** 2 + bad[1, 0, 3, 4, 2] ** 2) / bad[1, 0, 3, 4, 0] - 1.0
    with b2.Runtime([b2.Run(mesh, hydro, physics)]) as rt:
        rt.upload(0, bad, background=cons)
        with pytest.raises(b2.HydroError) as ei:
            rt.advance(1)
        assert ei.value.kind == "NegativePressure"
        assert ei.value.block == (1, 0) and ei.value.zone == (3, 4)


def test_batched_runs_match_single_runs():
    """Runs of uneven sizes advanced together equal the same runs advanced
    one at a time (each with its own dt)."""
    cases = [b2.presets.iso_disk(nb, 32, seed=20 + k, q=q, e=e, mach=m, nu=nu)
             for k, (nb, q, e, m, nu) in enumerate([(2, 0.3, 0.1, 12.0, 1e-4), (4, 1.0, 0.0, 10.0, 1e-3),
                                                    (3, 0.6, 0.5, 30.0, 5e-4)])]
    runs = [b2.Run(m, h, p) for (m, h, p, _) in cases]
    inits = [make_case(m, h, p, md, run=k)[0] for k, (m, h, p, md) in enumerate(cases)]
    with b2.Runtime(runs) as rt:
        for k, c in enumerate(inits):
            rt.upload(k, c)
        dts = [rt.advance(3) for _ in range(2)]
        batched = [rt.download(k)[0] for k in range(len(runs))]
    for k, (run, c) in enumerate(zip(runs, inits)):
        with b2.Runtime([run]) as rt:
            rt.upload(0, c)
            d = [rt.advance(3)[0] for _ in range(2)]
            single = rt.download(0)[0]
        assert np.array_equal(single, batched[k])
        assert np.array_equal(np.array(d), np.array([x[k] for x in dts]))


@pytest.mark.parametrize("precision,tol", [("fp32_state64", 2e-4), ("fp32_comp", 2e-4)])
def test_mixed_precision_close_to_fp64(precision, tol):
    """The FP32-stencil paths stay within FP32 round-off of the FP64 path
    over 60 steps (max-norm, relative per field)."""
    mesh, hydro, physics, model = b2.presets.iso_disk(8, 32, seed=12)
    r = run_pair(mesh, hydro, physics, model, fold=10, advances=6, precision=precision)
    err = rel_err(r["gpu"], r["ref"])
    l1 = np.abs(r["gpu"][..., 0] - r["ref"][..., 0]).sum() / np.abs(r["ref"][..., 0]).sum()
    assert l1 <= 1e-5, l1
    assert err <= tol, err
    assert ledger_err(r["led"], r["led_ref"]) <= 1e-4


def test_compensated_state_keeps_small_increments():
    """A state advanced by increments far below FP32 resolution: the
    compensated store keeps them, a plain FP32 store would not."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=13)
    physics = dataclasses.replace(physics, buffer_rate=0.0, sink_rate=0.0)
    r64 = run_pair(mesh, hydro, physics, model, fold=10, advances=3, precision="fp64")
    rc = run_pair(mesh, hydro, physics, model, fold=10, advances=3, precision="fp32_comp")
    d64 = r64["gpu"] - r64["cons0"]
    dc = rc["gpu"] - rc["cons0"]
    # the change itself is resolved to FP32 relative accuracy of the change
    num = np.abs(dc[..., 0] - d64[..., 0]).sum()
    den = np.abs(d64[..., 0]).sum()
    assert num / den < 1e-3, num / den


@pytest.mark.parametrize("precision", ["fp64", "fp32_comp"])
def test_page_locked_host_buffers(precision):
    """Uploads from and downloads into page-locked host buffers (read and
    written in place by the layout kernels) give the same bits as the
    staged copies of ordinary host arrays."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 64, seed=17)
    cons, _ = make_case(mesh, hydro, physics, model)
    outs = []
    for pinned in (False, True):
        src = np.ascontiguousarray(cons.copy())
        dst = np.zeros_like(src)
        if pinned:
            b2.pin(src)
            b2.pin(dst)
        try:
            with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
                rt.upload(0, cons)
                rt.upload_conserved(0, src)
                rt.advance(3)
                rt.download(0, out=dst)
                outs.append(dst.copy())
                # a download into a page-locked buffer round-trips through an upload
                rt.upload_conserved(0, dst)
                again, _, _ = rt.download(0)
                assert np.array_equal(again, dst)
        finally:
            if pinned:
                b2.unpin(src)
                b2.unpin(dst)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("precision", ["fp64", "fp32_comp"])
def test_layout_roundtrip_odd_element_count(precision):
    """A 15^2 mesh with 3 fields has an odd number of elements: the layout
    kernels' last element, through staged and page-locked buffers."""
    mesh = b2.Mesh(num_blocks=3, block_size=5, domain_radius=8.0)
    hydro, physics = b2.Isothermal(mach_number=10.0), b2.presets.iso_physics()
    cons = b2.initial_state(mesh, hydro, physics, b2.DiskModel(noise=1e-3, seed=3))
    assert cons.size % 2 == 1
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
        rt.upload(0, cons)
        out, _, _ = rt.download(0)
        src = np.ascontiguousarray(cons.copy())
        dst = np.zeros_like(src)
        b2.pin(src)
        b2.pin(dst)
        try:
            rt.upload_conserved(0, src)
            rt.download(0, out=dst)
        finally:
            b2.unpin(src)
            b2.unpin(dst)
    if precision == "fp64":
        assert np.array_equal(out, cons)
    assert np.array_equal(dst, out)


def test_pipelined_transfers_match_synchronous():
    """upload_async / advance_async / download_async in a loop, two steps in
    flight: each step's result is bitwise the synchronous loop's."""
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 64, seed=19)
    cons, _ = make_case(mesh, hydro, physics, model)
    inputs = [cons * (1.0 + 1e-3 * k) for k in range(4)]
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp32_comp") as rt:
        rt.upload(0, cons)
        want = []
        for x in inputs:
            rt.upload_conserved(0, x)
            rt.advance(2)
            want.append(rt.download(0)[0].copy())
    src = [np.ascontiguousarray(x) for x in inputs]
    dst = [np.zeros_like(x) for x in inputs]
    for a in src + dst:
        b2.pin(a)
    try:
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision="fp32_comp") as rt:
            rt.upload(0, cons)
            for k in range(len(src)):
                rt.upload_conserved_async(0, src[k])
                rt.advance_async(2)
                rt.download_async(0, dst[k])
                rt.transfers_wait(1)
                if k >= 1:
                    assert np.array_equal(dst[k - 1], want[k - 1])
            rt.transfers_wait(0)
            rt.synchronize()
    finally:
        for a in src + dst:
            b2.unpin(a)
    for k in range(len(src)):
        assert np.array_equal(dst[k], want[k])
