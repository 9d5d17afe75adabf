"""Massless tracer particles: oracle properties on CPU, GPU parity against the
oracle (FP64, 1e-12) and the FP32 paths' agreement with FP64."""
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from helpers import make_case
from oracle import binding


def _tracers(n=500, seed=3):
    xy = b2.presets.annulus_tracers(n, seed=seed)
    # a few near the periodic edges to exercise the wrap
    edge = np.array([[7.99, 0.3], [-7.999, -2.0], [0.5, 7.995], [-3.0, -7.9999], [7.9999, -7.9999]])
    return np.concatenate([xy, edge])


def test_oracle_tracers_follow_the_disk():
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=21)
    cons, cfg = make_case(mesh, hydro, physics, model)
    st = binding.OracleState(cfg, cons)
    xy0 = b2.presets.annulus_tracers(400, seed=1, r_in=3.0, r_out=5.0)
    st.set_tracers(xy0)
    st.advance(5, nthreads=4)
    r0 = np.hypot(*xy0.T)
    r1 = np.hypot(*st.tracers.T)
    assert np.all(np.abs(r1 / r0 - 1) < 0.01)                       # Keplerian: nearly circular
    dphi = np.angle((st.tracers[:, 0] + 1j * st.tracers[:, 1]) / (xy0[:, 0] + 1j * xy0[:, 1]))
    omega = dphi / st.time.value
    assert np.all(omega > 0)                                          # counter-clockwise, like the gas
    assert np.allclose(omega, r0 ** -1.5, rtol=0.05)                  # at the Kepler rate
    assert np.all(np.abs(st.tracers) < 8.0)


@pytest.mark.gpu
@pytest.mark.parametrize("rk", ["RK1", "RK2", "RK3"])
def test_tracers_gpu_match_oracle(rk):
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=22)
    physics = dataclasses.replace(physics, rk_order=rk)
    cons, cfg = make_case(mesh, hydro, physics, model)
    xy = _tracers()
    ref = binding.OracleState(cfg, cons)
    ref.set_tracers(xy)
    with b2.Runtime([b2.Run(mesh, hydro, physics)]) as rt:
        rt.upload(0, cons)
        rt.set_tracers(0, xy)
        for _ in range(3):
            rt.advance(4)
            ref.advance(4)
        got = rt.tracers(0)
        state, _, _ = rt.download(0)
    assert np.max(np.abs(got - ref.tracers)) <= 1e-12 * 8.0
    assert np.max(np.abs(state - ref.cons) / np.abs(ref.cons).max(axis=(0, 1, 2, 3))) <= 1e-12
    assert np.all(got >= -8.0) and np.all(got < 8.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32_state64", "fp32_comp"])
def test_tracers_mixed_precision(precision):
    mesh, hydro, physics, model = b2.presets.iso_disk(4, 32, seed=23)
    cons, _ = make_case(mesh, hydro, physics, model)
    xy = _tracers(300, seed=9)
    out = {}
    for p in ("fp64", precision):
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=p) as rt:
            rt.upload(0, cons)
            rt.set_tracers(0, xy)
            for _ in range(3):
                rt.advance(5)
            out[p] = rt.tracers(0)
    d = out[precision] - out["fp64"]
    d = (d + 8.0) % 16.0 - 8.0                      # compare on the same periodic image
    assert np.max(np.abs(d)) < 1e-5
