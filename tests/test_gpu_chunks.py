"""Row chunks across block rows on the TMA-staged FP32 kernel (stage2.cuh:
Euler, FP64-state and 32-column tiles): the state of block-aligned tiles bit
for bit, and the oracle within FP32 tolerance."""
import dataclasses

import numpy as np
import pytest

import binary2d as b2
from helpers import ledger_err, make_case, rel_err, run_pair

pytestmark = pytest.mark.gpu

BUFFER = 4


def euler_case():
    """The small Euler disk of the FP64 parity tests (4 x 4 blocks of 32^2,
    T^4 cooling, no cavity)."""
    mesh = b2.Mesh(num_blocks=4, block_size=32, domain_radius=8.0)
    hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
    physics = b2.presets.iso_physics(q=0.5, e=0.3)
    physics = dataclasses.replace(physics, sink_radius=0.3, softening_length=0.2)
    model = b2.DiskModel(surface_density=1.0, mach_number=5.0, noise=1e-3, seed=5, cavity_radius=0.0)
    return mesh, hydro, physics, model


def advance_with(mesh, hydro, physics, cons, precision, tile, rows, fold=3, advances=3):
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
        rt.set_tile(*tile)
        rt.set_strip_rows(rows)
        assert rt.strip_rows() == rows
        rt.upload(0, cons)
        dts = [rt.advance(fold)[0] for _ in range(advances)]
        s, t, it = rt.download(0)
        return s, t, dts, rt.ledger(0), rt.elements(0)


CASES = [
    # (case, precision, tiles): the first tile is block-aligned, the others chunked
    ("euler", "fp32_comp", [((32, 32), 0), ((32, 8), 12), ((32, 16), 20)]),
    ("euler", "fp32_state64", [((32, 32), 0), ((32, 8), 12)]),
    ("iso", "fp32_state64", [((64, 32), 0), ((64, 32), 40), ((32, 16), 20)]),
    ("iso", "fp32_comp", [((32, 32), 0), ((32, 32), 40)]),   # 32-column tiles: the TMA-staged kernel
]


@pytest.mark.parametrize("case,precision,tiles", CASES)
def test_stage2_row_chunks_match_block_tiles(case, precision, tiles):
    if case == "euler":
        mesh, hydro, physics, model = euler_case()
    else:
        mesh, hydro, physics, model = b2.presets.iso_disk(3, 64, seed=71)
    cons = make_case(mesh, hydro, physics, model)[0]
    out = [advance_with(mesh, hydro, physics, cons, precision, tile, rows) for tile, rows in tiles]
    s0, t0, dts0, led0, el0 = out[0]
    for s, t, dts, led, el in out[1:]:
        assert np.array_equal(s, s0)
        assert t == t0 and dts == dts0
        assert ledger_err(led, led0) <= 1e-5
        escale = np.maximum(np.abs(el0).max(axis=(0, 1)), 1e-300)
        assert (np.abs(el - el0).max(axis=(0, 1)) / escale).max() <= 1e-5


@pytest.mark.parametrize("precision", ["fp32_comp", "fp32_state64"])
def test_stage2_row_chunks_euler_vs_oracle(precision):
    mesh, hydro, physics, model = euler_case()
    r = run_pair(mesh, hydro, physics, model, fold=3, advances=3, precision=precision, tile=(32, 8),
                 strip_rows=12)
    assert np.all(np.isfinite(r["gpu"]))
    assert rel_err(r["gpu"], r["ref"]) <= 2e-4
    l1 = np.abs(r["gpu"][..., 0] - r["ref"][..., 0]).sum() / np.abs(r["ref"][..., 0]).sum()
    assert l1 <= 1e-5, l1
    err, zero = item_errors(r["led"], r["led_ref"])
    assert all(err[k] <= 1e-4 for k in range(7) if k != BUFFER), err
    assert err[BUFFER] <= 5e-3, err
    assert zero <= 1e-6, zero
    assert r["it"] == r["it_ref"]


def item_errors(led, ref):
    """Per ledger item, the largest |GPU - oracle| over blocks and fields
    against the item's largest |oracle|: a field that is zero up to rounding
    (the oracle's FP64 sum of a near-cancelling energy term is ~1e-12 where
    FP32 gives ~1e-10) is judged against its item.  Items the oracle leaves
    at zero are judged against the largest item."""
    scale = np.abs(ref).max(axis=(0, 1, 3))
    diff = np.abs(led - ref).max(axis=(0, 1, 3))
    err = np.where(scale > 0, diff / np.maximum(scale, 1e-300), 0.0)
    zero = float((diff[scale == 0] / scale.max()).max()) if (scale == 0).any() else 0.0
    return err, zero
