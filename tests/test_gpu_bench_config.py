"""The benchmarked configuration against the CPU oracle.

bench.py times the 2048^2 isothermal disk (16x16 blocks of 128^2, q = 1,
e = 0, Mach 10, nu = 1e-3, RK2, fold 10) on the compensated-FP32 path with
the tiling its autotuner settles on: 512-column tiles over four block columns
and 54-row chunks across block rows (4 strips x 38 chunks = 152 CTAs, one per
SM).  These tests run exactly that shape, and whatever shape the autotuner
picks on this GPU, for 10 advances of fold 10 (100 RK2 steps) against the
oracle's run of the same seeded state (scheme::advance, src/scheme.rs:323-349):

* fp32_comp: relative L1 of Sigma <= 1e-5, max-norm per field <= 2e-4, dt and
  time to 1e-5, ledger items to 1e-4 of each item's total (the buffer item,
  (u - u_bg) rate dt formed from FP32 high words, to 5e-3);
* fp64 with its default tiles: 1e-12 on the state, dt, time and ledger.

The oracle run (about 10 s on 16 host cores) is shared by all cases.
"""
import numpy as np
import pytest

import binary2d as b2
from helpers import ledger_err, make_case, rel_err
from oracle import binding

pytestmark = pytest.mark.gpu

FOLD, ADVANCES = 10, 10
BUFFER = 4


@pytest.fixture(scope="module")
def disk():
    mesh, hydro, physics, model = b2.presets.disk_2048(seed=1)
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons)
    dts = [ref.advance(FOLD) for _ in range(ADVANCES)]
    return dict(mesh=mesh, hydro=hydro, physics=physics, cons=cons, ref=ref.cons.copy(), led=ref.ledger.copy(),
                t=ref.time.value, it=ref.iteration.value, dts=np.array(dts))


def run_gpu(d, precision, tile=None, strip_rows=None, autotune=False):
    with b2.Runtime([b2.Run(d["mesh"], d["hydro"], d["physics"])], precision=precision) as rt:
        rt.upload(0, d["cons"])
        if autotune:
            rt.autotune(fold=2, reps=2)
        if tile:
            rt.set_tile(*tile)
        if strip_rows is not None:
            rt.set_strip_rows(strip_rows)
        shape = rt.tile() + (rt.strip_rows(),)
        dts = np.array([rt.advance(FOLD)[0] for _ in range(ADVANCES)])
        out, t, it = rt.download(0)
        led = rt.ledger(0)
    return dict(gpu=out, t=t, it=it, dts=dts, led=led, shape=shape)


def check_fp32(d, r):
    l1 = np.abs(r["gpu"][..., 0] - d["ref"][..., 0]).sum() / np.abs(d["ref"][..., 0]).sum()
    assert l1 <= 1e-5, (r["shape"], l1)
    assert rel_err(r["gpu"], d["ref"]) <= 2e-4, r["shape"]
    assert np.allclose(r["dts"], d["dts"], rtol=1e-5, atol=0)
    assert abs(r["t"] - d["t"]) <= 1e-5 * abs(d["t"])
    assert r["it"] == d["it"]
    items = [k for k in range(7) if k != BUFFER]
    assert ledger_err(r["led"][:, :, items], d["led"][:, :, items]) <= 1e-4
    assert ledger_err(r["led"][:, :, [BUFFER]], d["led"][:, :, [BUFFER]]) <= 5e-3


def test_bench_tiling_fp32_comp(disk):
    """512x64 tiles with 54-row chunks: the shape of the timed number."""
    r = run_gpu(disk, "fp32_comp", tile=(512, 64), strip_rows=54)
    assert r["shape"] == (512, 64, 54)
    check_fp32(disk, r)


def test_autotuned_tiling_fp32_comp(disk):
    """Whatever tiling the autotuner picks for the bench on this GPU."""
    r = run_gpu(disk, "fp32_comp", autotune=True)
    check_fp32(disk, r)


def test_fp64_default_tiles(disk):
    r = run_gpu(disk, "fp64")
    tol = 1e-12
    assert rel_err(r["gpu"], disk["ref"]) <= tol
    assert np.allclose(r["dts"], disk["dts"], rtol=tol, atol=0)
    assert abs(r["t"] - disk["t"]) <= tol * abs(disk["t"])
    assert r["it"] == disk["it"]
    assert ledger_err(r["led"], disk["led"]) <= tol
