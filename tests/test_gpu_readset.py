"""Read-set check of the stage kernels (a NaN-poisoned build).

The kernels stage tile rows with their guard columns in shared memory and
compute some guard values they do not need (the paired FP32 kernel's halo
lanes evaluate the outer guard columns -2 and TW + 1, whose own slopes need
stencil points outside the staged columns, and the y face at TW + 1).  The
claim is that no zone's update reads a shared-memory slot the kernel did not
write, nor any of those guard values (the halo extension of scheme.rs:
119-133 and the slice algebra of scheme.rs:250-268 need the 2-zone halo and
the corners to depth 1 only).

A build with B2D_POISON (app-binary2d_gb300/build.py, csrc/tma.cuh) fills
every stage kernel's dynamic shared memory with NaN before use and sets those
unused guard values to NaN.  Every case below runs in that build in a child
process and in the normal build here: the states must be finite and equal bit
for bit.  Cases cover every stage kernel: the generic kernel (8^2 blocks, FP64
and FP32), the FP64 kernel on 64^2 blocks, the TMA-staged kernel (32-column
tiles, Euler, FP64 state), the paired isothermal kernel (64-, 128- and
512-column tiles, row chunks) and the paired Euler kernel (64-, 256- and
512-column tiles, row chunks)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# name: (hydro, num_blocks, block_size, precision, tile (w, h) or None, strip rows)
CASES = {
    "generic_fp64_8": ("iso", 4, 8, "fp64", None, 0),
    "generic_fp32_8": ("iso", 4, 8, "fp32_comp", None, 0),
    "fp64_64": ("iso", 4, 64, "fp64", None, 0),
    "staged_32": ("iso", 4, 64, "fp32_comp", (32, 32), 0),
    "staged_euler_32": ("euler", 4, 64, "fp32_comp", (32, 32), 40),
    "staged_state64_64": ("iso", 4, 64, "fp32_state64", (64, 32), 0),
    "paired_64": ("iso", 4, 64, "fp32_comp", (64, 32), 0),
    "paired_128_chunks": ("iso", 4, 64, "fp32_comp", (128, 32), 50),
    "paired_512_chunks": ("iso", 4, 128, "fp32_comp", (512, 32), 100),
    "paired_euler_64": ("euler", 4, 64, "fp32_comp", (64, 32), 40),
    "paired_euler_256_chunks": ("euler", 4, 128, "fp32_comp", (256, 32), 60),
    "paired_euler_512_chunks": ("euler", 4, 128, "fp32_comp", (512, 32), 100),
}

RUNNER = r"""
import json, sys
import numpy as np
sys.path.insert(0, {pkg!r}); sys.path.insert(0, {root!r})
from binary2d import _lib
_lib.load({lib!r})
import binary2d as b2
cases = json.loads({cases!r})
out = {{}}
for name, (hyd, nb, bs, prec, tile, rows) in cases.items():
    if hyd == "iso":
        import dataclasses
        mesh, hydro, physics, model = b2.presets.iso_disk(nb, bs, seed=91)
        if bs < 32:   # dx = 0.5: the explicit buffer at rate 1000 drives edge zones negative
            physics = dataclasses.replace(physics, buffer_rate=10.0)
    else:
        import dataclasses
        mesh = b2.Mesh(num_blocks=nb, block_size=bs, domain_radius=8.0)
        hydro = b2.Euler(gamma_law_index=5.0 / 3.0, cooling_coefficient=1e-3)
        physics = dataclasses.replace(b2.presets.iso_physics(q=0.5, e=0.3), sink_radius=0.3,
                                      softening_length=0.2, viscosity=("alpha", 0.1))
        model = b2.DiskModel(surface_density=1.0, mach_number=5.0, noise=1e-3, seed=5)
    cons = b2.initial_state(mesh, hydro, physics, model)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=prec) as rt:
        if tile:
            rt.set_tile(*tile)
        rt.set_strip_rows(rows)
        rt.upload(0, cons)
        for _ in range(2):
            rt.advance(3)
        s = rt.download(0)[0]
    np.save({outdir!r} + "/" + name + ".npy", s)
print("done")
"""


def run_cases(lib, outdir):
    code = RUNNER.format(pkg=os.path.join(ROOT, "app-binary2d_gb300"), root=ROOT, lib=lib,
                         cases=json.dumps(CASES), outdir=str(outdir))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return {name: np.load(os.path.join(str(outdir), name + ".npy")) for name in CASES}


def test_poisoned_build_reproduces_the_states(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "app-binary2d_gb300"))
    import importlib.util
    spec = importlib.util.spec_from_file_location("b2d_build", os.path.join(ROOT, "app-binary2d_gb300", "build.py"))
    bld = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bld)
    normal, poisoned = bld.build(), bld.build(poison=True)
    (tmp_path / "n").mkdir()
    (tmp_path / "p").mkdir()
    a = run_cases(normal, tmp_path / "n")
    b = run_cases(poisoned, tmp_path / "p")
    for name in CASES:
        assert np.all(np.isfinite(b[name])), name
        assert np.array_equal(a[name], b[name]), name
