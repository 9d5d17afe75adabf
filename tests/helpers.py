"""Shared helpers of the parity tests: build a case, run it on the GPU
through the C ABI and on the oracle, compare."""
import copy

import numpy as np

import binary2d as b2
from oracle import binding


def make_case(mesh, hydro, physics, model, run=0):
    cons = b2.initial_state(mesh, hydro, physics, model, run=run)
    cfg = b2.to_c(mesh, hydro, physics)
    return cons, cfg


def rel_err(a, b):
    """Max-norm error per field, relative to the field's max magnitude."""
    nf = a.shape[-1]
    a2 = a.reshape(-1, nf)
    b2_ = b.reshape(-1, nf)
    scale = np.maximum(np.abs(b2_).max(axis=0), 1e-300)
    return (np.abs(a2 - b2_).max(axis=0) / scale).max()


def run_pair(mesh, hydro, physics, model, fold, advances, precision="fp64", tile=None, graphs=True,
             background=None, nthreads=None, strip_rows=0):
    """Advance the same initial state on the GPU and on the oracle."""
    cons, cfg = make_case(mesh, hydro, physics, model)
    ref = binding.OracleState(cfg, cons, background=background)
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=precision) as rt:
        if tile:
            rt.set_tile(*tile)
        if strip_rows:
            rt.set_strip_rows(strip_rows)
        rt.set_graphs(graphs)
        rt.upload(0, cons, background=background)
        dts, dts_ref = [], []
        for _ in range(advances):
            dts.append(rt.advance(fold)[0])
            dts_ref.append(ref.advance(fold, nthreads=nthreads))
        out, t, it = rt.download(0)
        led = rt.ledger(0)
    return dict(gpu=out, ref=ref.cons, t=t, t_ref=ref.time.value, it=it, it_ref=ref.iteration.value,
                dt=np.array(dts), dt_ref=np.array(dts_ref), led=led, led_ref=ref.ledger, cons0=cons)


def ledger_err(led, led_ref):
    """Ledger sums are accumulated in a different order on the GPU: compare
    against the magnitude of each item."""
    scale = np.maximum(np.abs(led_ref).sum(axis=(0, 1)), 1e-300)
    return (np.abs(led - led_ref).sum(axis=(0, 1)) / scale).max()
