"""One-orbit accuracy of the three precisions against the CPU oracle, on the
isothermal disk of 16 x 16 blocks of 128² or the Euler β-cooling disk (at a
resolution the oracle can afford), and FP32 against FP64 on the GPU alone
where the oracle cannot follow (the 8192² disk).

Two steps, because the oracle's orbit costs up to 8e10 zone-updates:

    python tests/orbit_accuracy.py oracle --out tests/_cache/orbit2048.npz [--threads N]
    python tests/orbit_accuracy.py gpu --cache tests/_cache/orbit2048.npz [--json OUT]
    (--workload euler --side 512 --fold 1 for the Euler disk, whose dt falls by
    3.6x in its first steps: one dt for ten of them breaks the CFL condition)
    python tests/orbit_accuracy.py compare --workload disk_8192 --steps 1000 [--json OUT]
    python tests/orbit_accuracy.py orbit --workload euler --side 4096 [--json OUT]

The first runs the oracle for one orbit (fold 10 advances until t >= 2π) and
caches Σ at the end and the time series of the domain totals of the
ItemizedChange ledger (state.rs:27-62) and of the orbital-element ledger
after every advance (TimeSeriesSample, app.rs:141-148).  The second runs the
same number of advances on the GPU in every precision and reports the
relative L1 error of Σ and the error of each ledger series against the
cached oracle run.  The cache is a regenerable test artefact and is not
committed.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "app-binary2d_gb300"))
sys.path.insert(0, ROOT)

FOLD = 10
ITEMS = ("sink1", "sink2", "grav1", "grav2", "buffer", "cooling", "fake_mass")


def _case(side, workload="disk"):
    import binary2d as b2
    if workload == "euler":
        # the workload's 128^2 blocks at full size (32 x 32 at 4096^2), 64^2 blocks at the oracle's sizes
        nb, bs = (side // 128, 128) if side >= 1024 else (side // 64, 64)
        mesh, hydro, physics, model = b2.presets.euler_beta_disk(nb, bs)
    elif workload == "disk_8192":
        mesh, hydro, physics, model = b2.presets.disk_8192()[:4]
    elif side == 2048:
        mesh, hydro, physics, model = b2.presets.disk_2048(seed=1)
    else:
        mesh, hydro, physics, model = b2.presets.iso_disk(side // 64, 64, seed=1)
    cons = b2.initial_state(mesh, hydro, physics, model)
    return mesh, hydro, physics, cons


def run_oracle(args):
    import binary2d as b2
    from oracle import binding
    mesh, hydro, physics, cons = _case(args.side, args.workload)
    st = binding.OracleState(b2.to_c(mesh, hydro, physics), cons)
    t_end = args.orbits * 2 * np.pi
    times, led, el, dts = [], [], [], []
    t0 = time.time()
    while st.time.value < t_end:
        dts.append(st.advance(args.fold, nthreads=args.threads))
        times.append(st.time.value)
        led.append(st.ledger.sum(axis=(0, 1)))
        el.append(st.elements.sum(axis=(0, 1)))
        if len(times) % 50 == 0:
            print("advance %d t=%.4f (%.0f s)" % (len(times), st.time.value, time.time() - t0), flush=True)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.savez(args.out, sigma=st.cons[..., 0], times=np.array(times), ledger=np.array(led),
             elements=np.array(el), dts=np.array(dts), side=args.side, orbits=args.orbits,
             seconds=time.time() - t0, workload=args.workload, fold=args.fold)
    print("wrote %s: %d advances, t=%.6f, %.0f s" % (args.out, len(times), st.time.value, time.time() - t0))


def run_gpu(args):
    import binary2d as b2
    ref = np.load(args.cache)
    side = int(ref["side"])
    workload = str(ref["workload"]) if "workload" in ref.files else "disk"
    mesh, hydro, physics, cons = _case(side, workload)
    n = len(ref["times"])
    fold = int(ref["fold"]) if "fold" in ref.files else FOLD
    sig_ref = ref["sigma"]
    out = {"workload": "%s %d^2, one orbit" % ("Euler beta-cooling disk" if workload == "euler" else "iso disk", side),
           "advances": n, "steps": n * fold,
           "orbits": float(ref["times"][-1] / (2 * np.pi)),
           "oracle_seconds": float(ref["seconds"]), "precisions": {}}
    for p in ("fp64", "fp32_state64", "fp32_comp"):
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=p) as rt:
            rt.autotune()
            rt.upload(0, cons)
            times, led, el = [], [], []
            t0 = time.time()
            for _ in range(n):
                rt.advance(fold)
                times.append(rt.time(0)[0])
                led.append(rt.ledger(0).sum(axis=(0, 1)))
                el.append(rt.elements(0).sum(axis=(0, 1)))
            secs = time.time() - t0
            s, t, _ = rt.download(0)
        led, el = np.array(led), np.array(el)
        l1 = float(np.abs(s[..., 0] - sig_ref).sum() / np.abs(sig_ref).sum())
        # per item: max over the series and fields of |gpu - oracle|, divided by the
        # item's largest |oracle| over the series and fields (a field that is zero up
        # to rounding, such as cooling's momentum, is judged against its item)
        scale = np.maximum(np.abs(ref["ledger"]).max(axis=(0, 2)), 1e-300)[:, None]
        led_err = (np.abs(led - ref["ledger"]).max(axis=0) / scale)
        escale = np.maximum(np.abs(ref["elements"]).max(axis=(0, 2)), 1e-300)[:, None]
        el_err = (np.abs(el - ref["elements"]).max(axis=0) / escale)
        acc = ref["ledger"][-1, 0:2, 0].sum()
        out["precisions"][p] = {
            "l1_sigma_rel": l1,
            "end_time_rel": float(abs(t - ref["times"][-1]) / ref["times"][-1]),
            "accreted_mass_rel": float(abs(led[-1, 0:2, 0].sum() - acc) / abs(acc)),
            "ledger_series_rel": {ITEMS[k]: float(led_err[k].max()) for k in range(7) if np.abs(ref["ledger"][:, k]).max() > 0},
            "elements_series_rel": {ITEMS[k]: float(el_err[k].max()) for k in range(4)},
            "seconds_with_host_sampling": secs,
        }
        print(p, json.dumps(out["precisions"][p]), flush=True)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out))


def run_compare(args):
    """FP32 paths against the FP64 GPU path after a fixed number of steps."""
    import binary2d as b2
    mesh, hydro, physics, cons = _case(0, args.workload)
    n = args.steps // FOLD
    res = {}
    for p in ("fp64", "fp32_comp"):
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=p) as rt:
            rt.upload(0, cons)
            if p != "fp64":
                rt.autotune()   # on the uploaded state; the trial advances are discarded
            t0 = time.time()
            for _ in range(n):
                rt.advance(FOLD)
            s, t, _ = rt.download(0)
            res[p] = (s[..., 0].copy(), rt.ledger(0).sum(axis=(0, 1)), t, time.time() - t0)
        print(p, "done in %.1f s" % res[p][3], flush=True)
    s64, l64, t64, _ = res["fp64"]
    s32, l32, t32, _ = res["fp32_comp"]
    acc64, acc32 = l64[0:2, 0].sum(), l32[0:2, 0].sum()
    out = {"workload": args.workload, "steps": n * FOLD, "time_fp64": t64, "end_time_rel": abs(t32 - t64) / t64,
           "l1_sigma_rel": float(np.abs(s32 - s64).sum() / np.abs(s64).sum()),
           "accreted_mass_rel": float(abs(acc32 - acc64) / abs(acc64)) if acc64 else None,
           "seconds": {"fp64": res["fp64"][3], "fp32_comp": res["fp32_comp"][3]}}
    if args.json:
        with open(args.json, "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out))


def run_orbit(args):
    """One orbit of the FP32 path alone on the full-size workload (the Euler
    beta-cooling disk at 4096^2: the oracle cannot follow it), with the run's
    end state: time reached, hydro status, finiteness, accreted mass."""
    import dataclasses
    import binary2d as b2
    mesh, hydro, physics, cons = _case(args.side, args.workload)
    # open parameters changed from the preset: --physics key=value, --model key=value
    def parse(items):
        out = {}
        for kv in items:
            k, v = kv.split("=", 1)
            out[k] = None if v == "none" else float(v)
        return out
    if args.physics or args.model:
        nb, bs = (args.side // 128, 128) if args.side >= 1024 else (args.side // 64, 64)
        mesh, hydro, physics, model = b2.presets.euler_beta_disk(nb, bs) if args.workload == "euler" else \
            b2.presets.iso_disk(nb, bs, seed=1)
        physics = dataclasses.replace(physics, **parse(args.physics))
        model = dataclasses.replace(model, **parse(args.model))
        cons = b2.initial_state(mesh, hydro, physics, model)
    t0 = time.time()
    status = "ok"
    with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=args.precision) as rt:
        rt.upload(0, cons)
        tile = rt.autotune()   # on the uploaded state; the trial advances are discarded
        rows = rt.strip_rows()
        n = 0
        try:
            while rt.time(0)[0] < args.orbits * 2 * np.pi:
                rt.advance(args.fold)
                n += 1
        except b2.HydroError as e:
            status = "%s at t=%.5f, block %s" % (e.kind, e.time, e.block)
        t, it = rt.time(0)
        s = rt.download(0)[0]
        led = rt.ledger(0)
    out = {"workload": "%s %d^2" % (args.workload, args.side), "changed": {"physics": args.physics, "model": args.model},
           "precision": args.precision, "fold": args.fold,
           "cfl": physics.cfl, "advances": n, "steps": it, "t_end": t, "orbits": t / (2 * np.pi), "status": status,
           "seconds": time.time() - t0, "tile": [tile[0], tile[1]], "strip_rows": rows,
           "state_finite": bool(np.isfinite(s).all()), "sigma_min": float(s[..., 0].min()),
           "sigma_max": float(s[..., 0].max()), "accreted_mass": float(-led[:, :, 0:2, 0].sum())}
    if args.json:
        with open(args.json, "w") as f:
            json.dump(out, f, indent=1)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    o = sub.add_parser("oracle")
    o.add_argument("--out", required=True)
    o.add_argument("--side", type=int, default=2048)
    o.add_argument("--orbits", type=float, default=1.0)
    o.add_argument("--threads", type=int, default=None)
    o.add_argument("--workload", default="disk", choices=["disk", "euler"])
    o.add_argument("--fold", type=int, default=FOLD, help="RK steps per advance (one dt per advance)")
    g = sub.add_parser("gpu")
    g.add_argument("--cache", required=True)
    g.add_argument("--json", default="")
    c = sub.add_parser("compare")
    c.add_argument("--workload", default="disk_8192", choices=["disk_8192"])
    c.add_argument("--steps", type=int, default=1000)
    c.add_argument("--json", default="")
    r = sub.add_parser("orbit")
    r.add_argument("--workload", default="euler", choices=["euler", "disk"])
    r.add_argument("--side", type=int, default=4096)
    r.add_argument("--orbits", type=float, default=1.0)
    r.add_argument("--fold", type=int, default=FOLD)
    r.add_argument("--precision", default="fp32_comp", choices=["fp64", "fp32_state64", "fp32_comp"])
    r.add_argument("--physics", nargs="*", default=[], help="Physics fields to change, key=value")
    r.add_argument("--model", nargs="*", default=[], help="DiskModel fields to change, key=value")
    r.add_argument("--json", default="")
    args = ap.parse_args()
    {"oracle": run_oracle, "gpu": run_gpu, "compare": run_compare, "orbit": run_orbit}[args.cmd](args)


if __name__ == "__main__":
    main()
