"""Throughput benchmark: zone-updates/s of binary2d's RK step on one GB300.

Workload (default): the isothermal circumbinary disk on 16x16 blocks of
128^2 zones (2048^2), q = 1, e = 0, Mach 10, nu = 1e-3, PLM theta = 1.5,
HLLE, RK2, CFL 0.4, synthetic initial state (Sigma = 1 with a cavity r < 2.5a,
Keplerian velocity, seeded +-1e-3 noise).  One bench step is one advance
(src/scheme.rs:323-349) with fold = 10 (setups/iso-circular.yaml:31): one dt,
then 10 RK2 steps; zone-updates per step = 2048^2 x 10.  The state (100 MB)
plus background exceed the 129 MB L2, so no flush is needed between steps.

Arms:
  --impl ours (default)  the CUDA path through the C ABI (libb2d.so)
  --impl reference       the reference's CPU algorithm restated in C (the
                         oracle port), all host threads, one advance of
                         fold 10 RK2 steps of the same mesh per bench step

Under torchrun (N > 1) every rank advances its own disk (independent runs,
weak scaling, no collective in the data path); timing is the max over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "app-binary2d_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

METRIC = "zone-updates/s: mixed-prec+batched vs plain FP64 on 1 GB300 at stated L1 err; %HBM"
UNIT = "zone-updates/s"
FOLD = 10
WORKLOAD_2048 = "iso disk 2048^2 (16x16 blocks of 128^2), q=1 e=0 Mach 10, RK2, fold 10"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def link_bandwidth(torch, host_src, host_dst):
    """Host-to-device and device-to-host copy rates (GB/s) of one page-locked
    state-sized buffer, measured with CUDA events: what bounds the end-to-end
    leg when a step's copies outlast its advance."""
    dev = torch.empty(host_src.nbytes, dtype=torch.uint8, device="cuda")
    src = torch.from_numpy(host_src.view(np.uint8).reshape(-1))
    dst = torch.from_numpy(host_dst.view(np.uint8).reshape(-1))
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    dev.copy_(src, non_blocking=True)
    dst.copy_(dev, non_blocking=True)
    e0.record()
    dev.copy_(src, non_blocking=True)
    e1.record()
    dst.copy_(dev, non_blocking=True)
    e2.record()
    e2.synchronize()
    n = host_src.nbytes / 1e6
    out = {"h2d": n / e0.elapsed_time(e1), "d2h": n / e1.elapsed_time(e2)}
    del dev
    return out


PROFILES = {("disk_2048", "fp32_comp"): "stage3_kernel_fp32comp_disk2048.md",
            ("euler_4096", "fp32_comp"): "stage3e_kernel_fp32comp_euler4096.md"}


def ncu_profile(workload, precision, key):
    """A row (`| key | value |`) of the committed ncu summary of this workload's
    stage kernel, or None."""
    name = PROFILES.get((workload, precision))
    if not name:
        return None
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith("| %s |" % key):
                return line.split("|")[2].strip()
    except OSError:
        return None
    return None


def ncu_traffic(workload, precision):
    """DRAM bytes (read + write) of one stage-kernel launch, or None."""
    v = ncu_profile(workload, precision, "traffic_bytes_per_launch")
    return int(v) if v else None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class NvmlSampler:
    """SM clock, its maximum and the clock-event reasons of one GPU, read from
    NVML (libnvidia-ml, read-only queries) every `period` seconds in a
    thread.  Raises at construction if NVML cannot be used."""
    # nvmlClocksEventReasons bits (nvml.h): SwPowerCap, HwSlowdown, SwThermalSlowdown, HwThermalSlowdown
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, bus_id, period=0.02):
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.lib, self.period = lib, period
        self.handle = ctypes.c_void_p()
        dom, rest = bus_id.split(":", 1)
        for bid in ("%08x:%s" % (int(dom, 16), rest), "%04x:%s" % (int(dom, 16), rest)):
            if lib.nvmlDeviceGetHandleByPciBusId_v2(bid.encode(), ctypes.byref(self.handle)) == 0:
                break
        else:
            raise RuntimeError("no NVML handle for " + bus_id)
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(self.handle, 1, ctypes.byref(mx)) != 0:   # NVML_CLOCK_SM
            raise RuntimeError("nvmlDeviceGetMaxClockInfo failed")
        self.max_mhz = float(mx.value)
        self.samples = []
        self.stop = threading.Event()

    def sample(self):
        mhz, bits = ctypes.c_uint(), ctypes.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(mhz)) == 0 and \
                self.reasons_fn(self.handle, ctypes.byref(bits)) == 0:
            self.samples.append((float(mhz.value), int(bits.value)))

    def run(self):
        while not self.stop.is_set():
            self.sample()
            time.sleep(self.period)

    def close(self):
        self.stop.set()
        self.lib.nvmlShutdown()


class Clocks:
    """Sample the SM clock and the clock-event reasons during the timed region:
    from NVML every 20 ms where libnvidia-ml loads, else from
    nvidia-smi every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.nvml = None
        self.lines = []

    def __enter__(self):
        try:
            import torch
            p = torch.cuda.get_device_properties(self.index)
            self.nvml = NvmlSampler("%x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id))
            self.t = threading.Thread(target=self.nvml.run, daemon=True)
            self.t.start()
            return self
        except Exception:
            self.nvml = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.nvml:
            self.nvml.sample()   # at least one sample at the end of the region
            self.nvml.stop.set()
            self.t.join(timeout=1)
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            smp = self.nvml.samples
            if not smp:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0, "source": "nvml"}
            reasons = sorted(n for n, b in NvmlSampler.BITS.items() if any(bits & b for _, bits in smp))
            return {"sm_mhz": statistics.median(m for m, _ in smp), "sm_max_mhz": self.nvml.max_mhz,
                    "reasons": reasons, "samples": len(smp), "source": "nvml, 20 ms"}
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz),
                "source": "nvidia-smi, 200 ms"}


def cpu_sample(mesh, hydro, physics, model, seconds, nthreads):
    """The oracle port on the host cores: advances of FOLD RK steps of the same
    mesh for about `seconds`; returns (zone-updates/s, RK steps).  The state
    comes from the oracle's own initial model, so this leg loads no product
    library."""
    from oracle import binding
    cons, cfg = binding.disk_initial_state(mesh, hydro, physics, model)
    st = binding.OracleState(cfg, cons)
    st.advance(FOLD, nthreads=nthreads)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        st.advance(FOLD, nthreads=nthreads)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds and n >= 2:
            break
    return mesh.total_zones() * FOLD * n / el, FOLD * n


def reference_arm(args):
    """The reference's algorithm on the host cores (the oracle port, C, FP64,
    one pool task per block and phase like the reference's tokio design,
    2 x cores threads as src/app.rs:125-131 defaults), on the GPU arm's
    workload and cadence: one bench step is one advance of FOLD RK2 steps of
    the 2048^2 disk (setups/iso-circular.yaml:31).  Loads only the oracle."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from binary2d import presets
    from oracle import binding
    mesh, hydro, physics, model = presets.disk_2048(seed=1)
    nthreads = 2 * (os.cpu_count() or 1)   # the reference's default, src/app.rs:125-131
    cons, cfg = binding.disk_initial_state(mesh, hydro, physics, model)
    st = binding.OracleState(cfg, cons)
    for _ in range(args.warmup):
        st.advance(FOLD, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st.advance(FOLD, nthreads=nthreads)
    el = time.perf_counter() - t0
    v = mesh.total_zones() * FOLD * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_2048, "global_batch": 1, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "%d advances of %d RK2 steps of the 2048^2 disk, %d threads on %d host cores"
                                   % (args.steps, FOLD, nthreads, os.cpu_count() or 1)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def ours(args):
    import torch
    import binary2d as b2

    ws, rank, local = dist_env()
    dist = ws > 1
    if dist:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    # libb2d has its own CUDA runtime: select the rank's device there too
    b2.set_device(local if dist else 0)

    if args.workload == "sweep":
        return sweep_bench(args, torch, b2, ws, rank, dist)
    if args.workload == "disk_2048":
        mesh, hydro, physics, model = b2.presets.disk_2048(seed=1 + rank)
        wname = WORKLOAD_2048
    elif args.workload == "disk_512":
        mesh, hydro, physics, model = b2.presets.disk_512(seed=1 + rank)
        wname = "iso disk 512^2 (8x8 blocks of 64^2), q=1 e=0 Mach 10, RK2, fold 10"
    elif args.workload == "disk_1024":
        mesh, hydro, physics, model = b2.presets.iso_disk(8, 128, seed=1 + rank)
        wname = "iso disk 1024^2 (8x8 blocks of 128^2)"
    elif args.workload == "euler_4096":
        mesh, hydro, physics, model = b2.presets.euler_beta_disk(seed=3 + rank)
        wname = ("Euler disk 4096^2 (32x32 blocks of 128^2), gamma 5/3, beta-cooling 10, alpha 0.1, "
                 "q=0.5 e=0.5, RK2, fold 10")
    elif args.workload == "disk_8192":
        mesh, hydro, physics, model = b2.presets.disk_8192(seed=5 + rank)
        wname = "iso disk 8192^2 (64x64 blocks of 128^2), q=1 e=0.1, RK2, fold 10"
        if args.tracers < 0:
            args.tracers = 10_000_000
    else:
        raise SystemExit("unknown workload")
    nf = b2.num_fields(hydro)
    zones = mesh.total_zones()
    cons = b2.initial_state(mesh, hydro, physics, model)
    run = b2.Run(mesh, hydro, physics)
    tracers = b2.presets.annulus_tracers(args.tracers, seed=5 + rank, mesh=mesh) if args.tracers > 0 else None

    tuned = {}

    def make(prec):
        rt = b2.Runtime([run], precision=prec)
        rt.upload(0, cons)
        if tracers is not None:
            rt.set_tracers(0, tracers)
        if args.tile:
            rt.set_tile(*[int(x) for x in args.tile.split("x")])
            rt.set_strip_rows(max(args.strip_rows, 0))
            tuned[prec] = rt.tile() + (rt.strip_rows(),)
        elif prec in tuned:
            rt.set_tile(*tuned[prec][:2])
            rt.set_strip_rows(tuned[prec][2])
        else:
            w, h, _ = rt.autotune(fold=2, reps=2)
            tuned[prec] = (w, h, rt.strip_rows())
        return rt

    def barrier():
        if dist:
            torch.distributed.barrier()

    def timed(rt, steps, warmup):
        stream = torch.cuda.ExternalStream(rt.stream())
        for _ in range(warmup):
            rt.advance_async(FOLD)
        rt.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = rt.launch_count()
        e0.record(stream)
        for _ in range(steps):
            rt.advance_async(FOLD)
        e1.record(stream)
        e1.synchronize()
        rt.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        launches = rt.launch_count() - l0
        if dist:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        barrier()
        return ms, launches

    prec = args.precision
    w = 8  # stored bytes per conserved word (FP64, or FP32 + FP32 compensation)
    # RK2: stage 1 reads U and U_bg and writes U1; stage 2 reads U1, U and U_bg and
    # writes U2: 7 accesses of nf words of w bytes per zone-update
    bytes_per_zone_update = 7 * nf * w
    hbm_peak, peak_kind = peaks()

    rt = make(prec)
    with Clocks(local) as clk:
        ms, launches = timed(rt, args.steps, args.warmup)
    value = zones * FOLD * args.steps / (ms / 1e3) * ws

    # dominant kernel: the stage kernels' share of an advance, from a pass with
    # CUDA events around every stage launch (graph replay bypassed) and around
    # each whole advance, applied to the graph-timed step, so that the stages
    # of a step never add up to more than the step
    rt.set_instrument(True)
    stream = torch.cuda.ExternalStream(rt.stream())
    adv_ms = 0.0
    for _ in range(max(2, args.steps // 4)):
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        rt.advance(FOLD)
        a1.record(stream)
        a1.synchronize()
        adv_ms += a0.elapsed_time(a1)
    nst, st_ms = rt.stage_stats()
    rt.set_instrument(False)
    stages_per_step = nst / max(2, args.steps // 4)
    stage_share = min(st_ms / adv_ms, 1.0) if adv_ms > 0 else 1.0
    stage_ms = (ms / args.steps) * stage_share / max(stages_per_step, 1)
    stage_ms_events = st_ms / max(nst, 1)
    bytes_per_launch = bytes_per_zone_update / 2.0 * zones      # average of the two RK2 stages
    achieved = bytes_per_launch / (stage_ms / 1e3) / 1e9
    rt.close()

    # end to end through the C ABI with page-locked host buffers: every step
    # uploads its input state, advances and downloads its result, pipelined
    # (the copies of one step overlap the neighbouring steps' advances; the
    # wait at the end of a step lets only the newest download stay in flight)
    host_in = [np.ascontiguousarray(cons.copy()) for _ in range(2)]
    host_out = [np.empty_like(cons) for _ in range(2)]
    for a in host_in + host_out:
        b2.pin(a)
    copy_gbs = link_bandwidth(torch, host_in[0], host_out[0])
    rt = make(prec)

    def e2e_step(k):
        rt.upload_conserved_async(0, host_in[k & 1])
        rt.advance_async(FOLD)
        rt.download_async(0, host_out[k & 1])
        rt.transfers_wait(1)

    # warm-up: enough steps for every start slot's CUDA graph to be captured
    # (the advance's start slot cycles through the four state slots)
    for k in range(max(4, args.warmup)):
        e2e_step(k)
    rt.transfers_wait(0)
    rt.synchronize()
    barrier()
    # three trials of the timed loop; the reported figure is the median trial.
    # The host link of these GPUs is shared with other tenants of the machine:
    # a trial's copies can run at a fraction of the link rate while the
    # advance on the device does not change, so one trial alone may be an
    # outlier (every trial is listed in the JSON line)
    e2e_steps = max(4, args.steps // 2)
    trials = []
    for _ in range(3):
        barrier()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            e2e_step(k)
        rt.transfers_wait(0)
        rt.synchronize()
        el = time.perf_counter() - t0
        if dist:
            t = torch.tensor([el], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        trials.append(zones * FOLD * e2e_steps / el * ws)
    e2e_value = statistics.median(trials)
    copy_gbs_after = link_bandwidth(torch, host_in[0], host_out[0])
    rt.close()
    for a in host_in + host_out:
        b2.unpin(a)

    # plain FP64 on the same workload (shorter)
    fp64_value = None
    if prec != "fp64" and not args.skip_fp64:
        rt64 = make("fp64")
        ms64, _ = timed(rt64, max(2, args.steps // 5), 2)
        fp64_value = zones * FOLD * max(2, args.steps // 5) / (ms64 / 1e3) * ws
        rt64.close()

    # accuracy of the mixed path against the FP64 path (512^2 disk, 1/4 orbit)
    accuracy = None
    if prec != "fp64" and not args.skip_accuracy and rank == 0:
        accuracy = accuracy_check(prec, orbits=args.accuracy_orbits)

    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        nthreads = 2 * (os.cpu_count() or 1)
        v, n = cpu_sample(mesh, hydro, physics, model, args.cpu_seconds, nthreads)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": "%d RK2 steps (advances of %d) of the same %d^2 mesh with the C oracle, %d threads on %d host cores"
                         % (n, FOLD, mesh.zones_per_side(), nthreads, os.cpu_count() or 1)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "fp32_state64": "f32 (f64 state)",
                                                             "fp32_comp": "f32 (compensated f32 state)"}[prec],
            "data": "synthetic",
            "config": {"workload": wname, "precision": prec, "zones": zones, "fold": FOLD,
                       "tracers": int(args.tracers) if tracers is not None else 0,
                       "tracer_bytes_per_step": (2 * 32 * FOLD * int(args.tracers)) if tracers is not None else 0,
                       "global_batch": ws, "parallelism": "replicas" if ws > 1 else "single GPU",
                       "l2": "state + background > L2 (no flush needed)",
                       "tile": "%dx%d" % tuned.get(prec, (0, 0, 0))[:2],
                       "strip_rows": tuned.get(prec, (0, 0, 0))[2],
                       "tile_source": "autotuner" if not args.tile else "--tile"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                         "traffic": ncu_traffic(args.workload, prec),
                         "traffic_note": ("mean DRAM bytes of the two RK2 stage launches of one step "
                                          "(algorithmic mean %.0f MB) from profiles/%s"
                                          % (bytes_per_launch / 1e6, PROFILES.get((args.workload, prec))))
                                         if ncu_traffic(args.workload, prec) else "no ncu capture of this workload",
                         "algorithmic_bytes_per_launch": bytes_per_launch,
                         "bytes_per_zone_update": bytes_per_zone_update, "stage_ms": stage_ms,
                         "stage_ms_note": ("graph-timed step x the stage kernels' share of an event-timed "
                                           "advance (%.1f %%) / %d stages; per-launch events alone: %.4f ms"
                                           % (100 * stage_share, round(stages_per_step), stage_ms_events)),
                         "limiter": ncu_profile(args.workload, prec, "limiter")
                                    or "instruction issue (no ncu capture of this workload)"},
            "fp64": {"value": fp64_value, "ratio": (value / fp64_value) if fp64_value else None},
            "accuracy": accuracy,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(cons.nbytes),
                    "d2h_bytes_per_step": int(cons.nbytes), "trials": trials, "steps_per_trial": e2e_steps,
                    "statistic": "median of the trials", "link_gbs": copy_gbs, "link_gbs_after": copy_gbs_after},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if dist:
        torch.distributed.destroy_process_group()
    return 0


def sweep_bench(args, torch, b2, ws, rank, dist):
    """Batched parameter sweep: 64 independent isothermal runs of uneven sides
    (256..1024 zones in 64^2 blocks; q, e, Mach, nu drawn by seed).  All runs
    of this rank advance in one context: one launch per RK stage for every
    run, the advance replayed as a CUDA graph.  Compared with the same runs
    advanced one context at a time.  Runs are dealt whole to ranks."""
    from binary2d.distributed import deal_runs, max_over_ranks
    cases = b2.presets.sweep(nruns=args.sweep_runs, seed=4)
    mine = deal_runs([c[0].total_zones() for c in cases], ws, rank)
    cases = [cases[k] for k in mine]
    runs = [b2.Run(m, h, p) for (m, h, p, _) in cases]
    inits = [b2.initial_state(m, h, p, md, run=mine[k]) for k, (m, h, p, md) in enumerate(cases)]
    zones = sum(r.mesh.total_zones() for r in runs)
    prec = args.precision

    rt = b2.Runtime(runs, precision=prec)
    for k, c in enumerate(inits):
        rt.upload(k, c)
    tile = rt.autotune(fold=2, reps=1)[:2]
    strip_rows = rt.strip_rows()
    stream = torch.cuda.ExternalStream(rt.stream())
    for _ in range(args.warmup):
        rt.advance_async(FOLD)
    rt.synchronize()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = rt.launch_count()
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            rt.advance_async(FOLD)
        e1.record(stream)
        e1.synchronize()
    rt.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), device="cuda" if dist else None)
    launches = rt.launch_count() - l0
    rt.set_instrument(True)
    for _ in range(2):
        rt.advance(FOLD)
    nst, st_ms = rt.stage_stats()
    rt.close()
    total_zones = zones * ws if not dist else None
    value = (zones * FOLD * args.steps / (ms / 1e3))
    if dist:
        from binary2d.distributed import sum_over_ranks
        value = sum_over_ranks(value, device="cuda")

    # the same runs one context at a time
    single_ms = 0.0
    nsteps = max(2, args.steps // 4)
    for r, c in zip(runs, inits):
        one = b2.Runtime([r], precision=prec)
        one.upload(0, c)
        one.set_tile(*tile)
        one.set_strip_rows(strip_rows)
        one.advance(FOLD)
        s = torch.cuda.ExternalStream(one.stream())
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(s)
        for _ in range(nsteps):
            one.advance(FOLD)          # a host loop of single runs, each advance synchronised
        a1.record(s)
        a1.synchronize()
        single_ms += a0.elapsed_time(a1) / nsteps * args.steps
        one.close()
    single_value = zones * FOLD * args.steps / (single_ms / 1e3)
    hbm_peak, peak_kind = peaks()
    stage_ms = st_ms / max(nst, 1)
    achieved = 7 * 3 * 8 / 2.0 * zones / (stage_ms / 1e3) / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"fp64": "f64", "fp32_state64": "f32 (f64 state)",
                                           "fp32_comp": "f32 (compensated f32 state)"}[prec],
            "data": "synthetic",
            "config": {"workload": "batched sweep: %d isothermal runs, sides 256-1024 in 64^2 blocks, fold 10"
                                   % args.sweep_runs, "runs_on_rank0": len(runs), "zones_rank0": zones,
                       "tile": "%dx%d" % tuple(tile), "strip_rows": strip_rows, "parallelism": "runs dealt to ranks" if dist else "single GPU"},
            "batched": {"value": value, "one_at_a_time": single_value, "ratio": value / single_value},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": None, "stage_ms": stage_ms},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        }))
    if dist:
        torch.distributed.destroy_process_group()
    return 0


def accuracy_check(prec, orbits):
    """Relative L1 error of Sigma and of the accreted mass (sink ledger) of the
    mixed path against the FP64 path on the 512^2 disk after `orbits` orbits
    (the FP64 run sets the number of advances)."""
    import binary2d as b2
    mesh, hydro, physics, model = b2.presets.disk_512(seed=1)
    cons = b2.initial_state(mesh, hydro, physics, model)
    out = {}
    advances = None
    for p in ("fp64", prec):
        with b2.Runtime([b2.Run(mesh, hydro, physics)], precision=p) as rt:
            rt.upload(0, cons)
            n = 0
            while (advances is None and rt.time(0)[0] < orbits * 2 * np.pi) or (advances is not None and n < advances):
                rt.advance(FOLD)
                n += 1
            advances = n
            s, t, _ = rt.download(0)
            led = rt.ledger(0)
        out[p] = (s, led, t)
    s64, led64, t64 = out["fp64"]
    s32, led32, _ = out[prec]
    l1 = float(np.abs(s32[..., 0] - s64[..., 0]).sum() / np.abs(s64[..., 0]).sum())
    acc64 = led64[:, :, 0:2, 0].sum()
    acc32 = led32[:, :, 0:2, 0].sum()
    return {"workload": "iso disk 512^2", "steps": advances * FOLD, "orbits": t64 / (2 * np.pi),
            "l1_sigma_rel": l1, "accreted_mass_rel": float(abs(acc32 - acc64) / abs(acc64)) if acc64 else None,
            "reference": "FP64 GPU path (matches the CPU oracle to 1e-12)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32_comp", choices=["fp64", "fp32_state64", "fp32_comp"])
    ap.add_argument("--workload", default="disk_2048")
    ap.add_argument("--tile", default="", help="WxH: fixed tile instead of the autotuner")
    ap.add_argument("--strip-rows", type=int, default=0,
                    help="with --tile: row chunks across block rows for the paired FP32 kernel (0: off)")
    ap.add_argument("--sweep-runs", type=int, default=64)
    ap.add_argument("--tracers", type=int, default=-1, help="tracer particles (-1: workload default)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--accuracy-orbits", type=float, default=1.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
