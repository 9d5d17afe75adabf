"""The application around the step: configuration, presets, the driver loop
and checkpoints — the host side of src/app.rs, src/main.rs, src/tasks.rs and
src/io.rs, driving the GB300 step through the C ABI.

* Configuration (app.rs:169-177) from YAML text or files, a preset name
  (app.rs:318-325, 354-360), and overrides `group.key=value` or extra `.yaml`
  files (app.rs:246-255), with deny_unknown_fields where the reference has it.
* run() is main.rs:run (main.rs:99-210): `fold` steps per advance, side
  effects after each (iteration message with Mzps, time series samples,
  progress, checkpoints; main.rs:27-86), a fallback stack with rewind and
  safe mode on a hydro error (main.rs:125-205), chkpt.fail.cbor when there is
  nothing to rewind to.
* Checkpoints are the App (app.rs:185-192) in CBOR with serde's layout
  (io.rs:7-18); restarting from one rebuilds BlockData from the model
  (main.rs:119-122).
"""
import copy
import dataclasses
import math
import os
import time as _time
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional

import numpy as np

from . import cbor, yaml_lite
from .config import ORBITAL_PERIOD, DiskModel, Euler, Isothermal, Mesh, Physics, num_fields
from .presets import REFERENCE_PRESETS
from .scheme import HydroError, Run, Runtime, initial_state

VERSION = "binary2d-gb300 0.1 (reference v0.2.1)"


class ConfigError(ValueError):
    pass


# ----------------------------------------------------------------------------
# Configuration

@dataclass
class Control:
    """Control (app.rs:94-131)."""
    num_orbits: float
    checkpoint_interval: float
    fold: int
    output_directory: str
    time_series_interval: Optional[float] = None
    num_threads: Optional[int] = None
    fallback_stack_size: int = 0

    def num_threads_or_default(self) -> int:      # app.rs:125-131
        return self.num_threads if self.num_threads is not None else 2 * (os.cpu_count() or 1)


@dataclass
class Configuration:
    hydro: Any
    model: DiskModel
    mesh: Mesh
    physics: Physics
    control: Control


_PHYSICS_FIELDS = {f.name for f in dataclasses.fields(Physics)} - {"lambda_"} | {"lambda"}
_ISO_FIELDS = {"mach_number", "density_floor"}
_EULER_FIELDS = {"gamma_law_index", "cooling_coefficient", "pressure_floor", "density_floor", "density_index",
                 "cooling_slow_start", "cooling_beta"}
_MODEL_FIELDS = {
    "infinite_disk": {"mach_number", "surface_density"},
    "infinite_alpha_disk": {"mach_number", "surface_density"},
    "finite_disk": {"disk_mass", "disk_width", "disk_radius", "softening_length", "mach_number"},
    "residual_test": set(),
}


def _deny_unknown(d: dict, allowed, where: str):
    extra = set(d) - set(allowed)
    if extra:
        raise ConfigError("unknown field(s) %s in %s" % (sorted(extra), where))


def _single_variant(d, where, variants):
    if not isinstance(d, dict) or len(d) != 1:
        raise ConfigError("%s must name exactly one variant of %s" % (where, sorted(variants)))
    (k, v), = d.items()
    if k not in variants:
        raise ConfigError("unknown variant %r of %s" % (k, where))
    return k, v or {}


def config_from_dict(d: dict) -> Configuration:
    """serde's Configuration (app.rs:169-177) from a parsed YAML mapping."""
    _deny_unknown(d, {"hydro", "model", "mesh", "physics", "control"}, "configuration")
    for k in ("hydro", "model", "mesh", "physics", "control"):
        if k not in d:
            raise ConfigError("missing field %r" % k)
    hk, hv = _single_variant(d["hydro"], "hydro", {"isothermal", "euler"})
    if hk == "isothermal":
        _deny_unknown(hv, _ISO_FIELDS, "hydro.isothermal")
        hydro = Isothermal(mach_number=float(hv["mach_number"]), density_floor=hv.get("density_floor"))
    else:
        _deny_unknown(hv, _EULER_FIELDS, "hydro.euler")
        hydro = Euler(gamma_law_index=float(hv["gamma_law_index"]),
                      cooling_coefficient=float(hv.get("cooling_coefficient", 0.0)),
                      pressure_floor=hv.get("pressure_floor"), density_floor=hv.get("density_floor"),
                      density_index=int(hv.get("density_index", 2)),
                      cooling_slow_start=bool(hv.get("cooling_slow_start", False)),
                      cooling_beta=hv.get("cooling_beta"))
    mk, mv = _single_variant(d["model"], "model", set(_MODEL_FIELDS))
    _deny_unknown(mv, _MODEL_FIELDS[mk], "model." + mk)
    model = DiskModel(kind=mk, surface_density=float(mv.get("surface_density") or 1.0),
                      mach_number=mv.get("mach_number"), disk_mass=float(mv.get("disk_mass", 0.0)),
                      disk_width=float(mv.get("disk_width", 1.0)), disk_radius=float(mv.get("disk_radius", 1.0)),
                      softening_length=float(mv.get("softening_length", 0.0)))
    # InitialModel::validate (disks.rs:159-169): a Mach number in hydro or model, not both
    hydro_mach = isinstance(hydro, Isothermal)
    if mk in ("infinite_disk", "infinite_alpha_disk", "finite_disk"):
        if hydro_mach and model.mach_number is not None:
            raise ConfigError("A Mach number must be specified either in hydro or model (not both)")
        if not hydro_mach and model.mach_number is None:
            raise ConfigError("A Mach number must be specified either in hydro or model")
    m = d["mesh"]
    _deny_unknown(m, {"num_blocks", "block_size", "domain_radius"}, "mesh")
    mesh = Mesh(num_blocks=int(m["num_blocks"]), block_size=int(m["block_size"]),
                domain_radius=float(m["domain_radius"]))
    p = dict(d["physics"])
    _deny_unknown(p, _PHYSICS_FIELDS, "physics")
    if "lambda" in p:
        p["lambda_"] = p.pop("lambda")
    if "viscosity" in p:
        vk, vv = _single_variant(p["viscosity"], "physics.viscosity", {"constant_nu", "alpha"})
        p["viscosity"] = (vk, float(vv))
    for k in ("rk_order", "safe_rk_order"):
        if p.get(k) is not None and p[k] not in ("RK1", "RK2", "RK3"):
            raise ConfigError("rk_order must be RK1, RK2 or RK3")
    for req in ("buffer_rate", "buffer_scale", "binary_eccentricity", "binary_mass_ratio", "cfl", "plm",
                "rk_order", "sink_radius", "sink_rate"):
        if req not in p:
            raise ConfigError("missing field physics.%s" % req)
    physics = Physics(**p)
    c = d["control"]
    control = Control(num_orbits=float(c["num_orbits"]), checkpoint_interval=float(c["checkpoint_interval"]),
                      fold=int(c["fold"]), output_directory=str(c["output_directory"]),
                      time_series_interval=c.get("time_series_interval"), num_threads=c.get("num_threads"),
                      fallback_stack_size=int(c.get("fallback_stack_size") or 0))
    return Configuration(hydro=hydro, model=model, mesh=mesh, physics=physics, control=control)


def config_to_dict(cfg: Configuration) -> dict:
    """The serde layout of Configuration (field names as in the reference)."""
    h = cfg.hydro
    if isinstance(h, Isothermal):
        hydro = {"isothermal": {"mach_number": h.mach_number, "density_floor": h.density_floor}}
    else:
        hydro = {"euler": {"gamma_law_index": h.gamma_law_index, "cooling_coefficient": h.cooling_coefficient,
                           "pressure_floor": h.pressure_floor, "density_floor": h.density_floor,
                           "density_index": h.density_index, "cooling_slow_start": h.cooling_slow_start}}
        if h.cooling_beta is not None:
            hydro["euler"]["cooling_beta"] = h.cooling_beta
    m = cfg.model
    if m.kind == "finite_disk":
        mv = {"disk_mass": m.disk_mass, "disk_width": m.disk_width, "disk_radius": m.disk_radius,
              "softening_length": m.softening_length, "mach_number": m.mach_number}
    elif m.kind == "residual_test":
        mv = {}
    else:
        mv = {"mach_number": m.mach_number, "surface_density": m.surface_density}
    ph = dataclasses.asdict(cfg.physics)
    ph["lambda"] = ph.pop("lambda_")
    kind, val = cfg.physics.viscosity
    ph["viscosity"] = {kind: val}
    ctl = dataclasses.asdict(cfg.control)
    return {"hydro": hydro, "model": {m.kind: mv}, "mesh": dataclasses.asdict(cfg.mesh), "physics": ph,
            "control": ctl}


def _merge(base: dict, patch: dict):
    for k, v in patch.items():
        if isinstance(v, dict) and isinstance(base.get(k), dict):
            _merge(base[k], v)
        else:
            base[k] = copy.deepcopy(v)


def patch_dict(d: dict, overrides: List[str]) -> dict:
    """Configuration::patch_from (app.rs:246-255): `.yaml` files are merged,
    other arguments are `group.key=value` with a YAML scalar value."""
    for o in overrides:
        if o.endswith(".yaml"):
            with open(o) as f:
                _merge(d, yaml_lite.loads(f.read()))
        else:
            if "=" not in o:
                raise ConfigError("override %r is not key=value" % o)
            path, value = o.split("=", 1)
            keys = path.strip().split(".")
            node = d
            for k in keys[:-1]:
                if not isinstance(node.get(k), dict):
                    node[k] = {}
                node = node[k]
            node[keys[-1]] = yaml_lite.parse_scalar(value)
    return d


def preset_dict(name: str) -> dict:
    """The compiled-in presets of App::presets (app.rs:354-360) as mappings."""
    p = REFERENCE_PRESETS[name]
    cfg = Configuration(hydro=p["hydro"], model=DiskModel(kind=p["model"][0], **{
        k: v for k, v in p["model"][1].items() if v is not None or k == "mach_number"}),
        mesh=p["mesh"], physics=p["physics"], control=Control(**p["control"]))
    return config_to_dict(cfg)


def presets() -> List[str]:
    return list(REFERENCE_PRESETS)


# ----------------------------------------------------------------------------
# Recurring tasks (src/tasks.rs)

@dataclass
class RecurringTask:
    count: int = 0
    next_time: float = 0.0
    last_performed: float = field(default_factory=_time.perf_counter)
    count_this_run: int = 0

    def advance(self, interval: float) -> float:
        """Mark performed; schedule the next time; return the wall seconds since
        the last time it was performed."""
        now = _time.perf_counter()
        elapsed = now - self.last_performed
        self.last_performed = now
        self.count += 1
        self.count_this_run += 1
        self.next_time += interval
        return elapsed

    def elapsed_hours(self) -> float:
        return (_time.perf_counter() - self.last_performed) / 3600.0


@dataclass
class Tasks:
    write_checkpoint: RecurringTask = field(default_factory=RecurringTask)
    iteration_message: RecurringTask = field(default_factory=RecurringTask)
    record_time_series: RecurringTask = field(default_factory=RecurringTask)
    report_progress: RecurringTask = field(default_factory=RecurringTask)
    simulation_startup: RecurringTask = field(default_factory=RecurringTask)

    def to_serde(self) -> dict:
        return {k: {"count": v.count, "next_time": v.next_time} for k, v in self.__dict__.items()}

    @staticmethod
    def from_serde(d: dict) -> "Tasks":
        t = Tasks()
        for k, v in d.items():
            setattr(t, k, RecurringTask(count=int(v["count"]), next_time=float(v["next_time"])))
        return t


# ----------------------------------------------------------------------------
# App state

ITEM_NAMES = ("sink1", "sink2", "grav1", "grav2", "buffer", "cooling", "fake_mass")


@dataclass
class AppState:
    cons: np.ndarray                       # [nb, nb, bs, bs, nf]
    ledger: np.ndarray                     # [nb, nb, 7, nf]
    time: float
    iteration: int
    elements: Optional[np.ndarray] = None  # [nb, nb, 7, 4] orbital-element change (zeros when not tracked)


@dataclass
class App:
    config: Configuration
    state: AppState
    tasks: Tasks
    time_series: List[dict]
    version: str = VERSION

    # -- construction (app.rs:283-325) --------------------------------------------
    @staticmethod
    def from_config(cfg: Configuration) -> "App":
        cons = initial_state(cfg.mesh, cfg.hydro, cfg.physics, cfg.model)
        nb, nf = cfg.mesh.num_blocks, num_fields(cfg.hydro)
        st = AppState(cons=cons, ledger=np.zeros((nb, nb, 7, nf)), time=0.0, iteration=0)
        return App(config=cfg, state=st, tasks=Tasks(), time_series=[])

    @staticmethod
    def from_preset_or_file(name: str, overrides: List[str] = ()) -> "App":
        if name in REFERENCE_PRESETS:
            return App.from_config(config_from_dict(patch_dict(preset_dict(name), list(overrides))))
        if name.endswith(".yaml"):
            with open(name) as f:
                return App.from_config(config_from_dict(patch_dict(yaml_lite.loads(f.read()), list(overrides))))
        if name.endswith(".cbor"):
            app = read_checkpoint(name)
            if overrides:
                app.config = config_from_dict(patch_dict(config_to_dict(app.config), list(overrides)))
            return app
        raise ConfigError("unknown input file type %s" % name)

    # -- serde layout (app.rs:185-192, state.rs:44-62) ------------------------------
    def to_serde(self) -> dict:
        cfg = self.config
        nb, bs = cfg.mesh.num_blocks, cfg.mesh.block_size
        hydro_key = "isothermal" if isinstance(cfg.hydro, Isothermal) else "euler"
        elements = self.state.elements if self.state.elements is not None else np.zeros((nb, nb, 7, 4))
        solution = {}
        for i in range(nb):
            for j in range(nb):
                block = self.state.cons[i, j]
                solution[(i, j)] = {
                    "conserved": cbor.ndarray((bs, bs), [list(map(float, z)) for z in block.reshape(-1, block.shape[-1])]),
                    "integrated_source_terms": {n: list(map(float, self.state.ledger[i, j, k]))
                                                for k, n in enumerate(ITEM_NAMES)},
                    "orbital_elements_change": {n: list(map(float, elements[i, j, k]))
                                                for k, n in enumerate(ITEM_NAMES)},
                }
        state = {"time": float(self.state.time), "iteration": [int(self.state.iteration), 1], "solution": solution}
        return {"state": {hydro_key: state}, "tasks": self.tasks.to_serde(),
                "time_series": {hydro_key: self.time_series}, "config": config_to_dict(cfg),
                "version": self.version}


def write_checkpoint(app: App, path: str):
    """io::write_cbor (io.rs:7-12)."""
    print("write %s" % path)
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(cbor.dumps(app.to_serde()))
    os.replace(tmp, path)


def read_checkpoint(path: str) -> App:
    """io::read_cbor (io.rs:14-18)."""
    with open(path, "rb") as f:
        d = cbor.loads(f.read())
    cfg = config_from_dict(d["config"])
    (hydro_key, st), = d["state"].items()
    nb, bs, nf = cfg.mesh.num_blocks, cfg.mesh.block_size, num_fields(cfg.hydro)
    cons = np.zeros((nb, nb, bs, bs, nf))
    ledger = np.zeros((nb, nb, 7, nf))
    elements = np.zeros((nb, nb, 7, 4))
    for key, blk in st["solution"].items():
        i, j = key
        cons[i, j] = np.array(blk["conserved"]["data"], dtype=np.float64).reshape(bs, bs, nf)
        for k, n in enumerate(ITEM_NAMES):
            ledger[i, j, k] = blk["integrated_source_terms"][n]
            elements[i, j, k] = blk["orbital_elements_change"][n]
    num, den = st["iteration"]
    state = AppState(cons=cons, ledger=ledger, time=float(st["time"]), iteration=int(num) // int(den),
                     elements=elements)
    (_, series), = d["time_series"].items()
    return App(config=cfg, state=state, tasks=Tasks.from_serde(d["tasks"]), time_series=list(series),
               version=d.get("version", ""))


# ----------------------------------------------------------------------------
# The driver (main.rs:99-210)

def _safety(physics: Physics, crashed: bool) -> Physics:
    """main.rs:131-147: safe-mode versions of cfl, plm, mach_ceiling, rk_order."""
    if not crashed:
        return physics
    p = dataclasses.replace(physics)
    if p.safe_cfl is not None:
        p.cfl = p.safe_cfl
    if p.safe_plm is not None:
        p.plm = p.safe_plm
    if p.safe_mach_ceiling is not None:
        p.mach_ceiling = p.safe_mach_ceiling
    if p.safe_rk_order is not None:
        p.rk_order = p.safe_rk_order
    return p


class Driver:
    """main.rs:run over a GB300 context.  `runtime_factory(physics)` builds a
    Runtime for a Physics (tests pass a fake).  With `autotune`, each context
    of an FP32 precision times its tile shapes and row chunks once, on the
    first state it holds (b2d_autotune leaves that state unchanged).  The FP64
    parity path always keeps its default tiles: its per-block ledgers are sums
    of per-tile partials whose rounding depends on the tile shape, so a tiling
    picked by timing would make ledgers differ from run to run and a restart
    from a checkpoint would not continue the run bit for bit."""

    def __init__(self, app: App, precision: str = "fp64", runtime_factory=None, background=None, log=print,
                 autotune: bool = True):
        self.app = app
        self.precision = precision
        self.log = log
        self.autotune = autotune and precision != "fp64"
        self._tuned = set()
        cfg = app.config
        self.background = background if background is not None else initial_state(
            cfg.mesh, cfg.hydro, cfg.physics, cfg.model)       # BlockData::from_model, main.rs:119-122
        self.factory = runtime_factory or (lambda physics: Runtime([Run(cfg.mesh, cfg.hydro, physics)], precision))
        self._rts: Dict[int, Any] = {}
        self._active = None
        self.dt = 0.0

    def _runtime(self, safe: bool):
        """The context for normal (False) or safe-mode (True) physics."""
        rt = self._rts.get(safe)
        if rt is None:
            rt = self.factory(_safety(self.app.config.physics, safe))
            self._rts[safe] = rt
        return rt

    def _load(self, rt):
        s = self.app.state
        rt.upload(0, s.cons, background=self.background, ledger=s.ledger, time=s.time, iteration=s.iteration)
        if s.elements is not None:
            rt.upload_elements(0, s.elements)
        if self.autotune and id(rt) not in self._tuned and hasattr(rt, "autotune"):
            rt.autotune()
            self._tuned.add(id(rt))
        self._active = rt

    def _store(self, rt):
        s = self.app.state
        s.cons, s.time, s.iteration = rt.download(0)
        s.ledger = rt.ledger(0)
        s.elements = rt.elements(0)

    # -- side effects (main.rs:27-86) ------------------------------------------------
    def side_effects(self, rt):
        app, cfg, tasks, s = self.app, self.app.config, self.app.tasks, self.app.state
        if tasks.iteration_message.next_time <= s.time:
            elapsed = tasks.iteration_message.advance(0.0)
            mzps = 1e-6 * cfg.mesh.total_zones() / max(elapsed, 1e-30) * cfg.control.fold
            if tasks.iteration_message.count_this_run > 1:
                self.log("[%05d] orbit=%.5f steps/orbit=%.2e Mzps=%.2f" % (
                    s.iteration, s.time / ORBITAL_PERIOD, ORBITAL_PERIOD / self.dt if self.dt else 0.0, mzps))
        if tasks.record_time_series.next_time <= s.time and cfg.control.time_series_interval is not None:
            tasks.record_time_series.advance(cfg.control.time_series_interval * ORBITAL_PERIOD)
            self._store(rt)
            elements = s.elements if s.elements is not None else np.zeros(s.ledger.shape[:2] + (7, 4))
            app.time_series.append({
                "time": s.time,
                "integrated_source_terms": {n: list(map(float, s.ledger[:, :, k].sum(axis=(0, 1))))
                                            for k, n in enumerate(ITEM_NAMES)},
                "orbital_elements_change": {n: list(map(float, elements[:, :, k].sum(axis=(0, 1))))
                                            for k, n in enumerate(ITEM_NAMES)},
            })
            self.log("record time series sample #%d" % len(app.time_series))
        if tasks.report_progress.next_time <= s.time:
            tasks.report_progress.advance(ORBITAL_PERIOD)
        if tasks.write_checkpoint.next_time <= s.time:
            os.makedirs(cfg.control.output_directory, exist_ok=True)
            path = os.path.join(cfg.control.output_directory, "chkpt.%04d.cbor" % tasks.write_checkpoint.count)
            if tasks.write_checkpoint.count_this_run > 0 or tasks.write_checkpoint.count == 0:
                self._store(rt)
                write_checkpoint(app, path)
            tasks.write_checkpoint.advance(cfg.control.checkpoint_interval * ORBITAL_PERIOD)

    def run(self):
        app, cfg = self.app, self.app.config
        fold = cfg.control.fold
        rt = self._runtime(False)
        self._load(rt)
        self.side_effects(rt)
        fallback: List[tuple] = []
        crash_time = None
        while app.state.time < cfg.control.num_orbits * ORBITAL_PERIOD:
            if cfg.control.fallback_stack_size > 1:
                if len(fallback) > cfg.control.fallback_stack_size:
                    fallback.pop(0)
                self._store(self._active)
                fallback.append((copy.deepcopy(app.state), copy.deepcopy(app.time_series), copy.deepcopy(app.tasks)))
            want = self._runtime(crash_time is not None)
            if want is not self._active:
                self._store(self._active)
                self._load(want)
            rt = self._active
            try:
                dts = rt.advance(fold)
                self.dt = float(dts[0])
                app.state.time, app.state.iteration = rt.time(0)
                if crash_time is not None and crash_time + cfg.physics.safe_mode_duration * ORBITAL_PERIOD < app.state.time:
                    crash_time = None
                    self.log("surpassed previous crash time plus a margin of %s orbits, proceeding in normal mode"
                             % cfg.physics.safe_mode_duration)
            except HydroError as e:
                if not fallback or crash_time is not None:
                    os.makedirs(cfg.control.output_directory, exist_ok=True)
                    path = os.path.join(cfg.control.output_directory, "chkpt.fail.cbor")
                    if app.tasks.write_checkpoint.count_this_run > 0 or app.tasks.write_checkpoint.count == 0:
                        self._store(rt)               # the state before the failing advance
                        write_checkpoint(app, path)
                    raise
                former_state, former_series, former_tasks = fallback[0]
                crash_time = fallback[-1][0].time
                fallback.clear()
                self.log("%s %s" % (e.kind, e))
                self.log("rewind to orbit %.5f, proceed in safety mode..." % (former_state.time / ORBITAL_PERIOD))
                app.state, app.time_series, app.tasks = former_state, former_series, former_tasks
                self._load(self._runtime(True))
            self.side_effects(self._active)
        self._store(self._active)
        return app

    def close(self):
        for rt in self._rts.values():
            close = getattr(rt, "close", None)
            if close:
                close()
