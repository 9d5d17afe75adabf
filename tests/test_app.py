"""Host application layer: YAML configuration, presets, overrides, CBOR
checkpoints and the driver loop (fallback stack, safe mode, side effects).
The driver is exercised on CPU with a fake context whose hydro failures are
injected on the host; a GPU test checks checkpoint/restart equivalence."""
import dataclasses
import math
import os

import numpy as np
import pytest

import binary2d as b2
from binary2d import app, cbor, yaml_lite
from binary2d._lib import B2DError

CONFIG = """
# an isothermal setup in the reference's layout
hydro:
  isothermal:
    mach_number: 10.0      # global Mach number
model:
  infinite_disk:
    mach_number: ~
    surface_density: 1e-3  # light gas: a coarse block's pull keeps the binary bound
mesh:
  block_size: 16
  num_blocks: 2
  domain_radius: 8.0
physics:
  binary_eccentricity: 0.0
  binary_mass_ratio: 1.0
  buffer_rate: 1e3
  buffer_scale: 0.3
  cfl: 0.4
  plm: 1.5
  rk_order: RK2
  viscosity:
    constant_nu: 0.001
  sink_radius: 0.05
  sink_rate: 10.0
  safe_cfl: 0.1
  safe_mode_duration: 0.0
control:
  num_orbits: 0.01
  checkpoint_interval: 0.005
  time_series_interval: 0.002
  fold: 2
  num_threads: ~
  output_directory: data
  fallback_stack_size: 3
"""


def test_yaml_subset():
    d = yaml_lite.loads(CONFIG)
    assert d["hydro"]["isothermal"]["mach_number"] == 10.0
    assert d["model"]["infinite_disk"]["mach_number"] is None
    assert d["physics"]["buffer_rate"] == 1000.0 and d["physics"]["rk_order"] == "RK2"
    assert d["control"]["fold"] == 2 and d["control"]["num_threads"] is None
    assert yaml_lite.loads(yaml_lite.dumps(d)) == d
    with pytest.raises(yaml_lite.YamlError):
        yaml_lite.loads("a:\n  - 1\n")


def test_configuration_and_overrides(tmp_path):
    cfg = app.config_from_dict(yaml_lite.loads(CONFIG))
    assert isinstance(cfg.hydro, b2.Isothermal) and cfg.mesh.num_blocks == 2
    assert cfg.physics.viscosity_model() == ("constant_nu", 0.001)
    extra = tmp_path / "extra.yaml"
    extra.write_text("physics:\n  plm: 1.8\nmesh:\n  num_blocks: 4\n")
    d = app.patch_dict(yaml_lite.loads(CONFIG), ["control.num_orbits=100", str(extra), "physics.nu=0.002"])
    cfg = app.config_from_dict(d)
    assert cfg.control.num_orbits == 100 and cfg.physics.plm == 1.8 and cfg.mesh.num_blocks == 4
    assert cfg.physics.viscosity_model() == ("constant_nu", 0.002)      # deprecated alias wins
    bad = yaml_lite.loads(CONFIG)
    bad["physics"]["not_a_field"] = 1
    with pytest.raises(app.ConfigError):
        app.config_from_dict(bad)
    bad = yaml_lite.loads(CONFIG)
    bad["model"]["infinite_disk"]["mach_number"] = 10.0
    with pytest.raises(app.ConfigError, match="not both"):
        app.config_from_dict(bad)


@pytest.mark.parametrize("name", ["iso-circular", "cooling-cbd", "test-grid-visc"])
def test_presets(name):
    cfg = app.config_from_dict(app.preset_dict(name))
    d = app.config_to_dict(cfg)
    assert app.config_from_dict(d) == cfg
    assert cfg.control.fold == 10


def test_cbor_roundtrip():
    obj = {"a": [1, -2, 3.5, float(2 ** 70), None, True, "x"], (1, 2): {"z": 1e-300}, "nested": [[0.1, 0.2]]}
    back = cbor.loads(cbor.dumps(obj))
    assert back["a"] == obj["a"] and back[cbor.Key((1, 2))]["z"] == 1e-300 and back["nested"] == [[0.1, 0.2]]
    assert cbor.dumps(1.5)[0] == 0xFA and cbor.dumps(0.1)[0] == 0xFB   # shortest exact float
    assert cbor.dumps(-1) == b"\x20" and cbor.dumps(500) == b"\x19\x01\xf4"


def test_checkpoint_roundtrip(tmp_path):
    a = app.App.from_config(app.config_from_dict(yaml_lite.loads(CONFIG)))
    a.state.ledger[...] = np.random.default_rng(0).normal(size=a.state.ledger.shape)
    a.state.time, a.state.iteration = 0.125, 17
    a.time_series.append({"time": 0.1, "integrated_source_terms": {}, "orbital_elements_change": {}})
    p = str(tmp_path / "chkpt.0000.cbor")
    app.write_checkpoint(a, p)
    b = app.read_checkpoint(p)
    assert np.array_equal(a.state.cons, b.state.cons) and np.array_equal(a.state.ledger, b.state.ledger)
    assert (b.state.time, b.state.iteration) == (0.125, 17)
    assert b.config == a.config and b.time_series == a.time_series
    c = app.App.from_preset_or_file(p, ["control.num_orbits=5"])
    assert c.config.control.num_orbits == 5


class FakeRuntime:
    """A context stand-in: time advances by fold * cfl; the advances listed in
    `fail_at` raise a hydro error (host-side injection)."""
    calls = 0

    def __init__(self, physics, fail_at):
        self.physics, self.fail_at = physics, fail_at
        self.cons = self._led = None
        self.t = 0.0
        self.it = 0

    def upload(self, run, cons, background=None, ledger=None, time=0.0, iteration=0):
        self.cons, self._led, self.t, self.it = cons.copy(), ledger.copy(), time, iteration

    def download(self, run=0):
        return self.cons.copy(), self.t, self.it

    def ledger(self, run=0):
        return self._led.copy()

    def upload_elements(self, run, elements):
        self._el = elements.copy()

    def elements(self, run=0):
        return getattr(self, "_el", np.zeros(self._led.shape[:2] + (7, 4))).copy()

    def time(self, run=0):
        return self.t, self.it

    def advance(self, fold):
        FakeRuntime.calls += 1
        if FakeRuntime.calls in self.fail_at:
            e = B2DError()
            e.code = 1
            raise b2.HydroError(e)
        self.t += fold * self.physics.cfl * 1e-3
        self.it += fold
        self.cons = self.cons * 1.0
        return np.array([self.physics.cfl * 1e-3])


def _fake_driver(tmp_path, fail_at, **control):
    d = yaml_lite.loads(CONFIG)
    d["control"].update(control)
    d["control"]["output_directory"] = str(tmp_path)
    a = app.App.from_config(app.config_from_dict(d))
    made = []

    def factory(physics):
        rt = FakeRuntime(physics, fail_at)
        made.append(rt)
        return rt

    FakeRuntime.calls = 0
    return app.Driver(a, runtime_factory=factory, background=a.state.cons, log=lambda *_: None), made


def test_driver_rewinds_into_safe_mode(tmp_path):
    drv, made = _fake_driver(tmp_path, fail_at={6})
    a = drv.run()
    assert a.state.time >= a.config.control.num_orbits * 2 * math.pi
    assert len(made) == 2 and made[1].physics.cfl == 0.1       # safe_cfl context after the crash
    assert a.time_series and os.path.exists(tmp_path / "chkpt.0000.cbor")


def test_driver_without_fallback_writes_fail_checkpoint(tmp_path):
    drv, _ = _fake_driver(tmp_path, fail_at={3}, fallback_stack_size=0)
    with pytest.raises(b2.HydroError):
        drv.run()
    assert os.path.exists(tmp_path / "chkpt.fail.cbor")
    fail = app.read_checkpoint(str(tmp_path / "chkpt.fail.cbor"))
    assert fail.state.iteration == 2 * 2                       # the state before the failing advance


def test_driver_second_crash_in_safe_mode_is_fatal(tmp_path):
    drv, _ = _fake_driver(tmp_path, fail_at={4, 5})
    with pytest.raises(b2.HydroError):
        drv.run()


@pytest.mark.gpu
def test_checkpoint_restart_is_bitwise_continuous(tmp_path):
    d = yaml_lite.loads(CONFIG)
    d["control"].update(num_orbits=0.004, output_directory=str(tmp_path / "a"), fallback_stack_size=0)
    cfg = app.config_from_dict(d)
    # default driver settings: the FP64 path keeps its default tiles (the
    # ledgers' per-tile partial sums round differently under different tile
    # shapes), so no autotune runs here
    whole = app.Driver(app.App.from_config(cfg), log=lambda *_: None)
    full = whole.run()
    whole.close()
    # restart from the first checkpoint and run to the same end time
    first = app.read_checkpoint(str(tmp_path / "a" / "chkpt.0000.cbor"))
    first.config.control.output_directory = str(tmp_path / "b")
    again = app.Driver(first, log=lambda *_: None)
    rest = again.run()
    again.close()
    assert rest.state.iteration == full.state.iteration
    assert np.array_equal(rest.state.cons, full.state.cons)
    assert np.array_equal(rest.state.ledger, full.state.ledger)
    assert np.array_equal(rest.state.elements, full.state.elements)
    assert np.abs(full.state.elements).max() > 0.0


@pytest.mark.gpu
def test_driver_autotune_keeps_the_run(tmp_path):
    """The driver's one autotune per FP32 context (trial advances on the
    loaded state, then discarded) leaves the run itself unchanged: the same
    state bit for bit, and the same ledgers up to the FP32 summation order of
    the tiles.  The FP64 driver does not autotune."""
    d = yaml_lite.loads(CONFIG)
    assert app.Driver(app.App.from_config(app.config_from_dict(d)), log=lambda *_: None,
                      runtime_factory=lambda p: None).autotune is False
    out = []
    for tune in (False, True):
        d = yaml_lite.loads(CONFIG)
        d["control"].update(num_orbits=0.004, output_directory=str(tmp_path / str(tune)), fallback_stack_size=0)
        d["mesh"]["block_size"] = 64      # 64-column blocks: the paired FP32 kernel's tiles are candidates
        drv = app.Driver(app.App.from_config(app.config_from_dict(d)), precision="fp32_comp",
                         log=lambda *_: None, autotune=tune)
        assert drv.autotune is tune
        res = drv.run()
        drv.close()
        out.append(res.state)
    a, b = out
    assert a.iteration == b.iteration and a.time == b.time
    assert np.array_equal(a.cons, b.cons)
    scale = np.maximum(np.abs(a.ledger).sum(axis=(0, 1)), 1e-300)
    # per-tile FP32 partial sums in another order: the FP32 ledger tolerance
    # of the parity tests
    assert (np.abs(a.ledger - b.ledger).sum(axis=(0, 1)) / scale).max() <= 1e-4
