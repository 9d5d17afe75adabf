"""Run configuration mirroring the reference's serde structs.

Mesh (src/mesh.rs:19-33), Isothermal / Euler (src/physics.rs:256-303),
Physics (src/physics.rs:121-218), InfiniteDisk model (src/disks.rs:80-84) and
Configuration (src/app.rs:169-177), with the same field names, defaults and
Option semantics (None = unset).  `to_c()` flattens one configuration into
the b2d_config struct of the C ABI.
"""
from dataclasses import dataclass, field, fields, asdict
from typing import Optional, Tuple
import math

from ._lib import B2DConfig

ORBITAL_PERIOD = 2.0 * math.pi  # src/physics.rs:21


@dataclass
class Mesh:
    num_blocks: int
    block_size: int
    domain_radius: float

    def block_length(self) -> float:          # mesh.rs:27-29
        return 2.0 * self.domain_radius / self.num_blocks

    def cell_spacing(self) -> float:          # mesh.rs:86-88
        return self.block_length() / self.block_size

    def total_zones(self) -> int:             # mesh.rs:90-92
        return self.num_blocks * self.num_blocks * self.block_size * self.block_size

    def zones_per_side(self) -> int:
        return self.num_blocks * self.block_size


@dataclass
class Isothermal:
    mach_number: float
    density_floor: Optional[float] = None


@dataclass
class Euler:
    gamma_law_index: float
    cooling_coefficient: float = 0.0
    pressure_floor: Optional[float] = None
    density_floor: Optional[float] = None
    density_index: int = 2                     # Euler::default_density_index, physics.rs:305-307
    cooling_slow_start: bool = False
    # β-cooling: not in the reference (None keeps the reference's T^4 law)
    cooling_beta: Optional[float] = None


@dataclass
class Physics:
    buffer_rate: float
    buffer_scale: float
    binary_eccentricity: float
    binary_mass_ratio: float
    cfl: float
    plm: float
    rk_order: str = "RK2"
    sink_radius: float = 0.05
    sink_rate: float = 1.0
    lambda_multiplier: float = 0.0
    viscosity: Tuple[str, float] = ("constant_nu", 1e-3)   # Physics::default_viscosity
    sink_model: str = "impartial"                          # Physics::default_sink
    plm_density_trigger: Optional[float] = None
    fake_mass_threshold: float = 0.0
    fake_mass_rate: float = 0.0
    one_body: bool = False
    mach_ceiling: Optional[float] = None
    softening_length: Optional[float] = None
    dt_min: Optional[float] = None
    safe_mode_duration: float = 0.0
    safe_cfl: Optional[float] = None
    safe_plm: Optional[float] = None
    safe_mach_ceiling: Optional[float] = None
    safe_rk_order: Optional[str] = None
    lambda_: Optional[float] = None                        # deprecated alias `lambda`
    nu: Optional[float] = None                             # deprecated alias
    alpha: Optional[float] = None                          # deprecated alias

    def viscosity_model(self) -> Tuple[str, float]:         # physics.rs:222-230
        if self.nu is not None:
            return ("constant_nu", self.nu)
        if self.alpha is not None:
            return ("alpha", self.alpha)
        return tuple(self.viscosity)

    def rk_substeps(self) -> int:                            # physics.rs:369-375
        return {"RK1": 1, "RK2": 2, "RK3": 3}[self.rk_order]

    def softening(self) -> float:                            # physics.rs:399-405
        return self.sink_radius if self.softening_length is None else self.softening_length


MODEL_KINDS = {"infinite_disk": 0, "infinite_alpha_disk": 1, "finite_disk": 2, "residual_test": 3}


@dataclass
class DiskModel:
    """An initial model of AnyModel (src/app.rs:41-48): `kind` is one of
    infinite_disk (disks.rs:137-157), infinite_alpha_disk (172-193),
    finite_disk (11-115; disk_mass, disk_width, disk_radius,
    softening_length) or residual_test (208-228).  The synthetic cavity,
    seeded multiplicative Σ noise and the rotating core are additions (the
    reference has none of them): inside `core_radius` the gas rotates as a
    solid body at the core edge's Keplerian rate, v and c_s scaled by
    (r / core_radius)^(3/2), instead of the model's r^(-1/2), which diverges
    at the origin; with `edge_width` the velocity is brought to rest at the
    domain edge, v * (1 - tanh((r - (R - w)) / (0.3 w))) / 2, so that the
    periodic boundary does not join counter-rotating flows."""
    surface_density: float = 1.0
    mach_number: Optional[float] = None
    cavity_radius: float = 0.0
    cavity_floor: float = 1e-4
    noise: float = 0.0
    seed: int = 0
    kind: str = "infinite_disk"
    disk_mass: float = 0.0
    disk_width: float = 1.0
    disk_radius: float = 1.0
    softening_length: float = 0.0
    core_radius: float = 0.0
    edge_width: float = 0.0


def to_c(mesh: Mesh, hydro, physics: Physics) -> B2DConfig:
    """Flatten (mesh, hydro, physics) into the C ABI's b2d_config."""
    c = B2DConfig()
    c.num_blocks = mesh.num_blocks
    c.block_size = mesh.block_size
    c.domain_radius = mesh.domain_radius
    if isinstance(hydro, Isothermal):
        c.hydro_kind = 0
        c.mach_number = hydro.mach_number
        c.gamma_law_index = 1.0
        c.density_index = 2
        if hydro.density_floor is not None:
            c.has_density_floor, c.density_floor = 1, hydro.density_floor
    elif isinstance(hydro, Euler):
        c.hydro_kind = 1
        c.gamma_law_index = hydro.gamma_law_index
        c.cooling_coefficient = hydro.cooling_coefficient
        c.density_index = hydro.density_index
        c.cooling_slow_start = int(bool(hydro.cooling_slow_start))
        if hydro.pressure_floor is not None:
            c.has_pressure_floor, c.pressure_floor = 1, hydro.pressure_floor
        if hydro.density_floor is not None:
            c.has_density_floor, c.density_floor = 1, hydro.density_floor
        if hydro.cooling_beta is not None:
            c.cooling_kind, c.cooling_beta = 1, hydro.cooling_beta
    else:
        raise TypeError("hydro must be Isothermal or Euler")
    p = physics
    c.buffer_rate = p.buffer_rate
    c.buffer_scale = p.buffer_scale
    c.binary_eccentricity = p.binary_eccentricity
    c.binary_mass_ratio = p.binary_mass_ratio
    c.lambda_multiplier = p.lambda_multiplier
    kind, value = p.viscosity_model()
    c.viscosity_kind = {"constant_nu": 0, "alpha": 1}[kind]
    c.viscosity = value
    c.sink_model = {"impartial": 0, "torque_free": 1}[p.sink_model]
    c.cfl = p.cfl
    c.plm = p.plm
    if p.plm_density_trigger is not None:
        c.has_plm_density_trigger, c.plm_density_trigger = 1, p.plm_density_trigger
    c.fake_mass_threshold = p.fake_mass_threshold
    c.fake_mass_rate = p.fake_mass_rate
    if p.mach_ceiling is not None:
        c.has_mach_ceiling, c.mach_ceiling = 1, p.mach_ceiling
    c.sink_radius = p.sink_radius
    c.sink_rate = p.sink_rate
    if p.softening_length is not None:
        c.has_softening_length, c.softening_length = 1, p.softening_length
    if p.dt_min is not None:
        c.has_dt_min, c.dt_min = 1, p.dt_min
    c.one_body = int(bool(p.one_body))
    c.rk_order = p.rk_substeps()
    return c


def num_fields(hydro) -> int:
    return 4 if isinstance(hydro, Euler) else 3
