"""Run configuration with the reference's section and key names.

Sections and defaults follow ``gurugram_flood/config.py:39-165``
(``PathsConfig``, ``TopologyConfig``, ``SolverConfig``, ``PhysicsConfig``,
``OutputsConfig``) and the loader follows ``load_config`` (``:180-221``): a
YAML or JSON mapping of sections plus dotted ``section.key`` overrides, with
an error for any unknown section or key.  PyYAML is optional: ``.json`` files and
plain dicts always work, ``.yaml`` files need PyYAML.
"""

from __future__ import annotations

import dataclasses
import json
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, Mapping

from .exceptions import ConfigError


@dataclass
class PathsConfig:
    """Locations of the reference's static city datasets (``config.py:39-71``).

    Kept for configuration and report compatibility: this library takes its
    inputs from the caller (``floodgb.domain`` reads the production topology
    NPZ given its path), so nothing here is opened by the solver."""

    data_dir: str = os.environ.get("GURUGRAM_FLOOD_DATA_DIR", str(Path("data") / "production_gurugram"))
    production_topology_npz: str = "production_topology/d_june5_exact_production_topology_and_mesh.npz"
    horton_bcr_npz: str = "production_topology/horton_bcr_fields.npz"
    recharge_csv: str = "drainage_june5/recharge/surface_recharge_exchange_table.csv"
    external_boundary_inflow_csv: str = (
        "external_boundary_inflow/gurugram_external_boundary_inflow_july2025_133mm_12h.csv")
    mesh_npz: str = "mesh/citywide_anuga_mesh_arrays.npz"
    dem_tif: str = "terrain/hydraulic_dtm_fabdem_5m.tif"
    drain_capacities_geojson: str = "drainage/best_guess_drain_capacities.geojson"
    outfall_inventory_geojson: str = "drainage/outfall_inventory.geojson"
    tailwater_priors_csv: str = "pragmatic_priors/outfall_tailwater_priors.csv"

    def resolve(self, name: str) -> Path:
        """A configured entry resolved against ``data_dir`` (absolute paths kept)."""
        raw = Path(getattr(self, name))
        return raw if raw.is_absolute() else Path(self.data_dir) / raw


@dataclass
class TopologyConfig:
    mode: str = "exact_production"
    drainage_capacity_fraction: float = 0.7
    initial_drainage_storage_fraction: float = 0.5
    tailwater_case: str = "moderate"


@dataclass
class SolverConfig:
    """Time stepping (reference defaults: CFL 0.85, dt <= 1 s, 32-step CFL cache x0.8)."""

    backend: str = "cupy"
    surface_step_mode: str = "full_swe"
    duration_min: float | None = None
    snapshot_interval_min: float = 60.0
    max_dt_s: float = 1.0
    cfl: float = 0.85
    cfl_update_interval_steps: int = 32
    cfl_reuse_safety_factor: float = 0.8
    max_speed_mps: float = 5.0
    finite_check_interval_steps: int = 1000


@dataclass
class PhysicsConfig:
    infiltration_mode: str = "production_horton"
    bcr_open_fraction: bool = True
    bcr_min_open_fraction: float = 0.05
    use_surface_recharge: bool = True
    simple_infiltration_open_mmhr: float = 6.5
    simple_infiltration_road_factor: float = 0.05
    use_external_boundary_inflow: bool = False
    external_boundary_max_snap_m: float = 500.0
    match_reference_initial_node_volume: bool = False
    reference_initial_node_volume_m3: float = 541810.5625
    # Inlet exchange knobs (the reference passes these as keyword defaults of
    # step_triangular_dynamic_pipe_network, triangular_backend.py:665-676).
    inlet_capture_rule: str = "orifice"
    inlet_orifice_area_m2: float = 0.04
    inlet_orifice_coefficient: float = 0.62
    inlet_weir_perimeter_m: float = 0.0
    inlet_weir_coefficient: float = 0.45


@dataclass
class OutputsConfig:
    wet_threshold_m: float = 0.05
    geojson_threshold_m: float = 0.05
    write_npz: bool = True
    # GeoJSON, basemap and PNG writers are outside this library (off by default)
    write_hourly_geojson: bool = False
    write_basemap_html: bool = False
    write_timeseries_png: bool = False
    basemap_max_features: int = 120_000
    basemap_color_max_m: float = 3.0
    mesh_crs: str = "EPSG:32643"


@dataclass
class RunConfig:
    paths: PathsConfig = field(default_factory=PathsConfig)
    topology: TopologyConfig = field(default_factory=TopologyConfig)
    solver: SolverConfig = field(default_factory=SolverConfig)
    physics: PhysicsConfig = field(default_factory=PhysicsConfig)
    outputs: OutputsConfig = field(default_factory=OutputsConfig)

    def validate(self) -> None:
        s, p = self.solver, self.physics
        if s.backend not in ("cupy", "floodgb"):
            raise ConfigError(
                f"production solver is GPU-only; solver.backend must be 'cupy' (or 'floodgb'), got {s.backend!r}"
            )
        if s.surface_step_mode not in ("full_swe", "local_inertial"):
            raise ConfigError(
                f"solver.surface_step_mode must be 'full_swe' or 'local_inertial', got {s.surface_step_mode!r}")
        if p.infiltration_mode not in ("production_horton", "simple_constant"):
            raise ConfigError(
                f"physics.infiltration_mode must be 'production_horton' or 'simple_constant', got {p.infiltration_mode!r}"
            )
        if p.inlet_capture_rule not in ("orifice", "weir_orifice", "capacity", "head_limited_capacity"):
            raise ConfigError(f"physics.inlet_capture_rule {p.inlet_capture_rule!r} is not supported")
        if s.duration_min is not None and s.duration_min <= 0:
            raise ConfigError("solver.duration_min must be positive")
        if not 0 < s.cfl <= 1:
            raise ConfigError("solver.cfl must be in (0, 1]")
        if s.cfl_update_interval_steps < 1:
            raise ConfigError("solver.cfl_update_interval_steps must be >= 1")
        if s.max_dt_s <= 0:
            raise ConfigError("solver.max_dt_s must be positive")
        if s.snapshot_interval_min <= 0:
            raise ConfigError("solver.snapshot_interval_min must be positive")

    def to_dict(self) -> dict[str, Any]:
        return dataclasses.asdict(self)


def _apply_section(section_obj: Any, values: Mapping[str, Any], section_name: str) -> None:
    valid = {f.name for f in dataclasses.fields(section_obj)}
    for key, value in values.items():
        if key not in valid:
            raise ConfigError(f"Unknown config key '{section_name}.{key}'")
        setattr(section_obj, key, value)


def _read_mapping(path: Path) -> dict:
    text = path.read_text(encoding="utf-8")
    if path.suffix.lower() == ".json":
        return json.loads(text) or {}
    try:
        import yaml  # type: ignore[import-not-found]
    except ImportError as exc:  # pragma: no cover - depends on the host
        raise ConfigError(f"PyYAML is needed to read {path}; pass a .json file or a dict instead") from exc
    return yaml.safe_load(text) or {}


def load_config(
    config_file: str | Path | Mapping[str, Any] | None = None,
    overrides: Mapping[str, Any] | None = None,
) -> RunConfig:
    """Build a validated :class:`RunConfig` (sections, then dotted overrides)."""

    cfg = RunConfig()
    loaded: Any = {}
    if isinstance(config_file, Mapping):
        loaded = dict(config_file)
    elif config_file is not None:
        path = Path(config_file)
        if not path.exists():
            raise ConfigError(f"Config file not found: {path}")
        loaded = _read_mapping(path)
    if not isinstance(loaded, dict):
        raise ConfigError("Config must be a mapping of sections")
    sections = {f.name: getattr(cfg, f.name) for f in dataclasses.fields(cfg)}
    for section_name, values in loaded.items():
        if section_name not in sections:
            raise ConfigError(f"Unknown config section '{section_name}'")
        if values is None:
            continue
        if not isinstance(values, dict):
            raise ConfigError(f"Config section '{section_name}' must be a mapping")
        _apply_section(sections[section_name], values, section_name)

    for dotted, value in (overrides or {}).items():
        if value is None:
            continue
        try:
            section_name, key = dotted.split(".", 1)
        except ValueError:
            raise ConfigError(f"Override keys must be 'section.key', got {dotted!r}") from None
        if section_name not in sections:
            raise ConfigError(f"Unknown config section in override '{dotted}'")
        _apply_section(sections[section_name], {key: value}, section_name)
    cfg.validate()
    return cfg
