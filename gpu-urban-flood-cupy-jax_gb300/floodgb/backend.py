"""Function-level mirror of the reference's triangular backend on the GPU.

Same names, arguments, return shapes and errors as the public step functions
of ``gurugram_flood.kernels.triangular_backend``:

* ``step_triangular_surface``              (``triangular_backend.py:478-528``)
* ``step_triangular_surface_local_inertial`` (``:531-590``)
* ``stable_local_inertial_triangular_timestep_s`` (``:975-994``)
* ``step_triangular_dynamic_pipe_network`` (``:665-830``)
* ``stable_triangular_timestep_s``         (``:955-972``)
* ``clamp_velocity``                       (``gurugram_flood/solver/stabilizers.py:8-27``)

Each call moves the given state through a device solver that is built once
per topology (and cached); it is the drop-in for callers that drive the step
from Python.  ``run_simulation`` (``floodgb.engine``) keeps everything on the
device and is the fast path.
"""

from __future__ import annotations

import weakref
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import native as N
from .config import load_config
from .domain import ProductionInfiltrationFields
from .solver import FloodSolver
from .topology import (
    TriangularNodeCouplingTopology,
    TriangularPipeNetworkState,
    TriangularPipeNetworkTopology,
    TriangularSurfaceForcing,
    TriangularSurfaceState,
    TriangularSurfaceTopology,
)


@dataclass(frozen=True)
class TriangularSurfaceDiagnostics:
    rainfall_input_m3: Any
    infiltration_loss_m3: Any
    boundary_net_flux_m3: Any
    boundary_inflow_m3: Any
    boundary_outflow_m3: Any
    final_surface_volume_m3: Any


@dataclass(frozen=True)
class TriangularPipeExchangeDiagnostics:
    surface_capture_m3: Any
    surface_surcharge_m3: Any
    link_abs_flow_m3: Any
    outfall_discharge_m3: Any
    overflow_surcharge_m3: Any
    unreturned_overflow_m3: Any
    final_node_volume_m3: Any
    surface_momentum_scale: Any | None = None
    outfall_m3_by_node: Any | None = None
    surface_surcharge_m3_by_node: Any | None = None
    overflow_surcharge_m3_by_node: Any | None = None


_CACHE: dict = {}


def _solver(key_objs, key_extra, factory):
    key = (tuple(id(o) for o in key_objs), key_extra)
    hit = _CACHE.get(key)
    if hit is not None:
        refs, solver = hit
        if all(r() is o for r, o in zip(refs, key_objs)):
            return solver
    solver = factory()
    _CACHE[key] = (tuple(weakref.ref(o) for o in key_objs), solver)
    return solver


def clear_cache() -> None:
    for _, s in _CACHE.values():
        s.close()
    _CACHE.clear()


def _cfg(cfl=0.85, max_speed=5.0, capture_rule="orifice", orifice_area=0.04, orifice_coef=0.62, weir_perimeter=0.0,
         weir_coef=0.45, mode="full_swe"):
    return load_config(None, {
        "solver.cfl": cfl, "solver.max_speed_mps": max_speed, "solver.duration_min": 1.0e9,
        "solver.surface_step_mode": mode,
        "physics.inlet_capture_rule": capture_rule, "physics.inlet_orifice_area_m2": orifice_area,
        "physics.inlet_orifice_coefficient": orifice_coef, "physics.inlet_weir_perimeter_m": weir_perimeter,
        "physics.inlet_weir_coefficient": weir_coef,
    })


def _surface_solver(topology, stage, per_cell, cfl=0.85, max_speed=5.0, mode="full_swe"):
    def make():
        c = topology.cell_count
        fields = None
        if per_cell:
            ones = np.ones(c, np.float32)
            fields = ProductionInfiltrationFields(ones, ones * 0, ones * 0, ones * 0, ones, ones > 0)
        return FloodSolver(topology, rainfall=None, infiltration_fields=fields, cfg=_cfg(cfl, max_speed, mode=mode),
                           duration_s=1.0e12, boundary_stage_m=stage, max_snapshots=1)

    return _solver([topology], ("surface", stage, per_cell, cfl, max_speed, mode), make)


def step_triangular_surface(state: TriangularSurfaceState, topology: TriangularSurfaceTopology,
                            forcing: TriangularSurfaceForcing, timestep_s: float):
    """One explicit FV step: fluxes, cell update + Manning, rain, infiltration."""

    return _surface_step(state, topology, forcing, timestep_s, "full_swe")


def step_triangular_surface_local_inertial(state: TriangularSurfaceState, topology: TriangularSurfaceTopology,
                                           forcing: TriangularSurfaceForcing, timestep_s: float):
    """One local-inertial routing step: face discharges from water-surface
    slopes, donor-limited volume transfer, momentum from the face discharges,
    rain and infiltration."""

    return _surface_step(state, topology, forcing, timestep_s, "local_inertial")


def _surface_step(state, topology, forcing, timestep_s, mode):
    if timestep_s <= 0.0:
        raise ValueError("timestep_s must be positive.")
    if topology.has_stage_boundary and forcing.boundary_stage_m is None:
        raise ValueError("dirichlet_stage triangular boundary requires boundary_stage_m.")
    stage = None if forcing.boundary_stage_m is None else float(forcing.boundary_stage_m)
    rain, infil = forcing.rainfall_rate_mps, forcing.infiltration_capacity_mps
    per_cell = np.ndim(rain) > 0 or np.ndim(infil) > 0
    s = _surface_solver(topology, stage, per_cell, mode=mode)
    if per_cell:
        c = topology.cell_count
        r = np.broadcast_to(np.asarray(rain, np.float32), (c,))
        f = np.broadcast_to(np.asarray(infil, np.float32), (c,))
        s.update_forcing(rain_multiplier=r, f0=f, fc=f, k=np.zeros(c, np.float32))
        rate = 1.0
    else:
        s.update_forcing(infiltration_mps=float(np.float32(infil)))
        rate = float(np.float32(rain))
    s.set_state(state.h_m, state.hu_m2ps, state.hv_m2ps)
    s.reset_clock()
    s.step(timestep_s, N.FL_PHASE_SURFACE, rate)
    h, hu, hv, _, _ = s.get_state()
    led = s.ledger()
    diag = TriangularSurfaceDiagnostics(
        rainfall_input_m3=led["rainfall_input_m3"], infiltration_loss_m3=led["infiltration_loss_m3"],
        boundary_net_flux_m3=led["boundary_net_flux_m3"], boundary_inflow_m3=led["boundary_inflow_m3"],
        boundary_outflow_m3=led["boundary_outflow_m3"], final_surface_volume_m3=led["surface_volume_m3"],
    )
    return TriangularSurfaceState(h, hu, hv), diag


def clamp_velocity(state: TriangularSurfaceState, max_speed_mps: float, xp=np,
                   topology: TriangularSurfaceTopology | None = None) -> TriangularSurfaceState:
    """Cap |velocity| at max_speed_mps keeping direction (``stabilizers.py:8-27``).

    The reference computes this elementwise; here it runs through the same
    device pass as the surface step, so a topology is needed (any mesh with
    the state's cell count).  Without one the elementwise formula is applied
    with NumPy.
    """

    if topology is None:
        h = np.asarray(state.h_m, np.float32)
        hu = np.asarray(state.hu_m2ps, np.float32)
        hv = np.asarray(state.hv_m2ps, np.float32)
        speed = np.sqrt(hu ** 2 + hv ** 2) / np.maximum(h, np.float32(1.0e-8))
        scale = np.minimum(np.float32(1.0), np.float32(max_speed_mps) / np.maximum(speed, np.float32(1.0e-12)))
        return TriangularSurfaceState(h, hu * scale, hv * scale)
    stage = 0.0 if topology.has_stage_boundary else None  # the stage does not enter the clamp
    s = _surface_solver(topology, stage, False, max_speed=float(max_speed_mps))
    s.set_state(state.h_m, state.hu_m2ps, state.hv_m2ps)
    s.reset_clock()
    s.step(1.0, N.FL_PHASE_CLAMP, 0.0)
    h, hu, hv, _, _ = s.get_state()
    return TriangularSurfaceState(h, hu, hv)


def stable_triangular_timestep_s(topology: TriangularSurfaceTopology, state: TriangularSurfaceState,
                                 cfl: float = 0.45, gravity_mps2: float = 9.80665, min_depth_m: float = 1.0e-5) -> float:
    """Global CFL dt: min over cells of cfl * l / (|u| + sqrt(g h))."""

    stage = 0.0 if topology.has_stage_boundary else None  # the stage does not enter the CFL dt
    s = _surface_solver(topology, stage, False, cfl=float(cfl))
    s.set_state(state.h_m, state.hu_m2ps, state.hv_m2ps)
    return s.stable_timestep()


def stable_local_inertial_triangular_timestep_s(topology: TriangularSurfaceTopology, state: TriangularSurfaceState,
                                                cfl: float = 0.45, gravity_mps2: float = 9.80665,
                                                min_depth_m: float = 1.0e-5) -> float:
    """Global dt from the gravity-wave speed only: min over cells of
    cfl * l / sqrt(g max(h, min_depth))."""

    stage = 0.0 if topology.has_stage_boundary else None
    s = _surface_solver(topology, stage, False, cfl=float(cfl), mode="local_inertial")
    s.set_state(state.h_m, state.hu_m2ps, state.hv_m2ps)
    return s.stable_timestep()


def step_triangular_dynamic_pipe_network(
    h_m, surface_topology: TriangularSurfaceTopology, coupling_topology: TriangularNodeCouplingTopology,
    pipe_topology: TriangularPipeNetworkTopology, pipe_state: TriangularPipeNetworkState, timestep_s: float,
    inlet_orifice_area_m2: float = 0.04, inlet_orifice_coefficient: float = 0.62, inlet_weir_perimeter_m: float = 0.0,
    inlet_weir_coefficient: float = 0.45, gravity_mps2: float = 9.80665, inlet_capture_rule: str = "orifice",
):
    """Inlet exchange, pipe links, outfalls and overflow return for one step."""

    if timestep_s <= 0.0:
        raise ValueError("timestep_s must be positive.")
    if inlet_capture_rule not in {"orifice", "weir_orifice", "capacity", "head_limited_capacity"}:
        raise ValueError("inlet_capture_rule must be 'orifice', 'weir_orifice', 'capacity', or 'head_limited_capacity'.")
    if int(np.asarray(pipe_state.node_volume_m3).shape[0]) != coupling_topology.node_count:
        raise ValueError("pipe_state.node_volume_m3 must have one value per coupling node.")
    if int(np.asarray(pipe_state.link_flow_m3ps).shape[0]) != pipe_topology.link_count:
        raise ValueError("pipe_state.link_flow_m3ps must have one value per pipe link.")
    extra = ("pipe", inlet_capture_rule, inlet_orifice_area_m2, inlet_orifice_coefficient, inlet_weir_perimeter_m,
             inlet_weir_coefficient)

    def make():
        cfg = _cfg(capture_rule=inlet_capture_rule, orifice_area=inlet_orifice_area_m2,
                   orifice_coef=inlet_orifice_coefficient, weir_perimeter=inlet_weir_perimeter_m,
                   weir_coef=inlet_weir_coefficient)
        return FloodSolver(surface_topology, coupling_topology, pipe_topology, cfg=cfg, duration_s=1.0e12,
                           max_snapshots=1, gravity_mps2=gravity_mps2)

    s = _solver([surface_topology, coupling_topology, pipe_topology], extra, make)
    zero = np.zeros(surface_topology.cell_count, np.float32)
    s.set_state(h_m, zero, zero, pipe_state.node_volume_m3, pipe_state.link_flow_m3ps)
    s.reset_clock()
    s.step(timestep_s, N.FL_PHASE_DRAINAGE, 0.0)
    h, _, _, V, Q = s.get_state()
    led = s.ledger()
    diag = TriangularPipeExchangeDiagnostics(
        surface_capture_m3=led["surface_capture_m3"], surface_surcharge_m3=led["surface_surcharge_m3"],
        link_abs_flow_m3=led["link_abs_flow_m3"], outfall_discharge_m3=led["outfall_discharge_m3"],
        overflow_surcharge_m3=led["overflow_surcharge_m3"], unreturned_overflow_m3=led["unreturned_overflow_m3"],
        final_node_volume_m3=led["node_volume_m3"],
    )
    return h, TriangularPipeNetworkState(node_volume_m3=V, link_flow_m3ps=Q), diag
