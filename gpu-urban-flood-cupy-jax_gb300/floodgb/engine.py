"""``run_simulation``: the reference engine's public entry point on the GPU loop.

Same signature, result fields, snapshot schedule and mass balance as
``gurugram_flood.solver.engine.run_simulation`` (``engine.py:68-411``).  The
adaptive loop itself runs on the device (libfloodgb ``fl_run``): CFL dt every
``cfl_update_interval_steps`` steps, reused x ``cfl_reuse_safety_factor``
otherwise, snapshots at the first step whose end time reaches each
``snapshot_interval_min`` boundary (and at the end), float64 ledger.  The
host touches the device only between snapshot intervals (when a progress
callback is given) or once at the end.

External boundary inflow (``city.external_boundary``), surface recharge
(``city.recharge_topology``), the weighted surcharge-return table and
``solver.surface_step_mode = "local_inertial"`` all run inside the device
loop.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Any, Callable

import numpy as np

from .config import RunConfig
from .exceptions import SimulationError
from .solver import solver_for_city

ProgressCallback = Callable[[float, dict[str, Any]], None]


@dataclass
class SimulationResult:
    """Host arrays of one run (reference ``SimulationResult``, ``engine.py:68-105``)."""

    snapshot_times_min: np.ndarray
    depth_snapshots_m: np.ndarray
    speed_snapshots_mps: np.ndarray
    node_volume_snapshots_m3: np.ndarray
    final_depth_m: np.ndarray
    final_hu_m2ps: np.ndarray
    final_hv_m2ps: np.ndarray
    final_node_volume_m3: np.ndarray
    final_link_flow_m3ps: np.ndarray
    max_depth_m: np.ndarray
    max_speed_mps: np.ndarray
    mass_balance: dict[str, float]
    step_count: int
    runtime_s: float
    cfl_eval_count: int
    cfl_reused_count: int
    backend_name: str
    is_gpu: bool
    duration_min: float
    city: Any = field(repr=False, default=None)
    rainfall: Any = field(repr=False, default=None)
    config: RunConfig = field(repr=False, default=None)
    ledger: dict = field(repr=False, default_factory=dict)


def snapshot_speed(h: np.ndarray, hu: np.ndarray, hv: np.ndarray) -> np.ndarray:
    """Speed where h > 1e-4 m, else 0 (float32, ``engine.py:314-318``)."""

    speed = np.zeros_like(h)
    wet = h > 1.0e-4
    speed[wet] = np.sqrt(hu[wet] ** 2 + hv[wet] ** 2) / h[wet]
    return speed


def run_simulation(city, rainfall, cfg: RunConfig, progress_callback: ProgressCallback | None = None,
                   device: int = 0) -> SimulationResult:
    s, ph = cfg.solver, cfg.physics
    duration_min = s.duration_min if s.duration_min is not None else rainfall.duration_min
    if duration_min <= 0:
        raise SimulationError(f"Simulation duration must be positive, got {duration_min} min")
    final_s = duration_min * 60.0
    topo = city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    solver = solver_for_city(city, rainfall, cfg, final_s, device=device)
    try:
        h0 = np.asarray(topo.surface_state.h_m, np.float64)
        initial_surface = float(np.sum(h0 * area))
        initial_node = float(np.sum(np.asarray(topo.pipe_state.node_volume_m3, np.float64)))
        valid = np.asarray(city.mesh.active_mask, bool) & ~np.asarray(city.mesh.building_mask, bool)
        t_run0 = time.perf_counter()
        if progress_callback is None:
            solver.run(final_s)
        else:
            interval = s.snapshot_interval_min * 60.0
            target = 0.0
            seen = 0
            while True:
                target = min(target + interval, final_s) if seen else min(1e-9, final_s)
                solver.run(target)
                p = solver.progress()
                if p.snapshot_count > seen:
                    t, h, hu, hv, v = solver.snapshots(p.snapshot_count - 1, 1)
                    elapsed = time.perf_counter() - t_run0
                    info = {
                        "t_min": float(t[0] / 60.0), "dt_s": p.last_dt_s, "step": p.step_count,
                        "wet_triangles": int((h[0][valid] >= cfg.outputs.wet_threshold_m).sum()),
                        "max_depth_m": float(h[0].max()), "steps_per_s": p.step_count / max(elapsed, 1e-9),
                        "elapsed_s": elapsed,
                    }
                    progress_callback(min(t[0] / final_s, 1.0), info)
                    seen = p.snapshot_count
                if p.t_s >= final_s:
                    break
        runtime_s = time.perf_counter() - t_run0
        prog = solver.progress()
        times, hs, hus, hvs, vs = solver.snapshots()
        final_h, final_hu, final_hv, final_v, final_q = solver.get_state()
        led = solver.ledger()
    finally:
        solver.close()

    speeds = np.stack([snapshot_speed(hs[k], hus[k], hvs[k]) for k in range(hs.shape[0])]) if len(times) else hs
    cum = {
        "rainfall_input_m3": led["rainfall_input_m3"],
        "infiltration_loss_m3": led["infiltration_loss_m3"],
        "boundary_net_flux_m3": led["boundary_net_flux_m3"],
        "outfall_discharge_m3": led["outfall_discharge_m3"],
        "overflow_surcharge_m3": led["overflow_surcharge_m3"],
        "unreturned_overflow_m3": led["unreturned_overflow_m3"],
        "external_boundary_inflow_m3": led["external_boundary_inflow_m3"],
        "surface_recharge_capture_m3": led["surface_recharge_capture_m3"],
        "surface_recharge_loss_m3": led["surface_recharge_loss_m3"],
    }
    final_surface = float(np.sum(final_h.astype(np.float64) * area))
    final_node = float(final_v.astype(np.float32).astype(np.float64).sum())
    lhs = initial_surface + initial_node + cum["rainfall_input_m3"] + cum["external_boundary_inflow_m3"]
    rhs = (final_surface + final_node + cum["infiltration_loss_m3"] + cum["outfall_discharge_m3"]
           + cum["unreturned_overflow_m3"] + cum["surface_recharge_loss_m3"] - cum["boundary_net_flux_m3"])
    residual = lhs - rhs
    mass_balance = {
        **cum,
        "initial_surface_volume_m3": initial_surface,
        "initial_node_volume_m3": initial_node,
        "final_surface_volume_m3": final_surface,
        "final_node_volume_m3": final_node,
        "mass_residual_m3": residual,
        "mass_residual_ratio": residual / max(abs(lhs), 1.0),
    }
    return SimulationResult(
        snapshot_times_min=np.asarray(times / 60.0, dtype=np.float32),
        depth_snapshots_m=hs,
        speed_snapshots_mps=speeds,
        node_volume_snapshots_m3=vs,
        final_depth_m=final_h,
        final_hu_m2ps=final_hu,
        final_hv_m2ps=final_hv,
        final_node_volume_m3=final_v.astype(np.float32),
        final_link_flow_m3ps=final_q.astype(np.float32),
        max_depth_m=np.max(hs, axis=0).astype(np.float32),
        max_speed_mps=np.max(speeds, axis=0).astype(np.float32),
        mass_balance=mass_balance,
        step_count=int(prog.step_count),
        runtime_s=runtime_s,
        cfl_eval_count=int(prog.cfl_eval_count),
        cfl_reused_count=int(prog.cfl_reused_count),
        backend_name="floodgb-sm_103a",
        is_gpu=True,
        duration_min=float(duration_min),
        city=city,
        rainfall=rainfall,
        config=cfg,
        ledger=led,
    )
