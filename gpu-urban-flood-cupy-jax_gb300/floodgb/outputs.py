"""Run outputs with the reference's on-disk names.

``save_run_npz`` writes ``flood_simulation_outputs.npz`` with the array names
of ``gurugram_flood/postprocessing/outputs.py:25-58`` and ``build_report``
assembles the ``run_report.json`` keys of ``:61-99``, so the reference's
parity validator (``hybrid_flood/operational/parity_validation.py``) can read
a run of this library next to a reference run.
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

RUN_NPZ_NAME = "flood_simulation_outputs.npz"
REPORT_NAME = "run_report.json"


def save_run_npz(result, out_dir) -> Path:
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    mesh = result.city.mesh
    topo = result.city.topologies
    cp, pp = topo.coupling_topology, topo.pipe_topology
    arrays = dict(
        snapshot_times_min=result.snapshot_times_min,
        snapshot_times_s=result.snapshot_times_min * 60.0,
        depth_snapshots_m=result.depth_snapshots_m,
        speed_snapshots_mps=result.speed_snapshots_mps,
        drain_node_volume_snapshots_m3=result.node_volume_snapshots_m3,
        final_depth_m=result.final_depth_m,
        max_depth_m=result.max_depth_m,
        final_hu_m2ps=result.final_hu_m2ps,
        final_hv_m2ps=result.final_hv_m2ps,
        max_speed_mps=result.max_speed_mps,
        final_node_volume_m3=result.final_node_volume_m3,
        final_link_flow_m3ps=result.final_link_flow_m3ps,
        nodes_world=np.asarray(mesh.nodes_xy, np.float32),
        triangles=np.asarray(mesh.triangles, np.int32),
        centroids_world=np.asarray(mesh.centroids_xy, np.float32),
        terrain_elevation_m=np.asarray(mesh.terrain_elevation_m, np.float32),
        active_surface_mask=np.asarray(mesh.active_mask, bool),
        building_mask=np.asarray(mesh.building_mask, bool),
        road_mask=np.asarray(mesh.road_mask, bool),
        drain_node_x_m=np.asarray(cp.node_x_m if cp.node_x_m is not None else np.zeros(cp.node_count), np.float32),
        drain_node_y_m=np.asarray(cp.node_y_m if cp.node_y_m is not None else np.zeros(cp.node_count), np.float32),
        drain_link_from=np.asarray(pp.link_from_node_index, np.int32),
        drain_link_to=np.asarray(pp.link_to_node_index, np.int32),
    )
    path = out / RUN_NPZ_NAME
    np.savez_compressed(path, **arrays)
    return path


def build_report(result, artifacts: dict | None = None) -> dict:
    cfg = result.config
    mesh = result.city.mesh
    topo = result.city.topologies
    valid = np.asarray(mesh.active_mask, bool) & ~np.asarray(mesh.building_mask, bool)
    return {
        "implementation": "floodgb_sm103a_device_loop",
        "topology_mode": result.city.topology_mode,
        "surface_step_mode": cfg.solver.surface_step_mode,
        "infiltration_mode": cfg.physics.infiltration_mode,
        "backend": result.backend_name,
        "is_gpu": result.is_gpu,
        "rainfall_csv": result.rainfall.source_csv,
        "rainfall_total_mm": result.rainfall.total_depth_mm,
        "duration_min": result.duration_min,
        "runtime_s": result.runtime_s,
        "step_count": result.step_count,
        "steps_per_s": result.step_count / max(result.runtime_s, 1e-9),
        "cfl": cfg.solver.cfl,
        "cfl_update_interval_steps": cfg.solver.cfl_update_interval_steps,
        "cfl_reuse_safety_factor": cfg.solver.cfl_reuse_safety_factor,
        "max_dt_s": cfg.solver.max_dt_s,
        "maximum_allowed_speed_mps": cfg.solver.max_speed_mps,
        "cfl_eval_count": result.cfl_eval_count,
        "cfl_reused_count": result.cfl_reused_count,
        "snapshot_count": int(len(result.snapshot_times_min)),
        "max_depth_m": float(np.nanmax(result.max_depth_m)),
        "wet_triangle_count_005m": int((result.final_depth_m[valid] >= cfg.outputs.wet_threshold_m).sum()),
        "drainage_node_count": int(topo.coupling_topology.node_count),
        "drainage_link_count": int(topo.pipe_topology.link_count),
        "mapped_inlet_count": int(topo.coupling_topology.inlet_count),
        **{k: float(v) for k, v in result.mass_balance.items()},
        "artifacts": artifacts or {},
        "config": cfg.to_dict(),
    }


def write_report(result, out_dir, artifacts: dict | None = None, topology_path=None) -> Path:
    """Write ``run_report.json``.  With ``topology_path`` (the production
    topology NPZ the run was built from, holding ``surface_cell_area_m2``) the
    report also carries what the reference's parity validator reads from a
    candidate run (parity_validation.py:84-88, 163-165): the topology path
    under ``input_report`` and the mass residual ratio under
    ``v1_compatible_mass_residual_ratio`` (this library's ledger is the V1
    ledger, engine.py:364-382)."""

    report = build_report(result, artifacts)
    if topology_path is not None:
        report["input_report"] = {"assets": {"assets": {"topology": {"path": str(Path(topology_path).resolve())}}}}
        report["v1_compatible_mass_residual_ratio"] = float(result.mass_balance["mass_residual_ratio"])
    path = Path(out_dir) / REPORT_NAME
    tmp = path.with_suffix(".json.partial")
    tmp.write_text(json.dumps(report, indent=2, sort_keys=True), encoding="utf-8")
    tmp.replace(path)
    return path
