"""Static city inputs bundled for one run.

Field names follow the reference containers the engine reads:
``CityDomain`` (``gurugram_flood/preprocessing/city_data.py:40-64``), ``RealMesh``
(``gurugram_flood/domain/real_gurugram_domain.py:39-56``) and
``ProductionInfiltrationFields``
(``gurugram_flood/domain/production_infiltration_support.py:11-20``).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np

from .topology import (
    TriangularNodeCouplingTopology,
    TriangularPipeNetworkState,
    TriangularPipeNetworkTopology,
    TriangularSurfaceState,
    TriangularSurfaceTopology,
)

MMHR_TO_MPS = 1.0 / (1000.0 * 3600.0)


@dataclass
class RealMesh:
    nodes_xy: np.ndarray
    triangles: np.ndarray
    centroids_xy: np.ndarray
    terrain_elevation_m: np.ndarray
    building_mask: np.ndarray
    road_mask: np.ndarray
    active_mask: np.ndarray

    @property
    def triangle_count(self) -> int:
        return int(self.triangles.shape[0])

    @property
    def node_count(self) -> int:
        return int(self.nodes_xy.shape[0])


@dataclass(frozen=True)
class ProductionInfiltrationFields:
    """Per-cell rainfall multiplier and Horton parameters (SI units)."""

    rainfall_multiplier: np.ndarray
    horton_f0_mps: np.ndarray
    horton_fc_mps: np.ndarray
    horton_k_per_s: np.ndarray
    open_fraction: np.ndarray
    active_mask: np.ndarray


@dataclass
class ProductionTopologies:
    mesh: RealMesh
    surface_topology: TriangularSurfaceTopology
    coupling_topology: TriangularNodeCouplingTopology
    pipe_topology: TriangularPipeNetworkTopology
    surface_state: TriangularSurfaceState
    pipe_state: TriangularPipeNetworkState
    building_fraction: np.ndarray | None = None
    impervious_fraction: np.ndarray | None = None
    rainfall_multiplier: np.ndarray | None = None
    horton_f0_mmhr: np.ndarray | None = None
    horton_fc_mmhr: np.ndarray | None = None
    horton_decay_per_hr: np.ndarray | None = None


@dataclass
class ExternalBoundaryInflowSurface:
    """Hydrographs entering at receiver cells (reference
    ``gurugram_flood/domain/production_event_support.py:24-29``):
    ``q_m3ps_by_receiver`` is [times x receivers] float32, ``times_s``
    strictly increasing float64."""

    receiver_cell_index: np.ndarray
    times_s: np.ndarray
    q_m3ps_by_receiver: np.ndarray
    peak_total_m3ps: float = 0.0
    report: dict | None = None


@dataclass
class June5RechargeTopology:
    """Pond / rain-water-harvesting rows (reference
    ``gurugram_flood/domain/june5_production_drainage.py:99-111``); the
    recharge step reads the source cell, capacities and stop depth."""

    source_cell_index: np.ndarray
    overflow_cell_index: np.ndarray
    storage_capacity_m3: np.ndarray
    capture_capacity_m3ps: np.ndarray
    recharge_capacity_m3ps: np.ndarray
    activation_depth_m: np.ndarray
    stop_depth_m: np.ndarray

    @property
    def row_count(self) -> int:
        return int(np.asarray(self.source_cell_index).size)


@dataclass
class CityDomain:
    topologies: ProductionTopologies
    topology_mode: str
    infiltration_fields: ProductionInfiltrationFields | None
    simple_infiltration_mps: np.ndarray | None
    recharge_topology: Any | None = None
    recharge_info: dict | None = None
    external_boundary: Any | None = None

    @property
    def mesh(self) -> RealMesh:
        return self.topologies.mesh


def empty_drainage(cell_count: int) -> tuple[TriangularNodeCouplingTopology, TriangularPipeNetworkTopology, TriangularPipeNetworkState]:
    """A coupling/pipe topology with no inlets, nodes or links."""

    z_i = np.zeros(0, dtype=np.int32)
    z_f = np.zeros(0, dtype=np.float32)
    coupling = TriangularNodeCouplingTopology(
        inlet_cell_index=z_i, inlet_node_index=z_i, node_surface_cell_index=z_i,
        node_invert_elevation_m=z_f, node_storage_area_m2=z_f, node_max_depth_m=z_f,
    )
    pipe = TriangularPipeNetworkTopology(
        link_from_node_index=z_i, link_to_node_index=z_i, link_length_m=z_f, link_area_m2=z_f,
        link_hydraulic_radius_m=z_f, link_manning_n=z_f,
        outfall_area_m2=z_f, outfall_coefficient=z_f, outfall_tailwater_head_m=z_f,
    )
    state = TriangularPipeNetworkState(node_volume_m3=np.zeros(0), link_flow_m3ps=np.zeros(0))
    return coupling, pipe, state


# ---------------------------------------------------------------------------
# exact production topology export (NPZ) and the per-cell infiltration fields
# ---------------------------------------------------------------------------
_NPZ_COUPLING_OPTIONAL = ("node_initial_fill_depth_m", "inlet_capture_capacity_m3ps", "inlet_surcharge_capacity_m3ps",
                          "surcharge_cell_index", "surcharge_node_index", "surcharge_return_weight", "node_x_m",
                          "node_y_m")
_NPZ_PIPE_OPTIONAL = ("link_flow_capacity_m3ps", "outfall_area_m2", "outfall_coefficient", "outfall_tailwater_head_m",
                      "outfall_flow_capacity_m3ps", "link_invert_elevation_m", "link_diameter_m",
                      "link_minor_loss_coefficient", "link_geometry_code", "link_rect_width_m", "link_rect_height_m")
_NPZ_FIELDS_OPTIONAL = ("building_fraction", "impervious_fraction", "rainfall_multiplier", "horton_f0_mmhr",
                        "horton_fc_mmhr", "horton_decay_per_hr")


def _optional_array(d, name: str):
    if name not in d.files:
        return None
    v = d[name]
    return None if v.size == 0 else v


def load_exact_production_topologies(npz_path) -> ProductionTopologies:
    """The exported exact mesh, surface topology, coupling and pipe graph, with
    the reference export's array names and dtypes
    (``gurugram_flood/domain/production_topology_loader.py:45-137``); the
    initial node volume is storage area x initial fill depth when given."""

    from pathlib import Path

    d = np.load(Path(npz_path), allow_pickle=False)
    mesh = RealMesh(
        nodes_xy=d["nodes_world"].astype(np.float64), triangles=d["triangles"].astype(np.int64),
        centroids_xy=d["centroids_world"].astype(np.float64),
        terrain_elevation_m=d["terrain_elevation_m"].astype(np.float32),
        building_mask=d["building_mask"].astype(bool), road_mask=d["road_mask"].astype(bool),
        active_mask=d["active_surface_mask"].astype(bool),
    )
    surface = TriangularSurfaceTopology(
        bed_elevation_m=d["bed_elevation_m"].astype(np.float64), manning_n=d["manning_n"].astype(np.float64),
        cell_area_m2=d["surface_cell_area_m2"].astype(np.float64),
        characteristic_length_m=d["surface_characteristic_length_m"].astype(np.float64),
        edge_left_cell=d["surface_edge_left_cell"].astype(np.int32),
        edge_right_cell=d["surface_edge_right_cell"].astype(np.int32),
        edge_normal_x=d["surface_edge_normal_x"].astype(np.float64),
        edge_normal_y=d["surface_edge_normal_y"].astype(np.float64),
        edge_length_m=d["surface_edge_length_m"].astype(np.float64),
        boundary_code=d["surface_boundary_code"].astype(np.int32),
        active_mask=d["active_surface_mask"].astype(np.float64),
    )
    coupling = TriangularNodeCouplingTopology(
        inlet_cell_index=d["inlet_cell_index"].astype(np.int32), inlet_node_index=d["inlet_node_index"].astype(np.int32),
        node_surface_cell_index=d["node_surface_cell_index"].astype(np.int32),
        node_invert_elevation_m=d["node_invert_elevation_m"].astype(np.float64),
        node_storage_area_m2=d["node_storage_area_m2"].astype(np.float64),
        node_max_depth_m=d["node_max_depth_m"].astype(np.float64),
        surcharge_return_weight_is_normalized=bool(d["surcharge_return_weight_is_normalized"][0]),
        **{n: _optional_array(d, n) for n in _NPZ_COUPLING_OPTIONAL},
    )
    pipe = TriangularPipeNetworkTopology(
        link_from_node_index=d["link_from_node_index"].astype(np.int32),
        link_to_node_index=d["link_to_node_index"].astype(np.int32),
        link_length_m=d["link_length_m"].astype(np.float64), link_area_m2=d["link_area_m2"].astype(np.float64),
        link_hydraulic_radius_m=d["link_hydraulic_radius_m"].astype(np.float64),
        link_manning_n=d["link_manning_n"].astype(np.float64),
        **{n: _optional_array(d, n) for n in _NPZ_PIPE_OPTIONAL},
    )
    c = mesh.triangle_count
    surface_state = TriangularSurfaceState(np.zeros(c), np.zeros(c), np.zeros(c))
    fill = coupling.node_initial_fill_depth_m
    v0 = (np.zeros(coupling.node_count) if fill is None
          else np.asarray(coupling.node_storage_area_m2, np.float64) * np.asarray(fill, np.float64))
    pipe_state = TriangularPipeNetworkState(v0.astype(np.float64), np.zeros(pipe.link_count))
    return ProductionTopologies(mesh, surface, coupling, pipe, surface_state, pipe_state,
                                **{n: _optional_array(d, n) for n in _NPZ_FIELDS_OPTIONAL})


def save_exact_production_topologies(npz_path, topo: ProductionTopologies) -> None:
    """Write a ProductionTopologies with the export's array names (the inverse
    of load_exact_production_topologies; absent optional arrays are left out)."""

    m, st, cp, pp = topo.mesh, topo.surface_topology, topo.coupling_topology, topo.pipe_topology
    out = {
        "nodes_world": m.nodes_xy, "triangles": m.triangles, "centroids_world": m.centroids_xy,
        "terrain_elevation_m": m.terrain_elevation_m, "building_mask": m.building_mask, "road_mask": m.road_mask,
        "active_surface_mask": (np.asarray(st.active_mask) > 0.5) if st.active_mask is not None else m.active_mask,
        "bed_elevation_m": st.bed_elevation_m, "manning_n": st.manning_n, "surface_cell_area_m2": st.cell_area_m2,
        "surface_characteristic_length_m": st.characteristic_length_m,
        "surface_edge_left_cell": st.edge_left_cell, "surface_edge_right_cell": st.edge_right_cell,
        "surface_edge_normal_x": st.edge_normal_x, "surface_edge_normal_y": st.edge_normal_y,
        "surface_edge_length_m": st.edge_length_m, "surface_boundary_code": st.boundary_code,
        "inlet_cell_index": cp.inlet_cell_index, "inlet_node_index": cp.inlet_node_index,
        "node_surface_cell_index": cp.node_surface_cell_index, "node_invert_elevation_m": cp.node_invert_elevation_m,
        "node_storage_area_m2": cp.node_storage_area_m2, "node_max_depth_m": cp.node_max_depth_m,
        "surcharge_return_weight_is_normalized": np.array([bool(cp.surcharge_return_weight_is_normalized)]),
        "link_from_node_index": pp.link_from_node_index, "link_to_node_index": pp.link_to_node_index,
        "link_length_m": pp.link_length_m, "link_area_m2": pp.link_area_m2,
        "link_hydraulic_radius_m": pp.link_hydraulic_radius_m, "link_manning_n": pp.link_manning_n,
    }
    for n in _NPZ_COUPLING_OPTIONAL:
        if getattr(cp, n) is not None:
            out[n] = getattr(cp, n)
    for n in _NPZ_PIPE_OPTIONAL:
        if getattr(pp, n) is not None:
            out[n] = getattr(pp, n)
    for n in _NPZ_FIELDS_OPTIONAL:
        if getattr(topo, n, None) is not None:
            out[n] = getattr(topo, n)
    np.savez_compressed(npz_path, **{k: np.asarray(v) for k, v in out.items()})


def prepare_production_infiltration_fields(*, active_mask, rainfall_multiplier=None, horton_f0_mmhr=None,
                                           horton_fc_mmhr=None, horton_decay_per_hr=None, building_fraction=None,
                                           impervious_fraction=None, use_bcr_open_fraction: bool = True,
                                           min_open_fraction: float = 0.05) -> ProductionInfiltrationFields:
    """Per-cell rainfall multiplier and Horton parameters from the export's
    arrays, with the reference's defaults where one is missing (f0 6.5 mm/h,
    fc 1 mm/h, decay 2 per hour; ``production_infiltration_support.py:44-93``)."""

    n = len(active_mask)
    mmhr = 1.0 / (1000.0 * 3600.0)
    sized = lambda a: a is not None and np.asarray(a).size == n  # noqa: E731
    rm = np.asarray(rainfall_multiplier, np.float32) if sized(rainfall_multiplier) else np.ones(n, np.float32)
    if use_bcr_open_fraction and sized(building_fraction):
        of = np.clip(1.0 - np.asarray(building_fraction, np.float32), min_open_fraction, 1.0).astype(np.float32)
    else:
        of = np.ones(n, np.float32)
    f0 = ((np.asarray(horton_f0_mmhr, np.float64) * mmhr).astype(np.float32) if sized(horton_f0_mmhr)
          else np.full(n, 6.5 * mmhr, np.float32))
    fc = ((np.asarray(horton_fc_mmhr, np.float64) * mmhr).astype(np.float32) if sized(horton_fc_mmhr)
          else np.full(n, 1.0 * mmhr, np.float32))
    k = ((np.asarray(horton_decay_per_hr, np.float64) / 3600.0).astype(np.float32) if sized(horton_decay_per_hr)
         else np.full(n, 2.0 / 3600.0, np.float32))
    return ProductionInfiltrationFields(rainfall_multiplier=rm, horton_f0_mps=f0, horton_fc_mps=fc, horton_k_per_s=k,
                                        open_fraction=of, active_mask=np.asarray(active_mask).astype(bool))


def production_city(npz_path, use_bcr_open_fraction: bool = True, min_open_fraction: float = 0.05) -> CityDomain:
    """A CityDomain ("exact_production" mode) from an exported production NPZ,
    with the Horton fields the export carries."""

    topo = load_exact_production_topologies(npz_path)
    fields = prepare_production_infiltration_fields(
        active_mask=topo.mesh.active_mask, rainfall_multiplier=topo.rainfall_multiplier,
        horton_f0_mmhr=topo.horton_f0_mmhr, horton_fc_mmhr=topo.horton_fc_mmhr,
        horton_decay_per_hr=topo.horton_decay_per_hr, building_fraction=topo.building_fraction,
        impervious_fraction=topo.impervious_fraction, use_bcr_open_fraction=use_bcr_open_fraction,
        min_open_fraction=min_open_fraction)
    return CityDomain(topo, "exact_production", fields, None)

