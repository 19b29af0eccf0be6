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
