"""Rebuild topologies and scenarios from the committed golden fixtures."""

from __future__ import annotations

import ast
from pathlib import Path

import numpy as np

from floodgb.domain import CityDomain, ProductionInfiltrationFields, ProductionTopologies, RealMesh
from floodgb.rainfall import rainfall_event
from floodgb.synthetic import Scenario
from floodgb.topology import (
    TriangularNodeCouplingTopology,
    TriangularPipeNetworkState,
    TriangularPipeNetworkTopology,
    TriangularSurfaceState,
    TriangularSurfaceTopology,
)

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str):
    return np.load(GOLDEN / name, allow_pickle=False)


def surface_topology(d, p: str) -> TriangularSurfaceTopology:
    return TriangularSurfaceTopology(
        bed_elevation_m=d[p + "bed"], manning_n=d[p + "manning"], cell_area_m2=d[p + "area"],
        characteristic_length_m=d[p + "char_len"], edge_left_cell=d[p + "left"], edge_right_cell=d[p + "right"],
        edge_normal_x=d[p + "nx"], edge_normal_y=d[p + "ny"], edge_length_m=d[p + "len"],
        boundary_code=d[p + "bcode"], active_mask=d[p + "active"] if int(d[p + "has_active"]) else None,
        has_stage_boundary=bool(int(d[p + "has_stage"])),
    )


def _opt(d, key):
    return d[key] if key in d.files else None


def coupling_pipe(d, p: str):
    cp = TriangularNodeCouplingTopology(
        inlet_cell_index=d[p + "inlet_cell_index"], inlet_node_index=d[p + "inlet_node_index"],
        node_surface_cell_index=d[p + "node_surface_cell_index"],
        node_invert_elevation_m=d[p + "node_invert_elevation_m"],
        node_storage_area_m2=d[p + "node_storage_area_m2"], node_max_depth_m=d[p + "node_max_depth_m"],
        inlet_capture_capacity_m3ps=_opt(d, p + "inlet_capture_capacity_m3ps"),
        inlet_surcharge_capacity_m3ps=_opt(d, p + "inlet_surcharge_capacity_m3ps"),
        surcharge_cell_index=_opt(d, p + "surcharge_cell_index"),
        surcharge_node_index=_opt(d, p + "surcharge_node_index"),
        surcharge_return_weight=_opt(d, p + "surcharge_return_weight"),
        surcharge_return_weight_is_normalized=bool(int(d[p + "surcharge_return_weight_is_normalized"]))
        if p + "surcharge_return_weight_is_normalized" in d.files else False,
    )
    names = ["link_flow_capacity_m3ps", "outfall_area_m2", "outfall_coefficient", "outfall_tailwater_head_m",
             "outfall_flow_capacity_m3ps", "link_invert_elevation_m", "link_diameter_m",
             "link_minor_loss_coefficient", "link_geometry_code", "link_rect_width_m", "link_rect_height_m"]
    pp = TriangularPipeNetworkTopology(
        link_from_node_index=d[p + "link_from_node_index"], link_to_node_index=d[p + "link_to_node_index"],
        link_length_m=d[p + "link_length_m"], link_area_m2=d[p + "link_area_m2"],
        link_hydraulic_radius_m=d[p + "link_hydraulic_radius_m"], link_manning_n=d[p + "link_manning_n"],
        **{n: _opt(d, p + n) for n in names},
    )
    return cp, pp


def scenario(d, p: str) -> Scenario:
    st = surface_topology(d, p + "mesh/")
    cp, pp = coupling_pipe(d, p + "net/")
    c = st.cell_count
    active = st.active_mask > 0.5 if st.active_mask is not None else np.ones(c, bool)
    mesh = RealMesh(nodes_xy=np.zeros((0, 2)), triangles=np.zeros((c, 3), np.int64),
                    centroids_xy=d[p + "centroids"], terrain_elevation_m=st.bed_elevation_m,
                    building_mask=np.zeros(c, bool), road_mask=np.zeros(c, bool), active_mask=active)
    state = TriangularSurfaceState(d[p + "h0"], d[p + "hu0"], d[p + "hv0"])
    pstate = TriangularPipeNetworkState(d[p + "V0"], d[p + "Q0"])
    fields = None
    if p + "f0" in d.files:
        fields = ProductionInfiltrationFields(
            rainfall_multiplier=d[p + "rain_mult"], horton_f0_mps=d[p + "f0"], horton_fc_mps=d[p + "fc"],
            horton_k_per_s=d[p + "k"], open_fraction=np.ones(c, np.float32), active_mask=active)
    topo = ProductionTopologies(mesh, st, cp, pp, state, pstate)
    city = CityDomain(topo, "exact_production" if fields is not None else "synthetic_grid", fields, None)
    hy = d[p + "hyeto"]
    rain = rainfall_event(hy[0], hy[1], hy[2])
    overrides = dict(ast.literal_eval(str(d[p + "overrides"])))
    return Scenario(p.strip("/"), city, rain, overrides)


def inflow(d, p: str):
    """ExternalBoundaryInflowSurface of a fixture prefix (None if absent)."""

    from floodgb.domain import ExternalBoundaryInflowSurface

    if p + "ext_cells" not in d.files:
        return None
    return ExternalBoundaryInflowSurface(receiver_cell_index=d[p + "ext_cells"], times_s=d[p + "ext_times"],
                                         q_m3ps_by_receiver=d[p + "ext_q"])


def recharge(d, p: str):
    """June5RechargeTopology of a fixture prefix (None if absent)."""

    from floodgb.domain import June5RechargeTopology

    if p + "rch_source_cell_index" not in d.files:
        return None
    cells = d[p + "rch_source_cell_index"]
    n = cells.size
    return June5RechargeTopology(
        source_cell_index=cells, overflow_cell_index=cells.copy(),
        storage_capacity_m3=d[p + "rch_storage_capacity_m3"], capture_capacity_m3ps=d[p + "rch_capture_capacity_m3ps"],
        recharge_capacity_m3ps=d[p + "rch_recharge_capacity_m3ps"], activation_depth_m=np.full(n, 0.05, np.float32),
        stop_depth_m=d[p + "rch_stop_depth_m"])


def forcing_scenario(d, p: str) -> Scenario:
    """scenario() plus the prefix's external inflow and recharge rows."""

    sc = scenario(d, p)
    sc.city.external_boundary = inflow(d, p)
    sc.city.recharge_topology = recharge(d, p)
    return sc
