"""Host-side topology and state containers for the triangular flood step.

The dataclasses keep the field names and meaning of the reference's
``gurugram_flood.kernels.triangular_backend`` containers
(``TriangularSurfaceTopology`` ``triangular_backend.py:58-90``,
``TriangularSurfaceState`` ``:49-55``, ``TriangularSurfaceForcing`` ``:93-101``,
``TriangularNodeCouplingTopology`` ``:130-154``,
``TriangularPipeNetworkTopology`` ``:172-200``,
``TriangularPipeNetworkState`` ``:203-208``) so that code written against the
reference can build them unchanged.  Arrays are host NumPy arrays; the device
layout is built once by the native library (``libfloodgb``) when a solver is
created.

``build_triangular_surface_topology`` restates the reference builder
(``triangular_backend.py:244-326`` with ``_orient_triangles_ccw`` ``:1815-1827``
and ``_build_edges`` ``:1830-1869``) with vectorised NumPy instead of a
per-triangle Python loop, producing the same edge order, left/right
assignment, normals, lengths and characteristic lengths.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np

BOUNDARY_CLOSED = 0
BOUNDARY_TRANSMISSIVE = 1
BOUNDARY_REFLECTIVE = 2
BOUNDARY_DIRICHLET_STAGE = 3
BOUNDARY_OUTFLOW = 4


@dataclass(frozen=True)
class TriangularSurfaceState:
    """2D state on triangular finite-volume cells (depth and unit discharges)."""

    h_m: Any
    hu_m2ps: Any
    hv_m2ps: Any


@dataclass(frozen=True)
class TriangularSurfaceTopology:
    """Flattened triangle and edge topology (reference field names)."""

    bed_elevation_m: Any
    manning_n: Any
    cell_area_m2: Any
    characteristic_length_m: Any
    edge_left_cell: Any
    edge_right_cell: Any
    edge_normal_x: Any
    edge_normal_y: Any
    edge_length_m: Any
    boundary_code: Any
    active_mask: Any | None = None
    has_stage_boundary: bool = False
    cell_edge_indices: Any | None = None

    @property
    def cell_count(self) -> int:
        return int(np.asarray(self.cell_area_m2).shape[0])

    @property
    def edge_count(self) -> int:
        return int(np.asarray(self.edge_length_m).shape[0])

    @property
    def boundary_edge_count(self) -> int:
        return int(np.count_nonzero(np.asarray(self.edge_right_cell) < 0))

    @property
    def interior_edge_count(self) -> int:
        return self.edge_count - self.boundary_edge_count


@dataclass(frozen=True)
class TriangularSurfaceForcing:
    """Source terms for one surface step (scalars or per-cell arrays)."""

    rainfall_rate_mps: Any | float = 0.0
    infiltration_capacity_mps: Any | float = 0.0
    boundary_stage_m: Any | float | None = None
    gravity_mps2: float = 9.80665
    min_depth_m: float = 1.0e-5


@dataclass(frozen=True)
class TriangularNodeCouplingTopology:
    """Triangle-to-storage-node exchange topology (reference field names)."""

    inlet_cell_index: Any
    inlet_node_index: Any
    node_surface_cell_index: Any
    node_invert_elevation_m: Any
    node_storage_area_m2: Any
    node_max_depth_m: Any
    node_initial_fill_depth_m: Any | None = None
    inlet_capture_capacity_m3ps: Any | None = None
    inlet_surcharge_capacity_m3ps: Any | None = None
    surcharge_cell_index: Any | None = None
    surcharge_node_index: Any | None = None
    surcharge_return_weight: Any | None = None
    surcharge_return_weight_is_normalized: bool = False
    node_x_m: Any | None = None
    node_y_m: Any | None = None

    @property
    def inlet_count(self) -> int:
        return int(np.asarray(self.inlet_cell_index).shape[0])

    @property
    def node_count(self) -> int:
        return int(np.asarray(self.node_storage_area_m2).shape[0])


@dataclass(frozen=True)
class TriangularPipeNetworkTopology:
    """Dynamic pipe graph; flow is positive from ``link_from`` to ``link_to``."""

    link_from_node_index: Any
    link_to_node_index: Any
    link_length_m: Any
    link_area_m2: Any
    link_hydraulic_radius_m: Any
    link_manning_n: Any
    link_flow_capacity_m3ps: Any | None = None
    outfall_area_m2: Any | None = None
    outfall_coefficient: Any | None = None
    outfall_tailwater_head_m: Any | None = None
    outfall_flow_capacity_m3ps: Any | None = None
    link_invert_elevation_m: Any | None = None
    link_diameter_m: Any | None = None
    link_minor_loss_coefficient: Any | None = None
    link_geometry_code: Any | None = None
    link_rect_width_m: Any | None = None
    link_rect_height_m: Any | None = None
    pressurized_wave_speed_mps: float = 30.0

    @property
    def link_count(self) -> int:
        return int(np.asarray(self.link_length_m).shape[0])


@dataclass(frozen=True)
class TriangularPipeNetworkState:
    """Dynamic drainage state: node storage volume and link discharge."""

    node_volume_m3: Any
    link_flow_m3ps: Any


def boundary_mode_code(mode: str) -> int:
    """Integer boundary code for a mode name (``triangular_backend.py:1050-1064``)."""

    value = mode.lower().replace("-", "_")
    if value in {"closed", "none", "no_flux", "wall"}:
        return BOUNDARY_CLOSED
    if value in {"transmissive", "open", "free"}:
        return BOUNDARY_TRANSMISSIVE
    if value in {"outflow", "open_outflow", "outflow_only", "no_inflow"}:
        return BOUNDARY_OUTFLOW
    if value in {"reflective"}:
        return BOUNDARY_REFLECTIVE
    if value in {"dirichlet_stage", "stage", "fixed_stage"}:
        return BOUNDARY_DIRICHLET_STAGE
    raise ValueError(f"Unsupported triangular boundary mode: {mode}.")


def orient_triangles_ccw(nodes: np.ndarray, triangles: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Swap vertices 1 and 2 of clockwise triangles; return (oriented, area).

    Same rule as the reference ``_orient_triangles_ccw``
    (``triangular_backend.py:1815-1827``): twice the signed area is the 2D
    cross product of (p1 - p0) and (p2 - p0) in float64.
    """

    oriented = np.array(triangles, dtype=np.int64, copy=True)
    p0 = nodes[oriented[:, 0]]
    p1 = nodes[oriented[:, 1]]
    p2 = nodes[oriented[:, 2]]
    a = p1 - p0
    b = p2 - p0
    twice = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
    cw = twice < 0.0
    if np.any(cw):
        tmp = oriented[cw, 1].copy()
        oriented[cw, 1] = oriented[cw, 2]
        oriented[cw, 2] = tmp
        twice = np.where(cw, -twice, twice)
    return oriented, 0.5 * twice


def build_edges(nodes: np.ndarray, triangles: np.ndarray):
    """Unique edges in first-appearance order with left = first owning cell.

    Half-edge ``k`` of cell ``c`` runs (t0,t1), (t1,t2), (t2,t0) for k = 0,1,2,
    and half-edges are visited in (cell, k) order, exactly as the reference
    loop in ``_build_edges`` (``triangular_backend.py:1830-1869``).  An edge
    takes its normal ``(dy, -dx)/len`` and length from its first half-edge.
    Returns (left, right, nx, ny, length, perimeter, half_edge_to_edge).
    """

    n_cells = triangles.shape[0]
    start = triangles[:, [0, 1, 2]].reshape(-1)
    end = triangles[:, [1, 2, 0]].reshape(-1)
    vec = nodes[end] - nodes[start]
    length = np.sqrt(vec[:, 0] * vec[:, 0] + vec[:, 1] * vec[:, 1])
    if np.any(length <= 1.0e-12):
        raise ValueError("triangles contain a zero-length edge.")
    per = length.reshape(n_cells, 3)
    perimeter = (per[:, 0] + per[:, 1]) + per[:, 2]

    lo = np.minimum(start, end)
    hi = np.maximum(start, end)
    key = lo * np.int64(nodes.shape[0]) + hi
    order = np.lexsort((np.arange(key.shape[0]), key))
    skey = key[order]
    new_group = np.empty(skey.shape[0], dtype=bool)
    new_group[0] = True
    new_group[1:] = skey[1:] != skey[:-1]
    group_id = np.cumsum(new_group) - 1
    group_start = np.flatnonzero(new_group)
    group_size = np.diff(np.append(group_start, skey.shape[0]))
    if np.any(group_size > 2):
        raise ValueError("triangular topology contains a non-manifold edge shared by more than two cells.")
    first_half = order[group_start]
    # Edge numbering follows first appearance of each key in loop order.
    edge_rank = np.empty(group_start.shape[0], dtype=np.int64)
    edge_rank[np.argsort(first_half, kind="stable")] = np.arange(group_start.shape[0])
    second_half = np.full(group_start.shape[0], -1, dtype=np.int64)
    has_second = group_size == 2
    second_half[has_second] = order[group_start[has_second] + 1]

    n_edges = group_start.shape[0]
    left = np.empty(n_edges, dtype=np.int64)
    right = np.full(n_edges, -1, dtype=np.int64)
    left[edge_rank] = first_half // 3
    right[edge_rank[has_second]] = second_half[has_second] // 3
    fvec = vec[first_half]
    flen = length[first_half]
    nx = np.empty(n_edges, dtype=np.float64)
    ny = np.empty(n_edges, dtype=np.float64)
    nx[edge_rank] = fvec[:, 1] / flen
    ny[edge_rank] = -fvec[:, 0] / flen
    elen = np.empty(n_edges, dtype=np.float64)
    elen[edge_rank] = flen
    half_to_edge = np.empty(key.shape[0], dtype=np.int64)
    half_to_edge[order] = edge_rank[group_id]
    return left, right, nx, ny, elen, perimeter, half_to_edge


def build_triangular_surface_topology(
    nodes_xy: np.ndarray,
    triangles: np.ndarray,
    bed_elevation_m: np.ndarray,
    manning_n: np.ndarray | float | None = None,
    active_mask: np.ndarray | None = None,
    boundary_mode: str = "closed",
) -> TriangularSurfaceTopology:
    """Build the static edge topology from node and triangle arrays.

    Mirrors ``build_triangular_surface_topology`` (``triangular_backend.py:244-326``):
    triangles are re-oriented counter-clockwise, each edge normal points
    outward from ``edge_left_cell``, exterior edges take ``boundary_mode``'s
    code, interior edges whose left cell is inactive and right cell active
    are swapped (normal negated) so the active cell is on the left, and the
    characteristic length is ``2 A / P``.  Raises the same ``ValueError`` s.
    """

    nodes = np.asarray(nodes_xy, dtype=np.float64)
    tri = np.asarray(triangles, dtype=np.int64)
    bed = np.asarray(bed_elevation_m, dtype=np.float32)
    if nodes.ndim != 2 or nodes.shape[1] != 2:
        raise ValueError("nodes_xy must have shape (node_count, 2).")
    if tri.ndim != 2 or tri.shape[1] != 3:
        raise ValueError("triangles must have shape (triangle_count, 3).")
    if bed.shape != (tri.shape[0],):
        raise ValueError("bed_elevation_m must have one value per triangle.")
    if np.any(tri < 0) or np.any(tri >= nodes.shape[0]):
        raise ValueError("triangles contain node indices outside nodes_xy.")

    oriented, area = orient_triangles_ccw(nodes, tri)
    if np.any(area <= 1.0e-12):
        raise ValueError("triangles contain degenerate or near-zero-area cells.")
    left, right, nx, ny, elen, perimeter, _ = build_edges(nodes, oriented)
    nx = nx.astype(np.float32)
    ny = ny.astype(np.float32)

    code = np.full(left.shape, -1, dtype=np.int32)
    code[right < 0] = boundary_mode_code(boundary_mode)

    if manning_n is None:
        manning = np.full(tri.shape[0], 0.035, dtype=np.float32)
    elif np.isscalar(manning_n):
        manning = np.full(tri.shape[0], float(manning_n), dtype=np.float32)
    else:
        manning = np.asarray(manning_n, dtype=np.float32)
        if manning.shape != (tri.shape[0],):
            raise ValueError("manning_n must be scalar or have one value per triangle.")

    active = None
    if active_mask is not None:
        active = np.asarray(active_mask, dtype=np.float32)
        if active.shape != (tri.shape[0],):
            raise ValueError("active_mask must have one value per triangle.")
        act = active > 0.5
        interior = right >= 0
        safe_right = np.where(interior, right, 0)
        swap = interior & (~act[left]) & act[safe_right]
        if np.any(swap):
            l0 = left.copy()
            left[swap] = right[swap]
            right[swap] = l0[swap]
            nx[swap] *= -1.0
            ny[swap] *= -1.0

    char_len = 2.0 * area / np.maximum(perimeter, 1.0e-12)
    return TriangularSurfaceTopology(
        bed_elevation_m=bed.astype(np.float32),
        manning_n=manning.astype(np.float32),
        cell_area_m2=area.astype(np.float32),
        characteristic_length_m=char_len.astype(np.float32),
        edge_left_cell=left.astype(np.int32),
        edge_right_cell=right.astype(np.int32),
        edge_normal_x=nx.astype(np.float32),
        edge_normal_y=ny.astype(np.float32),
        edge_length_m=elen.astype(np.float32),
        boundary_code=code,
        active_mask=active,
        has_stage_boundary=boundary_mode_code(boundary_mode) == BOUNDARY_DIRICHLET_STAGE,
    )


def cell_edge_indices(topology: TriangularSurfaceTopology) -> np.ndarray:
    """(C, 3) int32 table of each cell's edges (-1 pads).

    Same construction as ``triangular_topology_to_backend``
    (``triangular_backend.py:337-359``): the left incidences followed by the
    right incidences are stably sorted by cell, so a row lists the edges the
    cell is left of (ascending) before the edges it is right of (ascending).
    """

    left = np.asarray(topology.edge_left_cell, dtype=np.int64)
    right = np.asarray(topology.edge_right_cell, dtype=np.int64)
    n_cells = topology.cell_count
    n_edges = left.shape[0]
    cells = np.concatenate([left, np.where(right >= 0, right, -1)])
    edges = np.concatenate([np.arange(n_edges), np.arange(n_edges)])
    valid = cells >= 0
    vc = cells[valid]
    ve = edges[valid]
    order = np.argsort(vc, kind="stable")
    vc = vc[order]
    ve = ve[order]
    starts = np.searchsorted(vc, np.arange(n_cells))
    slot = np.arange(vc.shape[0]) - starts[vc]
    table = np.full((n_cells, 3), -1, dtype=np.int32)
    ok = slot < 3
    table[vc[ok], slot[ok]] = ve[ok]
    return table
