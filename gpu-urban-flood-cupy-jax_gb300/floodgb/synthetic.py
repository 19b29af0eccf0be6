"""Seeded synthetic city inputs.

The reference's production mesh, drainage export, Horton fields and rainfall
CSVs are not distributed, so runs here use seeded synthetic inputs with the
same shapes:

* ``make_grid_city`` -- a jittered square grid split into triangles, planar
  slope plus a Gaussian random field bed, uniform Manning n, outflow-only
  exterior, no infiltration, no drainage (the small CPU-runnable workload:
  100 x 100 squares over 1 km, 20,000 triangles, 30,200 edges; ensemble
  members use other grid sizes).
* ``make_coupled_city`` -- a seeded Delaunay mesh of a disk with an exact
  triangle / edge count (981,880 / 1,490,015 at full size, 817,573 active),
  slope + fractal-noise bed with a carved street grid, four Manning land
  classes, Horton infiltration on pervious classes, and a drainage network
  (spanning tree + loop links, lognormal circular pipes, inlets at the nearest
  triangles, outfalls at the lowest nodes).

All generators are deterministic in their seed.
"""

from __future__ import annotations

import hashlib
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .config import load_config
from .domain import MMHR_TO_MPS, CityDomain, ProductionInfiltrationFields, ProductionTopologies, RealMesh, empty_drainage
from .rainfall import RainfallEvent, hourly_rainfall, rainfall_event, uniform_rainfall
from .topology import (
    TriangularNodeCouplingTopology,
    TriangularPipeNetworkState,
    TriangularPipeNetworkTopology,
    TriangularSurfaceState,
    build_triangular_surface_topology,
)

# Front-loaded 24 h hyetograph (mm/h per hour), scaled to 160.09 mm total.
_FRONT_LOADED = np.array(
    [38.0, 26.0, 18.0, 13.0, 10.0, 8.0, 6.5, 5.5, 4.5, 4.0, 3.5, 3.0,
     2.8, 2.6, 2.4, 2.2, 2.0, 1.8, 1.6, 1.4, 1.2, 1.0, 0.9, 0.8]
)
FRONT_LOADED_24H_MMHR = _FRONT_LOADED * (160.09 / _FRONT_LOADED.sum())


@dataclass
class Scenario:
    """A city, its rainfall and the config overrides that describe the run."""

    name: str
    city: CityDomain
    rainfall: RainfallEvent
    overrides: dict

    @property
    def cell_count(self) -> int:
        return self.city.mesh.triangle_count


# ---------------------------------------------------------------------------
# random fields
# ---------------------------------------------------------------------------

def gaussian_random_field(
    rng: np.random.Generator,
    origin: tuple[float, float],
    extent: float,
    spacing: float,
    corr_len: float,
    sigma: float,
):
    """Return f(x, y): a smooth zero-mean field with std ``sigma``.

    White noise on a square raster is filtered in Fourier space with the
    transfer function exp(-(k corr_len)^2 / 8), i.e. a Gaussian covariance
    exp(-r^2 / corr_len^2) up to scale; the raster is normalised to unit std and
    sampled bilinearly.
    """

    n = int(np.ceil(extent / spacing)) + 2
    n = max(8, int(2 ** np.ceil(np.log2(n))))
    noise = rng.standard_normal((n, n))
    k = 2.0 * np.pi * np.fft.fftfreq(n, d=spacing)
    kx, ky = np.meshgrid(k, k, indexing="ij")
    transfer = np.exp(-(kx * kx + ky * ky) * corr_len * corr_len / 8.0)
    field = np.real(np.fft.ifft2(np.fft.fft2(noise) * transfer))
    field = (field - field.mean()) / max(field.std(), 1e-30) * sigma
    ox, oy = origin

    def sample(x: np.ndarray, y: np.ndarray) -> np.ndarray:
        fx = np.clip((np.asarray(x) - ox) / spacing, 0, n - 1.000001)
        fy = np.clip((np.asarray(y) - oy) / spacing, 0, n - 1.000001)
        i0 = np.floor(fx).astype(np.int64)
        j0 = np.floor(fy).astype(np.int64)
        tx = fx - i0
        ty = fy - j0
        i1 = np.minimum(i0 + 1, n - 1)
        j1 = np.minimum(j0 + 1, n - 1)
        return (
            field[i0, j0] * (1 - tx) * (1 - ty)
            + field[i1, j0] * tx * (1 - ty)
            + field[i0, j1] * (1 - tx) * ty
            + field[i1, j1] * tx * ty
        )

    return sample


# ---------------------------------------------------------------------------
# grid cities (small workload and ensemble members)
# ---------------------------------------------------------------------------

def grid_mesh(n: int, size_m: float, jitter_frac: float, rng: np.random.Generator):
    """(n+1)^2 jittered grid vertices and 2 n^2 triangles (one diagonal per square)."""

    h = size_m / n
    xs, ys = np.meshgrid(np.arange(n + 1) * h, np.arange(n + 1) * h, indexing="xy")
    pts = np.stack([xs.ravel(), ys.ravel()], axis=1).astype(np.float64)
    interior = (xs.ravel() > 0) & (xs.ravel() < size_m) & (ys.ravel() > 0) & (ys.ravel() < size_m)
    jit = rng.uniform(-jitter_frac * h, jitter_frac * h, size=pts.shape)
    pts[interior] += jit[interior]
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (j * (n + 1) + i).ravel()
    b = a + 1
    c = a + n + 1
    d = c + 1
    tris = np.empty((2 * n * n, 3), dtype=np.int64)
    tris[0::2] = np.stack([a, b, d], axis=1)
    tris[1::2] = np.stack([a, d, c], axis=1)
    return pts, tris


def make_grid_city(
    n: int = 100,
    size_m: float = 1000.0,
    seed: int = 0,
    slope: float = 0.005,
    grf_sigma: float = 0.3,
    grf_corr_m: float = 50.0,
    manning: float = 0.03,
    rain_mmhr: float = 50.0,
    duration_min: float = 60.0,
    boundary_mode: str = "outflow",
    hyetograph: RainfallEvent | None = None,
) -> Scenario:
    """Jittered-grid city: planar slope + GRF bed, uniform n, no drainage."""

    rng = np.random.default_rng(seed)
    pts, tris = grid_mesh(n, size_m, 0.2, rng)
    cen = pts[tris].mean(axis=1)
    grf = gaussian_random_field(np.random.default_rng(seed + 1), (-20.0, -20.0), size_m + 40.0, 2.0, grf_corr_m, grf_sigma)
    bed = (slope * cen[:, 0] + grf(cen[:, 0], cen[:, 1])).astype(np.float32)
    surface = build_triangular_surface_topology(pts, tris, bed, manning, None, boundary_mode)
    coupling, pipe, pipe_state = empty_drainage(len(tris))
    c = len(tris)
    mesh = RealMesh(
        nodes_xy=pts, triangles=tris, centroids_xy=cen, terrain_elevation_m=bed,
        building_mask=np.zeros(c, bool), road_mask=np.zeros(c, bool), active_mask=np.ones(c, bool),
    )
    state = TriangularSurfaceState(np.zeros(c, np.float32), np.zeros(c, np.float32), np.zeros(c, np.float32))
    topo = ProductionTopologies(mesh, surface, coupling, pipe, state, pipe_state)
    city = CityDomain(topo, "synthetic_grid", None, None)
    rain = hyetograph if hyetograph is not None else uniform_rainfall(rain_mmhr, duration_min)
    overrides = {
        "physics.infiltration_mode": "simple_constant",
        "solver.duration_min": duration_min,
    }
    return Scenario(f"grid{n}_s{seed}", city, rain, overrides)


# ---------------------------------------------------------------------------
# production-shaped coupled city
# ---------------------------------------------------------------------------

def _disk_points(n_boundary: int, n_interior: int, radius: float, rng: np.random.Generator) -> np.ndarray:
    th = 2.0 * np.pi * np.arange(n_boundary) / n_boundary
    boundary = np.stack([radius * np.cos(th), radius * np.sin(th)], axis=1)
    # jittered hexagonal lattice, a little denser than needed, then thinned
    a0 = np.sqrt(2.0 * np.pi * radius * radius / (np.sqrt(3.0) * n_interior))
    inner = radius - 0.7 * a0
    a = np.sqrt(2.0 * np.pi * inner * inner / (np.sqrt(3.0) * n_interior)) * 0.97
    ny = int(2 * radius / (a * np.sqrt(3) / 2)) + 3
    nx = int(2 * radius / a) + 3
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x = -radius - a + ii * a + (jj % 2) * 0.5 * a
    y = -radius - a + jj * a * np.sqrt(3) / 2
    lat = np.stack([x.ravel(), y.ravel()], axis=1)
    lat += rng.uniform(-0.22 * a, 0.22 * a, size=lat.shape)
    r = np.hypot(lat[:, 0], lat[:, 1])
    lat = lat[r < radius - 0.6 * a]
    if lat.shape[0] < n_interior:
        raise RuntimeError("lattice too sparse for the requested interior point count")
    keep = rng.choice(lat.shape[0], size=n_interior, replace=False)
    keep.sort()
    return np.concatenate([boundary, lat[keep]], axis=0)


def _street_grid(rng: np.random.Generator, lo: float, hi: float):
    pos = []
    p = lo + rng.uniform(0, 150)
    while p < hi:
        pos.append(p)
        p += rng.uniform(120.0, 260.0)
    pos = np.asarray(pos)
    depth = rng.uniform(0.3, 1.0, size=pos.shape[0])
    return pos, depth


def _nearest_line(v: np.ndarray, lines: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    idx = np.clip(np.searchsorted(lines, v), 1, len(lines) - 1)
    left = lines[idx - 1]
    right = lines[idx]
    use_left = np.abs(v - left) <= np.abs(v - right)
    best = np.where(use_left, idx - 1, idx)
    return best, np.abs(v - lines[best])


def make_coupled_city(
    n_triangles: int = 981_880,
    n_edges: int = 1_490_015,
    n_active: int = 817_573,
    n_nodes: int = 118_768,
    n_links: int = 139_798,
    n_inlets: int = 61_317,
    n_outfalls: int = 46,
    area_km2: float = 300.0,
    seed: int = 1,
    duration_min: float = 60.0,
    hourly_mmhr: np.ndarray | None = None,
) -> Scenario:
    """Production-shaped coupled city with exact mesh and network counts."""

    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import minimum_spanning_tree
    from scipy.spatial import Delaunay

    n_boundary = 2 * n_edges - 3 * n_triangles
    n_vertices = 1 + n_edges - n_triangles
    if n_boundary < 3 or n_vertices - n_boundary < 3:
        raise ValueError("inconsistent triangle/edge counts for a triangulated disk")
    rng = np.random.default_rng(seed)
    radius = float(np.sqrt(area_km2 * 1e6 / np.pi))
    pts = _disk_points(n_boundary, n_vertices - n_boundary, radius, rng)
    tri = Delaunay(pts).simplices.astype(np.int64)
    if tri.shape[0] != n_triangles:
        raise RuntimeError(f"Delaunay produced {tri.shape[0]} triangles, expected {n_triangles}")
    cen = pts[tri].mean(axis=1)
    cx, cy = cen[:, 0], cen[:, 1]
    c = n_triangles

    # bed: regional slope + fractal noise, streets carved along a seeded grid
    ang = rng.uniform(0, 2 * np.pi)
    bed = 220.0 + 0.003 * (np.cos(ang) * cx + np.sin(ang) * cy)
    for corr, amp in ((4000.0, 3.0), (1000.0, 1.2), (250.0, 0.4), (60.0, 0.12)):
        f = gaussian_random_field(rng, (-radius - 10, -radius - 10), 2 * radius + 20, corr / 6.0, corr, amp)
        bed = bed + f(cx, cy)
    xl, xd = _street_grid(rng, -radius, radius)
    yl, yd = _street_grid(rng, -radius, radius)
    ix, dx = _nearest_line(cx, xl)
    iy, dy = _nearest_line(cy, yl)
    half_width = 9.0
    on_x = dx < half_width
    on_y = dy < half_width
    carve = np.maximum(np.where(on_x, xd[ix], 0.0), np.where(on_y, yd[iy], 0.0))
    road = on_x | on_y
    bed = (bed - carve).astype(np.float32)

    # activity: outer band (cells touching the hull ring) + building footprints
    band = np.any(tri < n_boundary, axis=1)
    n_inactive = c - n_active
    n_build = n_inactive - int(band.sum())
    if n_build < 0:
        raise RuntimeError("boundary band exceeds the inactive cell budget")
    bfield = gaussian_random_field(rng, (-radius - 10, -radius - 10), 2 * radius + 20, 6.0, 30.0, 1.0)(cx, cy)
    bfield[band | road] = -np.inf
    building = np.zeros(c, dtype=bool)
    if n_build > 0:
        building[np.argpartition(-bfield, n_build - 1)[:n_build]] = True
    active = ~(band | building)
    assert int(active.sum()) == n_active

    # Manning land classes: streets 0.015, else urban/grass/vegetation by a field
    lfield = gaussian_random_field(rng, (-radius - 10, -radius - 10), 2 * radius + 20, 50.0, 300.0, 1.0)(cx, cy)
    q1, q2 = np.quantile(lfield, [0.55, 0.85])
    manning = np.where(lfield < q1, 0.035, np.where(lfield < q2, 0.06, 0.1))
    manning = np.where(road, 0.015, manning).astype(np.float32)
    pervious = manning >= 0.06

    surface = build_triangular_surface_topology(pts, tri, bed, manning, active.astype(np.float32), "outflow")
    if surface.edge_count != n_edges:
        raise RuntimeError(f"mesh has {surface.edge_count} edges, expected {n_edges}")

    f0 = np.where(pervious, 75.0, 0.0)
    fc = np.where(pervious, 10.0, 0.0)
    fields = ProductionInfiltrationFields(
        rainfall_multiplier=np.ones(c, np.float32),
        horton_f0_mps=(f0 * MMHR_TO_MPS).astype(np.float32),
        horton_fc_mps=(fc * MMHR_TO_MPS).astype(np.float32),
        horton_k_per_s=np.full(c, 4.0 / 3600.0, dtype=np.float32),
        open_fraction=np.ones(c, np.float32),
        active_mask=active.copy(),
    )

    coupling, pipe, pipe_state = _drainage(
        rng, pts, tri, cen, bed, active, road, n_nodes, n_links, n_inlets, n_outfalls,
        coo_matrix, minimum_spanning_tree, Delaunay,
    )
    mesh = RealMesh(
        nodes_xy=pts, triangles=tri, centroids_xy=cen, terrain_elevation_m=bed,
        building_mask=building, road_mask=road, active_mask=active,
    )
    state = TriangularSurfaceState(np.zeros(c, np.float32), np.zeros(c, np.float32), np.zeros(c, np.float32))
    topo = ProductionTopologies(mesh, surface, coupling, pipe, state, pipe_state)
    city = CityDomain(topo, "exact_production", fields, None)
    hourly = FRONT_LOADED_24H_MMHR if hourly_mmhr is None else np.asarray(hourly_mmhr, float)
    rain = hourly_rainfall(hourly)
    overrides = {"physics.infiltration_mode": "production_horton", "solver.duration_min": duration_min}
    return Scenario(f"coupled{n_triangles}_s{seed}", city, rain, overrides)


def _drainage(rng, pts, tri, cen, bed, active, road, n_nodes, n_links, n_inlets, n_outfalls,
              coo_matrix, minimum_spanning_tree, Delaunay):
    c = tri.shape[0]
    act_idx = np.flatnonzero(active)
    weight = np.where(road[act_idx], 4.0, 1.0)
    weight = weight / weight.sum()
    node_cell = rng.choice(act_idx, size=n_nodes, replace=False, p=weight)
    node_xy = cen[node_cell] + rng.uniform(-3.0, 3.0, size=(n_nodes, 2))
    depth = rng.uniform(1.5, 3.5, size=n_nodes)
    invert = (bed[node_cell].astype(np.float64) - depth).astype(np.float32)
    max_depth = depth.astype(np.float32)
    storage = rng.uniform(1.0, 4.0, size=n_nodes).astype(np.float32)
    fill = rng.uniform(0.0, 0.15, size=n_nodes).astype(np.float32)

    # spanning tree over the node Delaunay graph, plus short loop links
    dtri = Delaunay(node_xy).simplices
    e = np.concatenate([dtri[:, [0, 1]], dtri[:, [1, 2]], dtri[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    length = np.hypot(*(node_xy[e[:, 0]] - node_xy[e[:, 1]]).T)
    g = coo_matrix((length + 1e-9, (e[:, 0], e[:, 1])), shape=(n_nodes, n_nodes))
    mst = minimum_spanning_tree(g).tocoo()
    tree = np.stack([mst.row, mst.col], axis=1)
    if tree.shape[0] != n_nodes - 1:
        raise RuntimeError("node graph is not connected")
    tree_key = set(map(tuple, np.sort(tree, axis=1).tolist()))
    is_tree = np.array([tuple(x) in tree_key for x in e.tolist()])
    extra_pool = np.flatnonzero(~is_tree)
    extra_pool = extra_pool[np.argsort(length[extra_pool])][: max(len(extra_pool) * 2 // 5, n_links - tree.shape[0])]
    n_extra = n_links - tree.shape[0]
    extra = e[rng.choice(extra_pool, size=n_extra, replace=False)]
    links = np.concatenate([np.sort(tree, axis=1), extra])
    a, b = links[:, 0], links[:, 1]
    hi_first = invert[a] >= invert[b]
    frm = np.where(hi_first, a, b).astype(np.int32)
    to = np.where(hi_first, b, a).astype(np.int32)
    llen = np.maximum(np.hypot(*(node_xy[frm] - node_xy[to]).T), 1.0).astype(np.float32)
    diam = np.clip(np.exp(rng.normal(np.log(0.6), 0.45, size=n_links)), 0.3, 2.4).astype(np.float32)
    area = (0.25 * np.pi * diam.astype(np.float64) ** 2).astype(np.float32)
    radius = (diam / 4.0).astype(np.float32)
    nman = np.full(n_links, 0.013, np.float32)
    slope = np.maximum(np.abs(invert[frm].astype(float) - invert[to]) / llen, 1e-3)
    cap = (2.0 / 0.013 * area * (diam / 4.0) ** (2.0 / 3.0) * np.sqrt(slope)).astype(np.float32)
    minor = np.full(n_links, 0.3, np.float32)

    # inlets: mostly one per node, some nodes with two; cell = node cell or a neighbour
    base = rng.choice(n_nodes, size=n_inlets, replace=n_inlets > n_nodes)
    dup = rng.random(n_inlets) < 0.08
    base[dup] = rng.choice(n_nodes, size=int(dup.sum()))
    inlet_node = base.astype(np.int32)
    inlet_cell = node_cell[inlet_node].copy()
    move = rng.random(n_inlets) < 0.3
    if move.any():
        from scipy.spatial import cKDTree

        tree_c = cKDTree(cen[act_idx])
        _, nn = tree_c.query(cen[inlet_cell[move]], k=4)
        pick = nn[np.arange(nn.shape[0]), rng.integers(1, 4, size=nn.shape[0])]
        inlet_cell[move] = act_idx[pick]
    inlet_cell = inlet_cell.astype(np.int32)
    cap_in = rng.uniform(0.05, 0.3, size=n_inlets).astype(np.float32)
    sur_in = rng.uniform(0.05, 0.3, size=n_inlets).astype(np.float32)

    out_nodes = np.argsort(invert, kind="stable")[:n_outfalls]
    oa = np.zeros(n_nodes, np.float32)
    oc = np.zeros(n_nodes, np.float32)
    ot = invert.copy()
    oa[out_nodes] = np.float32(0.25 * np.pi * 1.2 * 1.2)
    oc[out_nodes] = np.float32(0.62)

    coupling = TriangularNodeCouplingTopology(
        inlet_cell_index=inlet_cell,
        inlet_node_index=inlet_node,
        node_surface_cell_index=node_cell.astype(np.int32),
        node_invert_elevation_m=invert,
        node_storage_area_m2=storage,
        node_max_depth_m=max_depth,
        node_initial_fill_depth_m=fill,
        inlet_capture_capacity_m3ps=cap_in,
        inlet_surcharge_capacity_m3ps=sur_in,
        node_x_m=node_xy[:, 0].astype(np.float32),
        node_y_m=node_xy[:, 1].astype(np.float32),
    )
    pipe = TriangularPipeNetworkTopology(
        link_from_node_index=frm,
        link_to_node_index=to,
        link_length_m=llen,
        link_area_m2=area,
        link_hydraulic_radius_m=radius,
        link_manning_n=nman,
        link_flow_capacity_m3ps=cap,
        outfall_area_m2=oa,
        outfall_coefficient=oc,
        outfall_tailwater_head_m=ot,
        link_diameter_m=diam,
        link_minor_loss_coefficient=minor,
    )
    volume = storage.astype(np.float64) * fill.astype(np.float64)
    state = TriangularPipeNetworkState(node_volume_m3=volume, link_flow_m3ps=np.zeros(n_links, np.float64))
    return coupling, pipe, state


# ---------------------------------------------------------------------------
# external boundary inflow and surface recharge
# ---------------------------------------------------------------------------

def add_boundary_forcing(sc: Scenario, n_receivers: int = 6, n_recharge: int = 40, seed: int = 0,
                         peak_m3ps: float = 2.0, step_s: float = 300.0) -> Scenario:
    """Seeded external inflow and recharge rows on a scenario's city.

    Receivers sit on active cells nearest the upstream (low-x) edge, two of
    them on one cell; each hydrograph is triangular with a random peak up to
    ``peak_m3ps`` at ``step_s`` spacing over the run (plus one step).
    Recharge rows sit on random active cells (two rows share a cell), with
    storage 5-500 m^3, capture 0.01-0.5 m^3/s, recharge 0.001-0.05 m^3/s,
    stop depth 1-5 cm and activation depth 5 cm (the reference's default).
    """

    from .domain import ExternalBoundaryInflowSurface, June5RechargeTopology

    rng = np.random.default_rng(seed)
    mesh = sc.city.mesh
    active = np.flatnonzero(np.asarray(mesh.active_mask, bool))
    dur_s = float(sc.overrides.get("solver.duration_min") or sc.rainfall.duration_min) * 60.0
    if n_receivers > 0:
        x = np.asarray(mesh.centroids_xy)[active, 0]
        near = active[np.argsort(x, kind="stable")[: max(4 * n_receivers, 8)]]
        cells = rng.choice(near, size=n_receivers, replace=False).astype(np.int32)
        if n_receivers > 1:
            cells[1] = cells[0]
        times = np.arange(0.0, dur_s + 2 * step_s, step_s)
        q = np.zeros((times.size, n_receivers), np.float32)
        for j in range(n_receivers):
            peak = rng.uniform(0.1, 1.0) * peak_m3ps
            tp = rng.uniform(0.2, 0.6) * dur_s
            shape = np.where(times <= tp, times / max(tp, 1.0), np.maximum(0.0, 1.0 - (times - tp) / max(dur_s - tp, 1.0)))
            q[:, j] = (peak * shape).astype(np.float32)
        sc.city.external_boundary = ExternalBoundaryInflowSurface(
            receiver_cell_index=cells, times_s=times.astype(np.float64), q_m3ps_by_receiver=q,
            peak_total_m3ps=float(q.sum(axis=1).max()))
    if n_recharge > 0:
        cells = rng.choice(active, size=n_recharge, replace=False).astype(np.int32)
        if n_recharge > 2:
            cells[2] = cells[1]
        sc.city.recharge_topology = June5RechargeTopology(
            source_cell_index=cells, overflow_cell_index=cells.copy(),
            storage_capacity_m3=rng.uniform(5.0, 500.0, n_recharge).astype(np.float32),
            capture_capacity_m3ps=rng.uniform(0.01, 0.5, n_recharge).astype(np.float32),
            recharge_capacity_m3ps=rng.uniform(0.001, 0.05, n_recharge).astype(np.float32),
            activation_depth_m=np.full(n_recharge, 0.05, np.float32),
            stop_depth_m=rng.uniform(0.01, 0.05, n_recharge).astype(np.float32))
    return sc


def add_surcharge_table(sc: Scenario, frac: float = 0.6, seed: int = 0, normalized: bool = False) -> Scenario:
    """A seeded weighted surcharge-return table on a coupled scenario: ``frac``
    of the nodes get one to three entries on active cells near their own
    surface cell (weights U(0, 2), normalized per node if asked); the other
    nodes keep the per-node return to their cell."""

    from .topology import TriangularNodeCouplingTopology

    rng = np.random.default_rng(seed)
    topo = sc.city.topologies
    cp = topo.coupling_topology
    mesh = sc.city.mesh
    active = np.flatnonzero(np.asarray(mesh.active_mask, bool))
    cen = np.asarray(mesh.centroids_xy)
    nodes = np.sort(rng.choice(cp.node_count, size=int(frac * cp.node_count), replace=False))
    cells, owner, weight = [], [], []
    for n in nodes:
        c0 = int(cp.node_surface_cell_index[n])
        if c0 < 0:
            continue
        d2 = np.sum((cen[active] - cen[c0]) ** 2, axis=1)
        near = active[np.argsort(d2)[:8]]
        k = int(rng.integers(1, 4))
        w = rng.uniform(0.0, 2.0, k)
        if normalized:
            w = w / w.sum()
        cells.extend(rng.choice(near, size=k, replace=False).tolist())
        owner.extend([int(n)] * k)
        weight.extend(w.tolist())
    topo.coupling_topology = TriangularNodeCouplingTopology(**{
        **cp.__dict__, "surcharge_cell_index": np.array(cells, np.int32),
        "surcharge_node_index": np.array(owner, np.int32), "surcharge_return_weight": np.array(weight, np.float32),
        "surcharge_return_weight_is_normalized": normalized})
    return sc


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------

def small_workload(seed: int = 0) -> Scenario:
    """100 x 100 jittered grid, 50 mm/h for one hour, outflow boundary."""

    return make_grid_city(n=100, seed=seed)


def coupled_test_city(scale: int = 1, seed: int = 3, duration_min: float = 60.0) -> Scenario:
    """A small coupled city (same generator as the production-shaped one)."""

    t = 4000 * scale
    b = 180 * int(np.sqrt(scale))
    if (3 * t + b) % 2:
        b += 1
    e = (3 * t + b) // 2
    return make_coupled_city(
        n_triangles=t, n_edges=e, n_active=int(0.83 * t), n_nodes=480 * scale, n_links=565 * scale,
        n_inlets=250 * scale, n_outfalls=4, area_km2=1.2 * scale, seed=seed, duration_min=duration_min,
    )


def _cache_dir() -> Path:
    return Path(os.environ.get("FLOODGB_CACHE", "/tmp/floodgb_cache"))


def production_workload(seed: int = 1, cache: bool = True) -> Scenario:
    """981,880-triangle coupled city, hour 1 of the front-loaded 24 h event.

    Generation takes ~20 s (mostly the Delaunay triangulation); with
    ``cache`` the arrays are kept in ``$FLOODGB_CACHE`` (default
    ``/tmp/floodgb_cache``) between processes.
    """

    if not cache:
        return make_coupled_city(seed=seed)
    import pickle

    tag = hashlib.sha1(f"production-v1-{seed}".encode()).hexdigest()[:12]
    path = _cache_dir() / f"production_{tag}.pkl"
    if path.exists():
        try:
            with open(path, "rb") as fh:
                return pickle.load(fh)
        except Exception:
            pass
    sc = make_coupled_city(seed=seed)
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        with open(tmp, "wb") as fh:
            pickle.dump(sc, fh, protocol=pickle.HIGHEST_PROTOCOL)
        tmp.replace(path)
    except OSError:
        pass
    return sc


# ---------------------------------------------------------------------------
# batched ensemble: ragged meshes, seeded storms
# ---------------------------------------------------------------------------
ENSEMBLE_GRID_N = (71, 158, 224, 354)  # 10,082 / 49,928 / 100,352 / 250,632 triangles


def storm_hyetograph(rng: np.random.Generator, peak_range=(20.0, 120.0), duration_h_range=(1.0, 6.0),
                     block_min: float = 10.0) -> RainfallEvent:
    """Seeded single-peak storm: triangular intensity in 10-minute blocks,
    peak U(20, 120) mm/h at a random 20-50 % of a U(1, 6) h duration."""

    peak = float(rng.uniform(*peak_range))
    dur_min = float(np.round(rng.uniform(*duration_h_range) * 60.0 / block_min) * block_min)
    dur_min = max(dur_min, block_min)
    t_peak = float(rng.uniform(0.2, 0.5)) * dur_min
    start = np.arange(0.0, dur_min, block_min)
    mid = start + 0.5 * block_min
    rise = np.clip(mid / max(t_peak, 1e-9), 0.0, 1.0)
    fall = np.clip((dur_min - mid) / max(dur_min - t_peak, 1e-9), 0.0, 1.0)
    inten = peak * np.where(mid <= t_peak, rise, fall)
    return rainfall_event(start, start + block_min, np.round(inten, 3))


def ensemble_workload(seed: int = 2, grid_n=ENSEMBLE_GRID_N, per_size: int = 16, size_m: float = 1000.0,
                      duration_cap_h: float | None = None) -> list:
    """Batched-ensemble members (mesh size cycles through grid_n, per_size each):
    jittered-grid cities like the 20,000-triangle case with their own seeded
    random-field beds and seeded storms; each runs for its storm's duration
    (capped at duration_cap_h when given)."""

    from .batch import Member

    rng = np.random.default_rng(seed)
    members = []
    for n in grid_n:
        for k in range(per_size):
            mseed = int(rng.integers(1 << 30))
            storm = storm_hyetograph(np.random.default_rng(mseed + 7))
            dur_min = storm.duration_min if duration_cap_h is None else min(storm.duration_min, duration_cap_h * 60.0)
            sc = make_grid_city(n=n, size_m=size_m, seed=mseed, hyetograph=storm, duration_min=dur_min)
            cfg = load_config(None, sc.overrides)
            members.append(Member(sc.city, sc.rainfall, cfg, dur_min * 60.0))
    return members
