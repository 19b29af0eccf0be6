"""Generate the golden fixtures from the reference's own NumPy code path.

Run from the repository root in a container that has the reference checkout:

    python tests/golden/make_golden.py <reference checkout> [--only=surface,pipe,run,forcing,li,topology,outputs]

(or with the checkout in $FLOODGB_REFERENCE).

The reference package ``gurugram_flood`` cannot be imported normally here
(its ``__init__`` needs PyYAML and its engine needs pandas), so bare package
stubs point at its source directories and only the NumPy-capable modules are
loaded: ``kernels/triangular_backend.py`` (with ``equations.py``,
``network_kernels.py``, ``pipe_kernels.py``), ``solver/stabilizers.py`` and
``domain/production_infiltration_support.py``, plus
``domain/production_event_support.py`` (external inflow) and
``domain/june5_production_drainage.py`` (recharge) behind an empty pandas
stand-in.  The engine loop (``solver/engine.py:219-344``) is restated here on
top of those functions.

Dtype discipline follows the reference's CuPy production path: every scalar
forcing is passed as ``np.float32`` and ``h`` is cast back to float32 after the
drainage step (the CuPy fused kernels keep the surface state float32 where
the NumPy drainage path would promote it to float64).

The fixtures are small ``.npz`` files committed next to this script; tests
read only the fixtures, never the reference.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "gpu-urban-flood-cupy-jax_gb300"))


def import_reference(ref_root: Path):
    src = ref_root / "HF_CUPY_JAX_COMPLETED_PROJECT" / "reproduction" / "source" / "src" / "gurugram_flood"
    for name, sub in (("gurugram_flood", ""), ("gurugram_flood.kernels", "kernels"),
                      ("gurugram_flood.domain", "domain"), ("gurugram_flood.solver", "solver")):
        mod = types.ModuleType(name)
        mod.__path__ = [str(src / sub) if sub else str(src)]
        sys.modules[name] = mod
    import gurugram_flood.domain.production_infiltration_support as pis
    import gurugram_flood.kernels.triangular_backend as tb
    import gurugram_flood.solver.stabilizers as stab

    return tb, stab, pis


def import_reference_forcing():
    """The reference's inflow and recharge modules.  Both import pandas at
    module level (for their CSV loaders, which are not called here); pandas is
    absent in this container, so an empty stand-in module satisfies the import."""

    sys.modules.setdefault("pandas", types.ModuleType("pandas"))
    import gurugram_flood.domain.june5_production_drainage as j5
    import gurugram_flood.domain.production_event_support as pes

    return pes, j5


def topo_arrays(prefix, st):
    return {
        f"{prefix}bed": st.bed_elevation_m, f"{prefix}manning": st.manning_n, f"{prefix}area": st.cell_area_m2,
        f"{prefix}char_len": st.characteristic_length_m, f"{prefix}left": st.edge_left_cell,
        f"{prefix}right": st.edge_right_cell, f"{prefix}nx": st.edge_normal_x, f"{prefix}ny": st.edge_normal_y,
        f"{prefix}len": st.edge_length_m, f"{prefix}bcode": st.boundary_code,
        f"{prefix}active": st.active_mask if st.active_mask is not None else np.ones(st.cell_count, np.float32),
        f"{prefix}has_active": np.int32(st.active_mask is not None),
        f"{prefix}has_stage": np.int32(st.has_stage_boundary),
    }


def coupling_arrays(prefix, cp, pp):
    out = {}
    for name in ("inlet_cell_index", "inlet_node_index", "node_surface_cell_index", "node_invert_elevation_m",
                 "node_storage_area_m2", "node_max_depth_m", "inlet_capture_capacity_m3ps",
                 "inlet_surcharge_capacity_m3ps", "surcharge_cell_index", "surcharge_node_index",
                 "surcharge_return_weight"):
        v = getattr(cp, name)
        if v is not None:
            out[f"{prefix}{name}"] = np.asarray(v)
    if cp.surcharge_cell_index is not None:
        out[f"{prefix}surcharge_return_weight_is_normalized"] = np.int32(cp.surcharge_return_weight_is_normalized)
    for name in ("link_from_node_index", "link_to_node_index", "link_length_m", "link_area_m2",
                 "link_hydraulic_radius_m", "link_manning_n", "link_flow_capacity_m3ps", "outfall_area_m2",
                 "outfall_coefficient", "outfall_tailwater_head_m", "outfall_flow_capacity_m3ps",
                 "link_invert_elevation_m", "link_diameter_m", "link_minor_loss_coefficient", "link_geometry_code",
                 "link_rect_width_m", "link_rect_height_m"):
        v = getattr(pp, name)
        if v is not None:
            out[f"{prefix}{name}"] = np.asarray(v)
    return out


def random_state(rng, n, wet_frac=0.7, hmax=0.6):
    h = rng.uniform(0.0, hmax, n).astype(np.float32)
    dry = rng.random(n) > wet_frac
    h[dry] = 0.0
    tiny = rng.random(n) < 0.05
    h[tiny] = np.float32(3e-6)
    u = rng.uniform(-1.5, 1.5, n).astype(np.float32)
    v = rng.uniform(-1.5, 1.5, n).astype(np.float32)
    return h, (h * u).astype(np.float32), (h * v).astype(np.float32)


def grid_topology(tb, rng, n=12, mode="outflow", active_frac=0.85):
    from floodgb.synthetic import grid_mesh

    pts, tris = grid_mesh(n, 10.0 * n, 0.2, rng)
    cen = pts[tris].mean(axis=1)
    bed = (0.01 * cen[:, 0] + rng.normal(0, 0.05, len(tris))).astype(np.float32)
    manning = rng.choice([0.015, 0.035, 0.06], len(tris)).astype(np.float32)
    active = (rng.random(len(tris)) < active_frac).astype(np.float32)
    return tb.build_triangular_surface_topology(pts, tris, bed, manning, active, mode), pts, tris


def with_mixed_codes(tb, st, rng, stage):
    code = np.array(st.boundary_code, copy=True)
    ext = np.flatnonzero(np.asarray(st.edge_right_cell) < 0)
    code[ext] = rng.choice([0, 1, 2, 3, 4], ext.size)
    return tb.TriangularSurfaceTopology(
        **{**st.__dict__, "boundary_code": code.astype(np.int32), "has_stage_boundary": True}
    )


def make_surface_cases(tb, stab):
    rng = np.random.default_rng(20261203)
    out = {}
    cases = []
    st, pts, tris = grid_topology(tb, rng)
    out["topo_nodes"] = pts
    out["topo_triangles"] = tris
    out["topo_bed"] = np.asarray(st.bed_elevation_m)
    out["topo_manning"] = np.asarray(st.manning_n)
    out["topo_active"] = np.asarray(st.active_mask)
    stage = float(np.mean(st.bed_elevation_m) + 0.25)
    mixed = with_mixed_codes(tb, st, rng, stage)
    cases.append(("mixed_scalar", mixed, stage, np.float32(50.0 / 3.6e6), np.float32(10.0 / 3.6e6), 0.7))
    cases.append(("outflow_percell", st, None,
                  (rng.uniform(0, 80, st.cell_count) / 3.6e6).astype(np.float32),
                  (rng.uniform(0, 120, st.cell_count) / 3.6e6).astype(np.float32), 0.25))
    st2, _, _ = grid_topology(tb, rng, n=10, mode="reflective", active_frac=1.0)
    st2 = tb.TriangularSurfaceTopology(**{**st2.__dict__, "active_mask": None})
    cases.append(("reflective_nomask", st2, None, np.float32(0.0), np.float32(0.0), 0.9))
    st3, _, _ = grid_topology(tb, rng, n=10, mode="transmissive", active_frac=0.9)
    cases.append(("transmissive_scalar", st3, None, np.float32(20.0 / 3.6e6), np.float32(0.0), 0.05))
    names = []
    for name, topo, stg, rain, infil, dt in cases:
        h, hu, hv = random_state(rng, topo.cell_count)
        state = tb.TriangularSurfaceState(h, hu, hv)
        forcing = tb.TriangularSurfaceForcing(rainfall_rate_mps=rain, infiltration_capacity_mps=infil,
                                              boundary_stage_m=stg)
        new, diag = tb.step_triangular_surface(state, topo, forcing, dt)
        assert new.h_m.dtype == np.float32
        clamped = stab.clamp_velocity(new, 5.0, np)
        p = f"{name}/"
        out.update(topo_arrays(p, topo))
        out[f"{p}stage"] = np.float64(stg if stg is not None else np.nan)
        out[f"{p}h"], out[f"{p}hu"], out[f"{p}hv"] = h, hu, hv
        out[f"{p}rain"] = np.asarray(rain)
        out[f"{p}infil"] = np.asarray(infil)
        out[f"{p}dt"] = np.float64(dt)
        out[f"{p}h_out"], out[f"{p}hu_out"], out[f"{p}hv_out"] = new.h_m, new.hu_m2ps, new.hv_m2ps
        out[f"{p}hu_clamped"], out[f"{p}hv_clamped"] = clamped.hu_m2ps, clamped.hv_m2ps
        out[f"{p}diag"] = np.array([
            float(diag.rainfall_input_m3), float(diag.infiltration_loss_m3), float(diag.boundary_net_flux_m3),
            float(diag.boundary_inflow_m3), float(diag.boundary_outflow_m3), float(diag.final_surface_volume_m3),
        ])
        out[f"{p}dt_cfl"] = np.float64(tb.stable_triangular_timestep_s(topo, state, cfl=0.85))
        names.append(name)
    out["cases"] = np.array(names)
    np.savez_compressed(OUT / "surface_cases.npz", **out)
    return names


def tiny_coupled(seed=5):
    from floodgb.synthetic import make_coupled_city

    t = 700
    b = 60
    e = (3 * t + b) // 2
    return make_coupled_city(n_triangles=t, n_edges=e, n_active=560, n_nodes=90, n_links=104, n_inlets=70,
                             n_outfalls=3, area_km2=0.25, seed=seed, duration_min=3.0)


def surcharge_table(tb, cp, st, rng, normalized: bool):
    """A weighted surcharge-return table on a coupling topology: about 60 % of
    nodes with one to three entries on random active cells (some sharing a
    cell), a few invalid entries (node or cell -1), zero and negative weights."""

    active = np.flatnonzero(np.asarray(st.active_mask) > 0.5)
    nodes = rng.choice(cp.node_count, size=int(0.6 * cp.node_count), replace=False)
    cells, owner, weight = [], [], []
    for n in nodes:
        k = int(rng.integers(1, 4))
        cells.extend(rng.choice(active, size=k).tolist())
        owner.extend([int(n)] * k)
        w = rng.uniform(0.0, 2.0, k)
        if normalized:
            w = (w / w.sum()).astype(np.float32)
        weight.extend(w.tolist())
    cells, owner = np.array(cells, np.int32), np.array(owner, np.int32)
    weight = np.array(weight, np.float32)
    order = rng.permutation(cells.size)
    cells, owner, weight = cells[order], owner[order], weight[order]
    if not normalized:
        weight[::11] = 0.0
        weight[5::17] = -0.5
    cells[3::23] = -1
    owner[7::29] = -1
    return tb.TriangularNodeCouplingTopology(**{
        **cp.__dict__, "surcharge_cell_index": cells, "surcharge_node_index": owner,
        "surcharge_return_weight": weight, "surcharge_return_weight_is_normalized": normalized})


def make_pipe_cases(tb):
    rng = np.random.default_rng(77)
    sc = tiny_coupled()
    topo = sc.city.topologies
    st, cp, pp = topo.surface_topology, topo.coupling_topology, topo.pipe_topology
    out = topo_arrays("mesh/", st)
    variants = []
    variants.append(("circular_orifice", pp, "orifice"))
    variants.append(("circular_weir", pp, "weir_orifice"))
    variants.append(("circular_capacity", pp, "capacity"))
    variants.append(("circular_headlimited", pp, "head_limited_capacity"))
    pre = tb.TriangularPipeNetworkTopology(**{**pp.__dict__, "link_diameter_m": None, "link_minor_loss_coefficient": None})
    variants.append(("precomputed_orifice", pre, "orifice"))
    L = pp.link_count
    geom = np.where(rng.random(L) < 0.4, 2, 1).astype(np.int32)
    inv = np.minimum(cp.node_invert_elevation_m[pp.link_from_node_index],
                     cp.node_invert_elevation_m[pp.link_to_node_index]).astype(np.float32) + np.float32(0.05)
    rect = tb.TriangularPipeNetworkTopology(**{
        **pp.__dict__, "link_geometry_code": geom, "link_rect_width_m": rng.uniform(0.5, 2.0, L).astype(np.float32),
        "link_rect_height_m": rng.uniform(0.4, 1.5, L).astype(np.float32), "link_invert_elevation_m": inv,
        "outfall_flow_capacity_m3ps": np.full(cp.node_count, 0.3, np.float32)})
    variants.append(("rect_invert_orifice", rect, "orifice"))
    trng = np.random.default_rng(78)  # its own stream: the cases above keep their inputs
    variants.append(("table_orifice", pp, "orifice", surcharge_table(tb, cp, st, trng, normalized=False)))
    variants.append(("table_normalized_capacity", pp, "capacity", surcharge_table(tb, cp, st, trng, normalized=True)))
    names = []
    base_cp = cp
    for name, pipe, rule, *alt in variants:
        cp = alt[0] if alt else base_cp
        h = rng.uniform(0.0, 0.4, st.cell_count).astype(np.float32)
        h[rng.random(st.cell_count) < 0.3] = 0.0
        if st.active_mask is not None:
            h = np.where(st.active_mask > 0.5, h, 0.0).astype(np.float32)
        V = (cp.node_storage_area_m2.astype(np.float64) * cp.node_max_depth_m.astype(np.float64)
             * rng.uniform(0.0, 1.3, cp.node_count))
        Q = rng.uniform(-0.5, 0.5, pipe.link_count)
        dt = 0.6
        h_new, state, diag = tb.step_triangular_dynamic_pipe_network(
            h, st, cp, pipe, tb.TriangularPipeNetworkState(V.copy(), Q.copy()), dt, inlet_capture_rule=rule)
        p = f"{name}/"
        out.update(coupling_arrays(p, cp, pipe))
        out[f"{p}rule"] = np.array(rule)
        out[f"{p}h"], out[f"{p}V"], out[f"{p}Q"], out[f"{p}dt"] = h, V, Q, np.float64(dt)
        out[f"{p}h_out"] = np.asarray(h_new, dtype=np.float64)
        out[f"{p}V_out"] = np.asarray(state.node_volume_m3)
        out[f"{p}Q_out"] = np.asarray(state.link_flow_m3ps)
        out[f"{p}diag"] = np.array([
            float(diag.surface_capture_m3), float(diag.surface_surcharge_m3), float(diag.link_abs_flow_m3),
            float(diag.outfall_discharge_m3), float(diag.overflow_surcharge_m3), float(diag.unreturned_overflow_m3),
            float(diag.final_node_volume_m3),
        ])
        names.append(name)
    out["cases"] = np.array(names)
    np.savez_compressed(OUT / "pipe_cases.npz", **out)
    return names


def reference_run(tb, stab, pis, sc, max_steps, snapshot_interval_s, extra=None, li=False):
    """engine.py:219-344 restated on the reference's NumPy step functions;
    ``extra`` = (production_event_support, june5_production_drainage) adds
    the external inflow and recharge steps (engine.py:263-289)."""

    from floodgb.config import load_config

    cfg = load_config(None, sc.overrides)
    s = cfg.solver
    topo = sc.city.topologies
    st, cp, pp = topo.surface_topology, topo.coupling_topology, topo.pipe_topology
    fields = sc.city.infiltration_fields
    if fields is not None:
        fields = pis.ProductionInfiltrationFields(
            rainfall_multiplier=fields.rainfall_multiplier, horton_f0_mps=fields.horton_f0_mps,
            horton_fc_mps=fields.horton_fc_mps, horton_k_per_s=fields.horton_k_per_s,
            open_fraction=fields.open_fraction, active_mask=fields.active_mask)
    mode = cfg.physics.infiltration_mode
    state = tb.TriangularSurfaceState(np.array(topo.surface_state.h_m, np.float32),
                                      np.array(topo.surface_state.hu_m2ps, np.float32),
                                      np.array(topo.surface_state.hv_m2ps, np.float32))
    pstate = tb.TriangularPipeNetworkState(np.array(topo.pipe_state.node_volume_m3, np.float64),
                                           np.array(topo.pipe_state.link_flow_m3ps, np.float64))
    wet = np.zeros(st.cell_count, np.float32)
    final_t = (s.duration_min if s.duration_min is not None else sc.rainfall.duration_min) * 60.0
    t = 0.0
    step = 0
    cached = None
    next_snap = 0.0
    snaps_t, snaps_h, snaps_hu, snaps_hv, snaps_v = [], [], [], [], []
    cum = np.zeros(9)
    has_drain = cp.node_count > 0
    ext = rch = rstore = None
    if extra is not None:
        pes, j5 = extra
        e = sc.city.external_boundary
        if e is not None:
            ext = pes.ExternalBoundaryInflowSurface(
                receiver_cell_index=np.asarray(e.receiver_cell_index, np.int32), times_s=np.asarray(e.times_s, np.float64),
                q_m3ps_by_receiver=np.asarray(e.q_m3ps_by_receiver, np.float32), peak_total_m3ps=0.0, report={})
        r = sc.city.recharge_topology
        if r is not None:
            rch = j5.recharge_to_backend(j5.June5RechargeTopology(
                source_cell_index=r.source_cell_index, overflow_cell_index=r.overflow_cell_index,
                storage_capacity_m3=r.storage_capacity_m3, capture_capacity_m3ps=r.capture_capacity_m3ps,
                recharge_capacity_m3ps=r.recharge_capacity_m3ps, activation_depth_m=r.activation_depth_m,
                stop_depth_m=r.stop_depth_m), np)
            rstore = np.zeros(r.source_cell_index.size, np.float32)
    while t < final_t and step < max_steps:
        if cached is None or step % s.cfl_update_interval_steps == 0:
            if li:
                dt = float(tb.stable_local_inertial_triangular_timestep_s(st, state, cfl=s.cfl))
            else:
                dt = float(tb.stable_triangular_timestep_s(st, state, cfl=s.cfl))
            cached = dt
        else:
            dt = cached * s.cfl_reuse_safety_factor
        dt = min(dt, s.max_dt_s, final_t - t)
        dt = max(dt, 1.0e-3)
        base = sc.rainfall.rate_fn(t)
        if mode == "production_horton" and fields is not None:
            rain = pis.rainfall_rate_for_step(xp=np, base_rainfall_rate_mps=base, mode=mode, fields=fields)
            infil = pis.build_infiltration_capacity_for_step(xp=np, mode=mode, wet_time_s=wet, fields=fields,
                                                             fallback_capacity_mps=None)
        else:
            rain = np.float32(base)
            infil = np.float32(0.0)
        forcing = tb.TriangularSurfaceForcing(rainfall_rate_mps=rain, infiltration_capacity_mps=infil)
        if li:
            state, sd = tb.step_triangular_surface_local_inertial(state, st, forcing, timestep_s=dt)
            state = tb.TriangularSurfaceState(np.asarray(state.h_m, np.float32), np.asarray(state.hu_m2ps, np.float32),
                                              np.asarray(state.hv_m2ps, np.float32))
        else:
            state, sd = tb.step_triangular_surface(state, st, forcing, timestep_s=dt)
        state = stab.clamp_velocity(state, s.max_speed_mps, np)
        od = us = 0.0
        ov = 0.0
        ea = rc = rl = 0.0
        if ext is not None:
            hx, added = pes.apply_external_boundary_inflow_depth(state.h_m, st.cell_area_m2, ext, timestep_s=dt,
                                                                 time_s=t + 0.5 * dt, xp=np)
            assert hx.dtype == np.float32
            state = tb.TriangularSurfaceState(hx, state.hu_m2ps, state.hv_m2ps)
            ea = float(added)
        if has_drain:
            h, pstate, pd = tb.step_triangular_dynamic_pipe_network(state.h_m, st, cp, pp, pstate, dt)
            state = tb.TriangularSurfaceState(np.asarray(h, np.float32), state.hu_m2ps, state.hv_m2ps)
            od, ov, us = float(pd.outfall_discharge_m3), float(pd.overflow_surcharge_m3), float(pd.unreturned_overflow_m3)
        if rch is not None:
            hr, rstore, c_m3, l_m3 = j5.apply_june5_surface_recharge(state.h_m, rch, rstore, st.cell_area_m2, dt, np)
            assert hr.dtype == np.float32 and rstore.dtype == np.float32
            state = tb.TriangularSurfaceState(hr, state.hu_m2ps, state.hv_m2ps)
            rc, rl = float(c_m3), float(l_m3)
        wet = wet + pis.wet_time_increment_s(xp=np, depth_m=state.h_m, dt_s=dt, min_depth_m=1e-5)
        cum += [float(sd.rainfall_input_m3), float(sd.infiltration_loss_m3), float(sd.boundary_net_flux_m3), od, ov, us,
                ea, rc, rl]
        t += dt
        step += 1
        if t >= next_snap or t >= final_t:
            snaps_t.append(t)
            snaps_h.append(np.array(state.h_m, np.float32))
            snaps_hu.append(np.array(state.hu_m2ps, np.float32))
            snaps_hv.append(np.array(state.hv_m2ps, np.float32))
            snaps_v.append(np.array(pstate.node_volume_m3, np.float32))
            next_snap += snapshot_interval_s
    return dict(step_count=np.int64(step), t_end=np.float64(t), snap_t=np.array(snaps_t), snap_h=np.array(snaps_h),
                snap_hu=np.array(snaps_hu), snap_hv=np.array(snaps_hv),
                snap_v=np.array(snaps_v) if has_drain else np.zeros((len(snaps_t), 0), np.float32),
                ledger=cum[:6] if extra is None else cum,
                final_V=np.asarray(pstate.node_volume_m3), final_Q=np.asarray(pstate.link_flow_m3ps),
                wet_time=wet, **({} if rstore is None else {"recharge_storage": np.asarray(rstore)}))


def scenario_arrays(prefix, sc):
    """Every input array of a scenario, so tests can rebuild it without the generator."""

    topo = sc.city.topologies
    out = topo_arrays(prefix + "mesh/", topo.surface_topology)
    out.update(coupling_arrays(prefix + "net/", topo.coupling_topology, topo.pipe_topology))
    out[prefix + "h0"] = np.asarray(topo.surface_state.h_m, np.float32)
    out[prefix + "hu0"] = np.asarray(topo.surface_state.hu_m2ps, np.float32)
    out[prefix + "hv0"] = np.asarray(topo.surface_state.hv_m2ps, np.float32)
    out[prefix + "V0"] = np.asarray(topo.pipe_state.node_volume_m3, np.float64)
    out[prefix + "Q0"] = np.asarray(topo.pipe_state.link_flow_m3ps, np.float64)
    out[prefix + "centroids"] = np.asarray(sc.city.mesh.centroids_xy)
    f = sc.city.infiltration_fields
    if f is not None:
        out[prefix + "rain_mult"] = f.rainfall_multiplier
        out[prefix + "f0"] = f.horton_f0_mps
        out[prefix + "fc"] = f.horton_fc_mps
        out[prefix + "k"] = f.horton_k_per_s
    r = sc.rainfall
    out[prefix + "hyeto"] = np.stack([r.start_min, r.end_min, r.intensity_mmhr])
    out[prefix + "overrides"] = np.array(repr(sorted(sc.overrides.items())))
    return out


def make_run_cases(tb, stab, pis):
    from floodgb.synthetic import make_grid_city

    out = {}
    sc = tiny_coupled(seed=9)
    sc.overrides["solver.snapshot_interval_min"] = 0.5
    sc.overrides["solver.duration_min"] = 3.0
    # a wetter start so drainage, Horton decay and the clamp all act
    st = sc.city.topologies.surface_topology
    rng = np.random.default_rng(11)
    h0 = np.where(st.active_mask > 0.5, rng.uniform(0, 0.3, st.cell_count), 0).astype(np.float32)
    topo = sc.city.topologies
    topo.surface_state = tb.TriangularSurfaceState(h0, np.zeros_like(h0), np.zeros_like(h0))
    out.update(scenario_arrays("coupled/", sc))
    res = reference_run(tb, stab, pis, sc, max_steps=400, snapshot_interval_s=30.0)
    out.update({f"coupled/{k}": v for k, v in res.items()})
    gsc = make_grid_city(n=20, size_m=200.0, seed=4, rain_mmhr=80.0, duration_min=4.0)
    gsc.overrides["solver.snapshot_interval_min"] = 1.0
    out.update(scenario_arrays("grid/", gsc))
    res = reference_run(tb, stab, pis, gsc, max_steps=100000, snapshot_interval_s=60.0)
    out.update({f"grid/{k}": v for k, v in res.items()})
    np.savez_compressed(OUT / "run_cases.npz", **out)


def make_li_cases(tb, stab, pis):
    """Local-inertial steps (the reference's NumPy path, triangular_backend.py
    :531-590 and :1181-1291) and its timestep, plus two multi-step runs of the
    restated engine loop in local-inertial mode."""

    from floodgb.synthetic import make_grid_city

    rng = np.random.default_rng(20261204)
    out = {}
    names = []
    st, _, _ = grid_topology(tb, rng, n=12, mode="outflow", active_frac=0.85)
    st2, _, _ = grid_topology(tb, rng, n=10, mode="transmissive", active_frac=0.9)
    st3, _, _ = grid_topology(tb, rng, n=10, mode="reflective", active_frac=1.0)
    st3 = tb.TriangularSurfaceTopology(**{**st3.__dict__, "active_mask": None})
    cases = [
        ("outflow_scalar", st, np.float32(60.0 / 3.6e6), np.float32(5.0 / 3.6e6), 0.7),
        ("outflow_percell", st, (rng.uniform(0, 80, st.cell_count) / 3.6e6).astype(np.float32),
         (rng.uniform(0, 120, st.cell_count) / 3.6e6).astype(np.float32), 0.3),
        ("transmissive_dry", st2, np.float32(0.0), np.float32(0.0), 1.0),
        ("reflective_nomask", st3, np.float32(20.0 / 3.6e6), np.float32(0.0), 0.5),
    ]
    for name, topo, rain, infil, dt in cases:
        h, hu, hv = random_state(rng, topo.cell_count, hmax=0.4)
        if name == "transmissive_dry":
            h[rng.random(topo.cell_count) < 0.5] = 0.0
        state = tb.TriangularSurfaceState(h, hu, hv)
        forcing = tb.TriangularSurfaceForcing(rainfall_rate_mps=rain, infiltration_capacity_mps=infil)
        new, diag = tb.step_triangular_surface_local_inertial(state, topo, forcing, dt)
        p = f"{name}/"
        out.update(topo_arrays(p, topo))
        out[f"{p}h"], out[f"{p}hu"], out[f"{p}hv"] = h, hu, hv
        out[f"{p}rain"], out[f"{p}infil"], out[f"{p}dt"] = np.asarray(rain), np.asarray(infil), np.float64(dt)
        out[f"{p}h_out"] = np.asarray(new.h_m, np.float32)
        out[f"{p}hu_out"] = np.asarray(new.hu_m2ps, np.float32)
        out[f"{p}hv_out"] = np.asarray(new.hv_m2ps, np.float32)
        out[f"{p}diag"] = np.array([
            float(diag.rainfall_input_m3), float(diag.infiltration_loss_m3), float(diag.boundary_net_flux_m3),
            float(diag.boundary_inflow_m3), float(diag.boundary_outflow_m3), float(diag.final_surface_volume_m3)])
        out[f"{p}dt_li"] = np.float64(tb.stable_local_inertial_triangular_timestep_s(topo, state, cfl=0.85))
        names.append(name)
    out["cases"] = np.array(names)
    sc = tiny_coupled(seed=21)
    sc.overrides["solver.snapshot_interval_min"] = 0.5
    sc.overrides["solver.duration_min"] = 3.0
    sc.overrides["solver.surface_step_mode"] = "local_inertial"
    st4 = sc.city.topologies.surface_topology
    rng2 = np.random.default_rng(14)
    h0 = np.where(st4.active_mask > 0.5, rng2.uniform(0, 0.3, st4.cell_count), 0).astype(np.float32)
    sc.city.topologies.surface_state = tb.TriangularSurfaceState(h0, np.zeros_like(h0), np.zeros_like(h0))
    out.update(scenario_arrays("coupled/", sc))
    res = reference_run(tb, stab, pis, sc, max_steps=400, snapshot_interval_s=30.0, li=True)
    out.update({f"coupled/{k}": v for k, v in res.items()})
    gsc = make_grid_city(n=20, size_m=200.0, seed=6, rain_mmhr=80.0, duration_min=4.0)
    gsc.overrides["solver.snapshot_interval_min"] = 1.0
    gsc.overrides["solver.surface_step_mode"] = "local_inertial"
    out.update(scenario_arrays("grid/", gsc))
    res = reference_run(tb, stab, pis, gsc, max_steps=100000, snapshot_interval_s=60.0, li=True)
    out.update({f"grid/{k}": v for k, v in res.items()})
    np.savez_compressed(OUT / "li_cases.npz", **out)
    return names


def forcing_arrays(prefix, city):
    out = {}
    e = city.external_boundary
    if e is not None:
        out[prefix + "ext_cells"] = np.asarray(e.receiver_cell_index, np.int32)
        out[prefix + "ext_times"] = np.asarray(e.times_s, np.float64)
        out[prefix + "ext_q"] = np.asarray(e.q_m3ps_by_receiver, np.float32)
    r = city.recharge_topology
    if r is not None:
        for k in ("source_cell_index", "storage_capacity_m3", "capture_capacity_m3ps", "recharge_capacity_m3ps",
                  "stop_depth_m"):
            out[prefix + "rch_" + k] = np.asarray(getattr(r, k))
    return out


def make_forcing_cases(tb, stab, pis, pes, j5):
    """Inflow and recharge alone (reference functions on seeded inputs) and a
    coupled run with both."""

    from floodgb.synthetic import add_boundary_forcing

    out = {}
    rng = np.random.default_rng(31)
    sc = tiny_coupled(seed=13)
    add_boundary_forcing(sc, n_receivers=5, n_recharge=24, seed=3, peak_m3ps=1.5, step_s=20.0)
    st = sc.city.topologies.surface_topology
    area = np.asarray(st.cell_area_m2, np.float32)
    out["unit/area"] = area
    out.update(forcing_arrays("unit/", sc.city))
    e = sc.city.external_boundary
    ext = pes.ExternalBoundaryInflowSurface(receiver_cell_index=e.receiver_cell_index, times_s=e.times_s,
                                            q_m3ps_by_receiver=e.q_m3ps_by_receiver, peak_total_m3ps=0.0, report={})
    h = np.where(st.active_mask > 0.5, rng.uniform(0, 0.2, st.cell_count), 0).astype(np.float32)
    out["unit/h"] = h
    times = [-5.0, 0.0, 7.3, 20.0, 33.33, 59.99, float(e.times_s[-1]), float(e.times_s[-1]) + 100.0]
    dts = [0.5, 0.37, 1.0, 0.01, 0.85, 0.2, 0.6, 1.0]
    ext_h, ext_v, ext_q = [], [], []
    for t, dt in zip(times, dts):
        hx, added = pes.apply_external_boundary_inflow_depth(h, st.cell_area_m2, ext, timestep_s=dt, time_s=t, xp=np)
        ext_h.append(np.asarray(hx, np.float32))
        ext_v.append(float(added))
        ext_q.append(pes.external_boundary_inflow_q_m3ps(ext, t))
    out["unit/ext_time"] = np.array(times)
    out["unit/ext_dt"] = np.array(dts)
    out["unit/ext_h_out"] = np.stack(ext_h)
    out["unit/ext_added"] = np.array(ext_v)
    out["unit/ext_q_at"] = np.stack(ext_q)
    r = sc.city.recharge_topology
    rb = j5.recharge_to_backend(j5.June5RechargeTopology(
        source_cell_index=r.source_cell_index, overflow_cell_index=r.overflow_cell_index,
        storage_capacity_m3=r.storage_capacity_m3, capture_capacity_m3ps=r.capture_capacity_m3ps,
        recharge_capacity_m3ps=r.recharge_capacity_m3ps, activation_depth_m=r.activation_depth_m,
        stop_depth_m=r.stop_depth_m), np)
    # deep water on the recharge cells so capture, storage limits and losses all act
    hr = h.copy()
    hr[r.source_cell_index] = rng.uniform(0.0, 0.6, r.source_cell_index.size).astype(np.float32)
    store = np.zeros(r.source_cell_index.size, np.float32)
    store[::5] = np.asarray(r.storage_capacity_m3, np.float32)[::5] * np.float32(0.97)
    out["unit/rch_h"], out["unit/rch_storage0"] = hr.copy(), store.copy()
    rh, rs, rc, rl = [], [], [], []
    for dt in (0.9, 30.0, 5.0, 120.0):
        hr, store, c_m3, l_m3 = j5.apply_june5_surface_recharge(hr, rb, store, st.cell_area_m2, dt, np)
        rh.append(np.asarray(hr, np.float32))
        rs.append(np.asarray(store, np.float32))
        rc.append(float(c_m3))
        rl.append(float(l_m3))
    out["unit/rch_dt"] = np.array([0.9, 30.0, 5.0, 120.0])
    out["unit/rch_h_out"], out["unit/rch_storage_out"] = np.stack(rh), np.stack(rs)
    out["unit/rch_capture"], out["unit/rch_loss"] = np.array(rc), np.array(rl)

    # a coupled run with both
    run_sc = tiny_coupled(seed=9)
    run_sc.overrides["solver.snapshot_interval_min"] = 0.5
    run_sc.overrides["solver.duration_min"] = 3.0
    add_boundary_forcing(run_sc, n_receivers=4, n_recharge=20, seed=5, peak_m3ps=0.8, step_s=30.0)
    rst = run_sc.city.topologies.surface_topology
    rng2 = np.random.default_rng(12)
    h0 = np.where(rst.active_mask > 0.5, rng2.uniform(0, 0.3, rst.cell_count), 0).astype(np.float32)
    run_sc.city.topologies.surface_state = tb.TriangularSurfaceState(h0, np.zeros_like(h0), np.zeros_like(h0))
    out.update(scenario_arrays("run/", run_sc))
    out.update(forcing_arrays("run/", run_sc.city))
    res = reference_run(tb, stab, pis, run_sc, max_steps=400, snapshot_interval_s=30.0, extra=(pes, j5))
    out.update({f"run/{k}": v for k, v in res.items()})
    np.savez_compressed(OUT / "forcing_cases.npz", **out)


def make_topology_cases(tb):
    """Reference topology builds (build_triangular_surface_topology,
    triangular_backend.py:244-326, with _orient_triangles_ccw / _build_edges
    :1815-1869) on irregular meshes: seeded Delaunay triangulations with about
    half of the triangles listed clockwise, jittered grids, every boundary
    mode and some of its aliases (boundary_mode_code, :1050-1064), per-cell /
    scalar / default Manning n, with and without an active mask; and the
    ValueError text of each invalid input the builder rejects."""

    from scipy.spatial import Delaunay

    from floodgb.synthetic import grid_mesh

    rng = np.random.default_rng(20261204)
    out = {}

    def delaunay(npts, size):
        pts = np.vstack([rng.uniform(0.0, size, (npts, 2)), [[0, 0], [size, 0], [0, size], [size, size]]])
        tri = Delaunay(pts).simplices.astype(np.int64)
        flip = rng.random(len(tri)) < 0.5
        tri[flip] = tri[flip][:, [0, 2, 1]]
        return pts, tri

    def grid(n, size):
        pts, tri = grid_mesh(n, size, 0.2, rng)
        tri = np.asarray(tri, np.int64).copy()
        flip = rng.random(len(tri)) < 0.3
        tri[flip] = tri[flip][:, [1, 0, 2]]
        return pts, tri

    cases = [
        ("delaunay_outflow", delaunay(300, 400.0), "outflow", "cell", True),
        ("delaunay_closed_default_n", delaunay(200, 150.0), "closed", "none", True),
        ("delaunay_stage_scalar_n", delaunay(250, 900.0), "Dirichlet-Stage", "scalar", False),
        ("grid_reflective", grid(11, 110.0), "reflective", "cell", True),
        ("grid_open_alias", grid(9, 45.0), "open", "cell", True),
        ("grid_wall_alias", grid(7, 700.0), "wall", "scalar", False),
        ("grid_outflow_only_alias", grid(8, 80.0), "outflow_only", "cell", True),
    ]
    names = []
    for name, (pts, tri), mode, mkind, with_active in cases:
        c = len(tri)
        bed = (rng.normal(10.0, 2.0, c)).astype(np.float32)
        manning = {"cell": rng.choice([0.015, 0.035, 0.06, 0.1], c).astype(np.float32), "none": None,
                   "scalar": 0.021}[mkind]
        active = (rng.random(c) < 0.8).astype(np.float32) if with_active else None
        st = tb.build_triangular_surface_topology(pts, tri, bed, manning, active, mode)
        p = f"{name}/"
        out[p + "nodes"], out[p + "triangles"], out[p + "in_bed"] = pts, tri, bed
        out[p + "mode"] = np.array(mode)
        out[p + "manning_kind"] = np.array(mkind)
        out[p + "in_manning"] = np.asarray(manning if manning is not None else np.nan, np.float64 if mkind != "cell"
                                           else np.float32)
        out[p + "in_active"] = active if active is not None else np.zeros(0, np.float32)
        out.update(topo_arrays(p + "out/", st))
        names.append(name)
    out["cases"] = np.array(names)

    # invalid inputs and the reference's error text
    pts, tri = delaunay(30, 10.0)
    bed = np.zeros(len(tri), np.float32)
    degenerate_pts = np.vstack([pts, [[20.0, 20.0], [21.0, 21.0], [22.0, 22.0]]])
    k = len(pts)
    nonmanifold_pts = np.vstack([pts, [[50.0, 0.0], [51.0, 0.0], [50.5, 1.0], [50.5, -1.0], [50.5, 2.0]]])
    bad = {
        "nodes_shape": (pts[:, :1], tri, bed, None, None, "closed"),
        "triangles_shape": (pts, tri[:, :2], bed, None, None, "closed"),
        "bed_length": (pts, tri, bed[:-1], None, None, "closed"),
        "node_index_range": (pts, np.vstack([tri, [[0, 1, k + 5]]]), np.zeros(len(tri) + 1, np.float32), None, None,
                             "closed"),
        "degenerate": (degenerate_pts, np.vstack([tri, [[k, k + 1, k + 2]]]), np.zeros(len(tri) + 1, np.float32),
                       None, None, "closed"),
        "nonmanifold": (nonmanifold_pts, np.vstack([tri, [[k, k + 1, k + 2], [k, k + 1, k + 3], [k, k + 1, k + 4]]]),
                        np.zeros(len(tri) + 3, np.float32), None, None, "closed"),
        "manning_length": (pts, tri, bed, np.full(len(tri) - 1, 0.03, np.float32), None, "closed"),
        "active_length": (pts, tri, bed, None, np.ones(len(tri) + 2, np.float32), "closed"),
        "unsupported_mode": (pts, tri, bed, None, None, "sticky"),
    }
    err_names = []
    for name, args in bad.items():
        try:
            tb.build_triangular_surface_topology(*args)
        except ValueError as e:
            msg = str(e)
        else:
            raise AssertionError(f"reference accepted invalid input {name}")
        p = f"err/{name}/"
        nodes, tris, b, man, act, mode = args
        out[p + "nodes"], out[p + "triangles"], out[p + "bed"] = nodes, tris, b
        out[p + "manning"] = man if man is not None else np.zeros(0, np.float32)
        out[p + "active"] = act if act is not None else np.zeros(0, np.float32)
        out[p + "mode"] = np.array(mode)
        out[p + "message"] = np.array(msg)
        err_names.append(name)
    out["errors"] = np.array(err_names)
    np.savez_compressed(OUT / "topology_cases.npz", **out)
    return names + err_names


def import_reference_outputs():
    """The reference's output writer (postprocessing/outputs.py), its engine's
    SimulationResult (solver/engine.py:68-105) and RunConfig (config.py), and
    its parity validator (hybrid_flood/operational/parity_validation.py).
    Their package ``__init__``s are bypassed like the kernels'; PyYAML (read by
    config.load_config only) and pandas (CSV loaders only) get empty
    stand-ins."""

    src = sys.modules["gurugram_flood"].__path__[0]
    hf = str(Path(src).parent / "hybrid_flood")
    for name, path in (("gurugram_flood.postprocessing", str(Path(src) / "postprocessing")),
                       ("hybrid_flood", hf), ("hybrid_flood.operational", str(Path(hf) / "operational"))):
        mod = types.ModuleType(name)
        mod.__path__ = [path]
        sys.modules[name] = mod
    sys.modules.setdefault("pandas", types.ModuleType("pandas"))
    sys.modules.setdefault("yaml", types.ModuleType("yaml"))
    import gurugram_flood.config as rcfg
    import gurugram_flood.postprocessing.outputs as routs
    import gurugram_flood.solver.engine as reng
    import hybrid_flood.operational.parity_validation as rpv

    return rcfg, reng, routs, rpv


def output_result_arrays(tb, stab, pis, rng):
    """A short coupled reference run (the restated engine loop) as the arrays
    of a SimulationResult; the candidate is the same run with seeded depth
    perturbations (some cells cross the 0.05 m threshold)."""

    import json as _json

    sc = tiny_coupled(seed=13)
    st = sc.city.topologies.surface_topology
    h0 = np.where(np.asarray(st.active_mask) > 0.5, rng.uniform(0.0, 0.12, st.cell_count), 0).astype(np.float32)
    sc.city.topologies.surface_state = tb.TriangularSurfaceState(h0, np.zeros_like(h0), np.zeros_like(h0))
    sc.overrides["solver.duration_min"] = 2.0
    res = reference_run(tb, stab, pis, sc, max_steps=10_000, snapshot_interval_s=30.0)
    mesh = sc.city.mesh
    topo = sc.city.topologies
    cp, pp = topo.coupling_topology, topo.pipe_topology
    n_nodes = cp.node_count

    def result_of(snap_h, snap_hu, snap_hv):
        speed = np.zeros_like(snap_h)
        wet = snap_h > 1.0e-4
        speed[wet] = np.sqrt(snap_hu[wet] ** 2 + snap_hv[wet] ** 2) / snap_h[wet]
        area = np.asarray(st.cell_area_m2, np.float64)
        return {
            "snapshot_times_min": np.asarray(res["snap_t"] / 60.0, np.float32),
            "depth_snapshots_m": snap_h, "speed_snapshots_mps": speed,
            "node_volume_snapshots_m3": np.asarray(res["snap_v"], np.float32),
            "final_depth_m": snap_h[-1], "final_hu_m2ps": snap_hu[-1], "final_hv_m2ps": snap_hv[-1],
            "final_node_volume_m3": np.asarray(res["final_V"], np.float32),
            "final_link_flow_m3ps": np.asarray(res["final_Q"], np.float32),
            "max_depth_m": np.max(snap_h, axis=0).astype(np.float32),
            "max_speed_mps": np.max(speed, axis=0).astype(np.float32),
            "mass_balance": mass_balance(snap_h[-1], area),
        }

    def mass_balance(final_h, area):
        # the keys and formula of the reference engine's mass balance (engine.py:203-214, 364-382)
        led = [float(x) for x in res["ledger"]]
        cum = dict(zip(("rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
                        "overflow_surcharge_m3", "unreturned_overflow_m3"), led[:6]))
        cum.update(external_boundary_inflow_m3=0.0, surface_recharge_capture_m3=0.0, surface_recharge_loss_m3=0.0)
        vs0 = float(np.sum(h0.astype(np.float64) * area))
        vn0 = float(np.sum(np.asarray(topo.pipe_state.node_volume_m3, np.float64)))
        vs = float(np.sum(final_h.astype(np.float64) * area))
        vn = float(np.asarray(res["final_V"], np.float32).sum())
        lhs = vs0 + vn0 + cum["rainfall_input_m3"]
        rhs = (vs + vn + cum["infiltration_loss_m3"] + cum["outfall_discharge_m3"] + cum["unreturned_overflow_m3"]
               - cum["boundary_net_flux_m3"])
        return {**cum, "initial_surface_volume_m3": vs0, "initial_node_volume_m3": vn0,
                "final_surface_volume_m3": vs, "final_node_volume_m3": vn, "mass_residual_m3": lhs - rhs,
                "mass_residual_ratio": (lhs - rhs) / max(abs(lhs), 1.0)}

    ref = result_of(res["snap_h"], res["snap_hu"], res["snap_hv"])
    pert = rng.normal(0.0, 2.0e-3, res["snap_h"].shape).astype(np.float32)
    cand_h = np.maximum(res["snap_h"] + pert * (res["snap_h"] > 0), 0).astype(np.float32)
    cand = result_of(cand_h, res["snap_hu"], res["snap_hv"])
    static = {
        "mesh/nodes_xy": np.asarray(mesh.nodes_xy, np.float64), "mesh/triangles": np.asarray(mesh.triangles, np.int64),
        "mesh/centroids_xy": np.asarray(mesh.centroids_xy, np.float64),
        "mesh/terrain_elevation_m": np.asarray(mesh.terrain_elevation_m, np.float64),
        "mesh/active_mask": np.asarray(mesh.active_mask, bool),
        "mesh/building_mask": (rng.random(st.cell_count) < 0.05),
        "mesh/road_mask": (rng.random(st.cell_count) < 0.2),
        "cp/node_x_m": rng.uniform(0, 100, n_nodes), "cp/node_y_m": rng.uniform(0, 100, n_nodes),
        "cp/node_count": np.int64(n_nodes), "cp/inlet_count": np.int64(cp.inlet_count),
        "pp/link_from_node_index": np.asarray(pp.link_from_node_index, np.int64),
        "pp/link_to_node_index": np.asarray(pp.link_to_node_index, np.int64), "pp/link_count": np.int64(pp.link_count),
        "cell_area_m2": np.asarray(st.cell_area_m2, np.float64),
    }
    meta = {"step_count": int(res["step_count"]), "runtime_s": 1.25, "cfl_eval_count": 3, "cfl_reused_count": 90,
            "backend_name": "numpy", "is_gpu": False, "duration_min": 2.0, "topology_mode": "exact_production",
            "source_csv": "synthetic_storm.csv", "total_depth_mm": 42.5}
    return ref, cand, static, _json.dumps(meta)


def make_output_cases(tb, stab, pis):
    """The reference writer's NPZ (save_run_npz, outputs.py:25-58) and report
    (build_report, :61-99) for a short coupled run; and the reference's
    validate_v1_parity_run (parity_validation.py:43-253) applied to that run
    as the reference directory and, as the candidate directory, a
    perturbed copy written by this library's floodgb.outputs."""

    import json as _json
    import tempfile
    from types import SimpleNamespace

    from floodgb import outputs as fout
    from floodgb.config import load_config

    rcfg, reng, routs, rpv = import_reference_outputs()
    rng = np.random.default_rng(20261205)
    ref, cand, static, meta_json = output_result_arrays(tb, stab, pis, rng)
    meta = _json.loads(meta_json)

    def city_of():
        mesh = SimpleNamespace(**{k.split("/", 1)[1]: v for k, v in static.items() if k.startswith("mesh/")})
        cp = SimpleNamespace(node_x_m=static["cp/node_x_m"], node_y_m=static["cp/node_y_m"],
                             node_count=int(static["cp/node_count"]), inlet_count=int(static["cp/inlet_count"]))
        pp = SimpleNamespace(link_from_node_index=static["pp/link_from_node_index"],
                             link_to_node_index=static["pp/link_to_node_index"], link_count=int(static["pp/link_count"]))
        return SimpleNamespace(mesh=mesh, topologies=SimpleNamespace(coupling_topology=cp, pipe_topology=pp),
                               topology_mode=meta["topology_mode"])

    rain = SimpleNamespace(source_csv=meta["source_csv"], total_depth_mm=meta["total_depth_mm"])
    keys = ("step_count", "runtime_s", "cfl_eval_count", "cfl_reused_count", "backend_name", "is_gpu", "duration_min")
    cfg = rcfg.RunConfig()
    cfg.solver.duration_min = 2.0
    rres = reng.SimulationResult(**ref, **{k: meta[k] for k in keys}, city=city_of(), rainfall=rain, config=cfg)
    out = {"meta": np.array(meta_json)}
    out.update({f"ref/{k}": v for k, v in ref.items() if k != "mass_balance"})
    out.update({f"cand/{k}": v for k, v in cand.items() if k != "mass_balance"})
    out["ref/mass_balance"] = np.array(_json.dumps(ref["mass_balance"]))
    out["cand/mass_balance"] = np.array(_json.dumps(cand["mass_balance"]))
    out.update({f"static/{k}": v for k, v in static.items()})
    with tempfile.TemporaryDirectory() as tmp:
        rdir, cdir = Path(tmp) / "reference", Path(tmp) / "candidate"
        rdir.mkdir()
        cdir.mkdir()
        path = routs.save_run_npz(rres, rdir)
        with np.load(path, allow_pickle=False) as z:
            out["npz_names"] = np.array(sorted(z.files))
            for name in z.files:
                out[f"npz/{name}"] = z[name]
        report = routs.build_report(rres, {"npz": str(path)})
        out["report_json"] = np.array(_json.dumps(report, sort_keys=True))
        routs.save_report(report, rdir)
        # candidate: this library's writer (the reference validator reads it)
        topo_npz = Path(tmp) / "topology.npz"
        np.savez(topo_npz, surface_cell_area_m2=static["cell_area_m2"])
        fcfg = load_config(None, {"solver.duration_min": 2.0})
        cres = SimpleNamespace(**cand, **{k: meta[k] for k in keys}, city=city_of(), rainfall=rain, config=fcfg)
        fout.save_run_npz(cres, cdir)
        fout.write_report(cres, cdir, {"npz": "flood_simulation_outputs.npz"}, topology_path=topo_npz)
        payload = rpv.validate_v1_parity_run(reference_dir=rdir, candidate_dir=cdir)
        for k in ("reference_dir", "candidate_dir"):
            payload.pop(k, None)
        out["validation_json"] = np.array(_json.dumps(payload, sort_keys=True))
    np.savez_compressed(OUT / "output_cases.npz", **out)
    return sorted(payload["summary"])


def reference_root() -> Path:
    """The reference checkout: the first argument, else $FLOODGB_REFERENCE."""

    import os

    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("FLOODGB_REFERENCE")
    if not root:
        raise SystemExit("usage: make_golden.py <reference checkout> [--only name,...] "
                         "(or set FLOODGB_REFERENCE)")
    return Path(root)


def main():
    ref = reference_root()
    only = None
    for a in sys.argv[1:]:
        if a.startswith("--only="):
            only = set(a.split("=", 1)[1].split(","))
    want = lambda name: only is None or name in only  # noqa: E731
    tb, stab, pis = import_reference(ref)
    if want("surface"):
        print("surface:", make_surface_cases(tb, stab))
    if want("pipe"):
        print("pipe:", make_pipe_cases(tb))
    if want("run"):
        make_run_cases(tb, stab, pis)
    if want("forcing"):
        pes, j5 = import_reference_forcing()
        make_forcing_cases(tb, stab, pis, pes, j5)
    if want("li"):
        print("local inertial:", make_li_cases(tb, stab, pis))
    if want("topology"):
        print("topology:", make_topology_cases(tb))
    if want("outputs"):
        print("outputs:", make_output_cases(tb, stab, pis))
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
