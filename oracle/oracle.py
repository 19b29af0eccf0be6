"""ctypes wrapper of the C oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` (as a checker) and ``bench.py``'s
CPU-baseline leg use this module.  The product path (``floodgb`` +
``libfloodgb.so``) never imports it.

``liborc.so`` is built from ``flood_oracle.c`` with ``build()``; the C file
restates the reference's hot-path algorithm (see ``flood_oracle.h`` for the
reference file:line each part follows).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liborc.so"
_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "flood_oracle.c"
    hdr = HERE / "flood_oracle.h"
    if LIB_PATH.exists() and not force:
        if LIB_PATH.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
            return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    tmp.replace(LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
        _lib.orc_stable_dt.restype = C.c_double
        _lib.orc_li_stable_dt.restype = C.c_double
        _lib.orc_num_threads.restype = C.c_int
        _lib.orc_external_inflow.restype = C.c_double
        _lib.orc_inflow_q.restype = C.c_float
    return _lib


f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)


class OrcMesh(C.Structure):
    _fields_ = [
        ("cell_count", C.c_int32), ("edge_count", C.c_int32),
        ("bed", f32p), ("manning", f32p), ("area", f32p), ("char_len", f32p), ("active", f32p),
        ("left", i32p), ("right", i32p), ("bcode", i32p),
        ("nx", f32p), ("ny", f32p), ("len", f32p),
        ("cell_edges", i32p),
        ("has_stage", C.c_int32), ("stage", C.c_float),
    ]


class OrcDrain(C.Structure):
    _fields_ = [
        ("node_count", C.c_int32), ("link_count", C.c_int32), ("inlet_count", C.c_int32),
        ("inlet_cell", i32p), ("inlet_node", i32p), ("node_cell", i32p),
        ("node_invert", f32p), ("node_area", f32p), ("node_maxdepth", f32p),
        ("cap_capacity", f32p), ("sur_capacity", f32p),
        ("link_from", i32p), ("link_to", i32p),
        ("link_len", f32p), ("link_area", f32p), ("link_radius", f32p), ("link_n", f32p),
        ("link_capacity", f32p), ("link_invert", f32p), ("link_diam", f32p), ("link_minor", f32p),
        ("link_geom", i32p), ("link_rect_w", f32p), ("link_rect_h", f32p),
        ("out_area", f32p), ("out_coef", f32p), ("out_tail", f32p), ("out_capacity", f32p),
        ("wave_speed", C.c_float),
        ("capture_rule", C.c_int32),
        ("orifice_area", C.c_float), ("orifice_coef", C.c_float),
        ("weir_perimeter", C.c_float), ("weir_coef", C.c_float),
        ("sur_count", C.c_int32), ("sur_cell", i32p), ("sur_node", i32p), ("sur_weight", f32p),
        ("sur_normalized", C.c_int32),
    ]


class OrcForcing(C.Structure):
    _fields_ = [
        ("rain_kind", C.c_int32), ("rain_scalar", C.c_float), ("rain_cell", f32p),
        ("infil_kind", C.c_int32), ("infil_scalar", C.c_float), ("infil_cell", f32p),
    ]


class OrcInflow(C.Structure):
    _fields_ = [
        ("receiver_count", C.c_int32), ("time_count", C.c_int32),
        ("receiver_cell", i32p), ("times_s", f64p), ("q_m3ps", f32p),
    ]


class OrcRecharge(C.Structure):
    _fields_ = [
        ("row_count", C.c_int32), ("source_cell", i32p),
        ("storage_capacity", f32p), ("capture_capacity", f32p), ("recharge_capacity", f32p), ("stop_depth", f32p),
    ]


class OrcRunParams(C.Structure):
    _fields_ = [
        ("cfl", C.c_double), ("safety", C.c_double), ("max_dt", C.c_double), ("max_speed", C.c_double),
        ("duration_s", C.c_double), ("snapshot_interval_s", C.c_double),
        ("cfl_interval", C.c_int32), ("finite_interval", C.c_int32),
        ("g", C.c_double), ("min_depth", C.c_float),
        ("horton", C.c_int32),
        ("rain_mult", f32p), ("f0", f32p), ("fc", f32p), ("k", f32p),
        ("infil_kind", C.c_int32), ("infil_scalar", C.c_float), ("infil_cell", f32p),
        ("hyeto_n", C.c_int32),
        ("hyeto_start_s", f64p), ("hyeto_end_s", f64p), ("hyeto_rate", f64p),
        ("has_drainage", C.c_int32),
        ("max_steps", C.c_int64),
        ("max_snapshots", C.c_int32),
        ("inflow", C.POINTER(OrcInflow)), ("recharge", C.POINTER(OrcRecharge)), ("recharge_storage", f32p),
        ("local_inertial", C.c_int32),
        ("t_start_s", C.c_double), ("step_start", C.c_int64), ("cached_dt_s", C.c_double),
        ("next_snapshot_s", C.c_double),
    ]


class OrcRunResult(C.Structure):
    _fields_ = [
        ("step_count", C.c_int64), ("cfl_evals", C.c_int64), ("cfl_reused", C.c_int64),
        ("snapshot_count", C.c_int32), ("error", C.c_int32),
        ("error_step", C.c_int64), ("t_end", C.c_double),
        ("ledger", C.c_double * 12),
        ("cached_dt_s", C.c_double), ("next_snapshot_s", C.c_double),
    ]


CAPTURE_RULES = {"capacity": 0, "head_limited_capacity": 1, "orifice": 2, "weir_orifice": 3}


def _p(arr, ctype):
    if arr is None:
        return C.cast(None, C.POINTER(ctype))
    return arr.ctypes.data_as(C.POINTER(ctype))


class _Keep:
    """Holds the contiguous arrays a ctypes struct points into."""

    def __init__(self):
        self.items = []

    def f32(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a), dtype=np.float32)
        self.items.append(a)
        return a

    def i32(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a), dtype=np.int32)
        self.items.append(a)
        return a

    def f64(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a), dtype=np.float64)
        self.items.append(a)
        return a


def make_mesh(topo, stage: float | None = None):
    from floodgb.topology import cell_edge_indices

    k = _Keep()
    cei = topo.cell_edge_indices if topo.cell_edge_indices is not None else cell_edge_indices(topo)
    m = OrcMesh(
        cell_count=topo.cell_count, edge_count=topo.edge_count,
        bed=_p(k.f32(topo.bed_elevation_m), C.c_float), manning=_p(k.f32(topo.manning_n), C.c_float),
        area=_p(k.f32(topo.cell_area_m2), C.c_float), char_len=_p(k.f32(topo.characteristic_length_m), C.c_float),
        active=_p(k.f32(topo.active_mask), C.c_float),
        left=_p(k.i32(topo.edge_left_cell), C.c_int32), right=_p(k.i32(topo.edge_right_cell), C.c_int32),
        bcode=_p(k.i32(topo.boundary_code), C.c_int32),
        nx=_p(k.f32(topo.edge_normal_x), C.c_float), ny=_p(k.f32(topo.edge_normal_y), C.c_float),
        len=_p(k.f32(topo.edge_length_m), C.c_float),
        cell_edges=_p(k.i32(cei), C.c_int32),
        has_stage=1 if topo.has_stage_boundary else 0,
        stage=float(stage) if stage is not None else 0.0,
    )
    return m, k


def make_drain(coupling, pipe, capture_rule="orifice", orifice_area=0.04, orifice_coef=0.62,
               weir_perimeter=0.0, weir_coef=0.45):
    k = _Keep()
    rect = pipe.link_geometry_code is not None and pipe.link_rect_width_m is not None and pipe.link_rect_height_m is not None
    d = OrcDrain(
        node_count=coupling.node_count, link_count=pipe.link_count, inlet_count=coupling.inlet_count,
        inlet_cell=_p(k.i32(coupling.inlet_cell_index), C.c_int32),
        inlet_node=_p(k.i32(coupling.inlet_node_index), C.c_int32),
        node_cell=_p(k.i32(coupling.node_surface_cell_index), C.c_int32),
        node_invert=_p(k.f32(coupling.node_invert_elevation_m), C.c_float),
        node_area=_p(k.f32(coupling.node_storage_area_m2), C.c_float),
        node_maxdepth=_p(k.f32(coupling.node_max_depth_m), C.c_float),
        cap_capacity=_p(k.f32(coupling.inlet_capture_capacity_m3ps), C.c_float),
        sur_capacity=_p(k.f32(coupling.inlet_surcharge_capacity_m3ps), C.c_float),
        link_from=_p(k.i32(pipe.link_from_node_index), C.c_int32),
        link_to=_p(k.i32(pipe.link_to_node_index), C.c_int32),
        link_len=_p(k.f32(pipe.link_length_m), C.c_float), link_area=_p(k.f32(pipe.link_area_m2), C.c_float),
        link_radius=_p(k.f32(pipe.link_hydraulic_radius_m), C.c_float), link_n=_p(k.f32(pipe.link_manning_n), C.c_float),
        link_capacity=_p(k.f32(pipe.link_flow_capacity_m3ps), C.c_float),
        link_invert=_p(k.f32(pipe.link_invert_elevation_m), C.c_float),
        link_diam=_p(k.f32(pipe.link_diameter_m), C.c_float),
        link_minor=_p(k.f32(pipe.link_minor_loss_coefficient), C.c_float),
        link_geom=_p(k.i32(pipe.link_geometry_code) if rect else None, C.c_int32),
        link_rect_w=_p(k.f32(pipe.link_rect_width_m) if rect else None, C.c_float),
        link_rect_h=_p(k.f32(pipe.link_rect_height_m) if rect else None, C.c_float),
        out_area=_p(k.f32(pipe.outfall_area_m2), C.c_float), out_coef=_p(k.f32(pipe.outfall_coefficient), C.c_float),
        out_tail=_p(k.f32(pipe.outfall_tailwater_head_m), C.c_float),
        out_capacity=_p(k.f32(pipe.outfall_flow_capacity_m3ps), C.c_float),
        wave_speed=float(pipe.pressurized_wave_speed_mps),
        capture_rule=CAPTURE_RULES[capture_rule],
        orifice_area=orifice_area, orifice_coef=orifice_coef, weir_perimeter=weir_perimeter, weir_coef=weir_coef,
    )
    # the weighted return table is used when all three arrays are given (reference :1424-1428)
    sc, sn, sw = (getattr(coupling, a, None) for a in ("surcharge_cell_index", "surcharge_node_index",
                                                        "surcharge_return_weight"))
    if sc is not None and sn is not None and sw is not None:
        d.sur_count = int(np.asarray(sc).size)
        d.sur_cell = _p(k.i32(sc), C.c_int32)
        d.sur_node = _p(k.i32(sn), C.c_int32)
        d.sur_weight = _p(k.f32(sw), C.c_float)
        d.sur_normalized = int(bool(getattr(coupling, "surcharge_return_weight_is_normalized", False)))
    return d, k


def _forcing(value, keep):
    if np.ndim(value) == 0:
        return 0, float(np.float32(value)), None
    arr = keep.f32(value)
    return 1, 0.0, arr


def surface_step(topo, h, hu, hv, dt, rainfall=0.0, infiltration=0.0, stage=None, g=9.80665, min_depth=1e-5):
    """One surface step (fluxes + cell update + sources); returns (h, hu, hv, diag[6])."""

    m, keep = make_mesh(topo, stage)
    rk, rs, ra = _forcing(rainfall, keep)
    ik, is_, ia = _forcing(infiltration, keep)
    f = OrcForcing(rain_kind=rk, rain_scalar=rs, rain_cell=_p(ra, C.c_float),
                   infil_kind=ik, infil_scalar=is_, infil_cell=_p(ia, C.c_float))
    h = keep.f32(h)
    hu = keep.f32(hu)
    hv = keep.f32(hv)
    n = topo.cell_count
    ho, huo, hvo = np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n, np.float32)
    diag = np.zeros(6, np.float64)
    rc = lib().orc_surface_step(C.byref(m), _p(h, C.c_float), _p(hu, C.c_float), _p(hv, C.c_float), C.byref(f),
                                C.c_double(dt), C.c_double(g), C.c_float(min_depth),
                                _p(ho, C.c_float), _p(huo, C.c_float), _p(hvo, C.c_float), _p(diag, C.c_double))
    if rc != 0:
        raise RuntimeError(f"orc_surface_step failed: {rc}")
    return ho, huo, hvo, diag


def li_step(topo, h, hu, hv, dt, rainfall=0.0, infiltration=0.0, g=9.80665, min_depth=1e-5):
    """One local-inertial surface step (discharge, donor scale, gather + sources)."""

    m, keep = make_mesh(topo, None)
    rk, rs, ra = _forcing(rainfall, keep)
    ik, is_, ia = _forcing(infiltration, keep)
    f = OrcForcing(rain_kind=rk, rain_scalar=rs, rain_cell=_p(ra, C.c_float),
                   infil_kind=ik, infil_scalar=is_, infil_cell=_p(ia, C.c_float))
    h, hu, hv = keep.f32(h), keep.f32(hu), keep.f32(hv)
    n = topo.cell_count
    ho, huo, hvo = np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n, np.float32)
    diag = np.zeros(6, np.float64)
    rc = lib().orc_li_step(C.byref(m), _p(h, C.c_float), _p(hu, C.c_float), _p(hv, C.c_float), C.byref(f),
                           C.c_double(dt), C.c_double(g), C.c_float(min_depth),
                           _p(ho, C.c_float), _p(huo, C.c_float), _p(hvo, C.c_float), _p(diag, C.c_double))
    if rc != 0:
        raise RuntimeError(f"orc_li_step failed: {rc}")
    return ho, huo, hvo, diag


def li_stable_dt(char_len, h, cfl=0.85, g=9.80665, min_depth=1e-5):
    cl = np.ascontiguousarray(char_len, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    v = lib().orc_li_stable_dt(C.c_int32(h.size), _p(cl, C.c_float), _p(h, C.c_float), C.c_float(cfl),
                               C.c_float(g), C.c_float(min_depth))
    if v < 0:
        raise ValueError("No finite cells are available for timestep calculation.")
    return float(v)


def clamp_velocity(h, hu, hv, max_speed=5.0):
    h = np.ascontiguousarray(h, np.float32)
    hu = np.array(hu, np.float32)
    hv = np.array(hv, np.float32)
    lib().orc_clamp_velocity(C.c_int32(h.size), _p(h, C.c_float), _p(hu, C.c_float), _p(hv, C.c_float), C.c_float(max_speed))
    return hu, hv


def stable_dt(char_len, h, hu, hv, cfl=0.85, g=9.80665, min_depth=1e-5):
    cl = np.ascontiguousarray(char_len, np.float32)
    h = np.ascontiguousarray(h, np.float32)
    hu = np.ascontiguousarray(hu, np.float32)
    hv = np.ascontiguousarray(hv, np.float32)
    v = lib().orc_stable_dt(C.c_int32(h.size), _p(cl, C.c_float), _p(h, C.c_float), _p(hu, C.c_float),
                            _p(hv, C.c_float), C.c_float(cfl), C.c_float(g), C.c_float(min_depth))
    if v < 0:
        raise ValueError("No finite cells are available for timestep calculation.")
    return float(v)


def pipe_step(topo, coupling, pipe, h, node_volume, link_flow, dt, g=9.80665, **inlet_kw):
    """Drainage step (inlets, links, outfalls, overflow); returns (h, V, Q, diag[7])."""

    m, k1 = make_mesh(topo)
    d, k2 = make_drain(coupling, pipe, **inlet_kw)
    h = np.array(h, np.float32)
    V = np.array(node_volume, np.float64)
    Q = np.array(link_flow, np.float64)
    diag = np.zeros(7, np.float64)
    rc = lib().orc_pipe_step(C.byref(m), C.byref(d), _p(h, C.c_float), _p(V, C.c_double), _p(Q, C.c_double),
                             C.c_double(dt), C.c_float(g), _p(diag, C.c_double))
    if rc != 0:
        raise RuntimeError(f"orc_pipe_step failed: {rc}")
    return h, V, Q, diag


def make_inflow(external, keep):
    """OrcInflow of an ExternalBoundaryInflowSurface-like object (receiver_cell_index,
    times_s, q_m3ps_by_receiver [times x receivers])."""

    cells = keep.i32(external.receiver_cell_index)
    times = keep.f64(external.times_s)
    q = keep.f32(np.asarray(external.q_m3ps_by_receiver, np.float32).reshape(times.size, cells.size))
    return OrcInflow(receiver_count=cells.size, time_count=times.size, receiver_cell=_p(cells, C.c_int32),
                     times_s=_p(times, C.c_double), q_m3ps=_p(q, C.c_float))


def make_recharge(topo, keep):
    """OrcRecharge of a June5RechargeTopology-like object (float32 rows)."""

    cells = keep.i32(topo.source_cell_index)
    return OrcRecharge(row_count=cells.size, source_cell=_p(cells, C.c_int32),
                       storage_capacity=_p(keep.f32(topo.storage_capacity_m3), C.c_float),
                       capture_capacity=_p(keep.f32(topo.capture_capacity_m3ps), C.c_float),
                       recharge_capacity=_p(keep.f32(topo.recharge_capacity_m3ps), C.c_float),
                       stop_depth=_p(keep.f32(topo.stop_depth_m), C.c_float))


def external_inflow(area, external, h, time_s: float, dt: float):
    """apply_external_boundary_inflow_depth on a copy of h: (new h, added m^3)."""

    keep = _Keep()
    x = make_inflow(external, keep)
    a = keep.f32(area)
    out = np.array(h, np.float32)
    added = lib().orc_external_inflow(a.size, _p(a, C.c_float), C.byref(x), C.c_double(time_s), C.c_double(dt),
                                      _p(out, C.c_float))
    return out, float(added)


def inflow_q(external, time_s: float) -> np.ndarray:
    keep = _Keep()
    x = make_inflow(external, keep)
    return np.array([lib().orc_inflow_q(C.byref(x), j, C.c_double(time_s)) for j in range(x.receiver_count)],
                    np.float32)


def recharge(area, topo, h, storage, dt: float):
    """apply_june5_surface_recharge on copies: (new h, new storage, capture m^3, loss m^3)."""

    keep = _Keep()
    r = make_recharge(topo, keep)
    a = keep.f32(area)
    out = np.array(h, np.float32)
    st = np.array(storage, np.float32)
    diag = np.zeros(2, np.float64)
    lib().orc_recharge(C.byref(r), _p(a, C.c_float), C.c_double(dt), _p(out, C.c_float), _p(st, C.c_float),
                       _p(diag, C.c_double))
    return out, st, float(diag[0]), float(diag[1])


@dataclass
class OracleRun:
    step_count: int
    cfl_evals: int
    cfl_reused: int
    t_end: float
    snapshot_times_s: np.ndarray
    depth: np.ndarray
    hu: np.ndarray
    hv: np.ndarray
    node_volume: np.ndarray
    final_h: np.ndarray
    final_hu: np.ndarray
    final_hv: np.ndarray
    final_node_volume: np.ndarray
    final_link_flow: np.ndarray
    wet_time: np.ndarray
    ledger: dict
    error: int
    error_step: int
    recharge_storage: np.ndarray | None = None
    # where the run stopped, for run(..., start=this): absolute step count,
    # the cached CFL dt and the next snapshot time
    step_end: int = 0
    cached_dt_s: float = -1.0
    next_snapshot_s: float = 0.0


def run(scenario, cfg=None, max_steps: int = 0, max_snapshots: int | None = None,
        start: OracleRun | None = None) -> OracleRun:
    """Restated engine loop (engine.py:219-344) on the oracle step functions.

    With ``start`` (the result of an earlier run of the same scenario and
    config, stopped by ``max_steps``) the loop continues from that run's final
    state, simulated time, step count, cached CFL dt and snapshot schedule;
    ``step_count``, snapshots and ledger then cover the resumed part only."""

    from floodgb.config import load_config
    from floodgb.rainfall import hyetograph_arrays

    cfg = cfg or load_config(None, scenario.overrides)
    city = scenario.city
    topo = city.topologies
    st = topo.surface_topology
    s, ph = cfg.solver, cfg.physics
    duration = s.duration_min if s.duration_min is not None else scenario.rainfall.duration_min
    m, k1 = make_mesh(st)
    has_drain = topo.coupling_topology.node_count > 0
    d, k2 = make_drain(topo.coupling_topology, topo.pipe_topology, ph.inlet_capture_rule, ph.inlet_orifice_area_m2,
                       ph.inlet_orifice_coefficient, ph.inlet_weir_perimeter_m, ph.inlet_weir_coefficient)
    keep = _Keep()
    hs, he, hr = hyetograph_arrays(scenario.rainfall)
    hs, he, hr = keep.f64(hs), keep.f64(he), keep.f64(hr)
    horton = ph.infiltration_mode == "production_horton" and city.infiltration_fields is not None
    fields = city.infiltration_fields
    infil_cell = None
    if not horton and city.simple_infiltration_mps is not None:
        infil_cell = keep.f32(city.simple_infiltration_mps)
    n_snap = max_snapshots or int(np.ceil(duration / s.snapshot_interval_min)) + 2
    p = OrcRunParams(
        cfl=s.cfl, safety=s.cfl_reuse_safety_factor, max_dt=s.max_dt_s, max_speed=s.max_speed_mps,
        duration_s=duration * 60.0, snapshot_interval_s=s.snapshot_interval_min * 60.0,
        cfl_interval=s.cfl_update_interval_steps, finite_interval=s.finite_check_interval_steps,
        g=9.80665, min_depth=1e-5, horton=1 if horton else 0,
        rain_mult=_p(keep.f32(fields.rainfall_multiplier) if horton else None, C.c_float),
        f0=_p(keep.f32(fields.horton_f0_mps) if horton else None, C.c_float),
        fc=_p(keep.f32(fields.horton_fc_mps) if horton else None, C.c_float),
        k=_p(keep.f32(fields.horton_k_per_s) if horton else None, C.c_float),
        infil_kind=1 if infil_cell is not None else 0, infil_scalar=0.0, infil_cell=_p(infil_cell, C.c_float),
        hyeto_n=hs.size, hyeto_start_s=_p(hs, C.c_double), hyeto_end_s=_p(he, C.c_double), hyeto_rate=_p(hr, C.c_double),
        has_drainage=1 if has_drain else 0, max_steps=int(max_steps), max_snapshots=n_snap,
        local_inertial=1 if s.surface_step_mode == "local_inertial" else 0,
    )
    if start is not None:
        p.t_start_s = start.t_end
        p.step_start = start.step_end
        p.cached_dt_s = start.cached_dt_s
        p.next_snapshot_s = start.next_snapshot_s
    ext = getattr(city, "external_boundary", None)
    rch = getattr(city, "recharge_topology", None)
    rstore = None
    if ext is not None and np.asarray(ext.receiver_cell_index).size:
        xin = make_inflow(ext, keep)
        keep.items.append(xin)
        p.inflow = C.pointer(xin)
    if rch is not None and np.asarray(rch.source_cell_index).size:
        xr = make_recharge(rch, keep)
        keep.items.append(xr)
        p.recharge = C.pointer(xr)
        rstore = np.zeros(xr.row_count, np.float32)
        p.recharge_storage = _p(rstore, C.c_float)
    n = st.cell_count
    nn = topo.coupling_topology.node_count
    if start is None:
        h = np.array(topo.surface_state.h_m, np.float32)
        hu = np.array(topo.surface_state.hu_m2ps, np.float32)
        hv = np.array(topo.surface_state.hv_m2ps, np.float32)
        V = np.array(topo.pipe_state.node_volume_m3, np.float64)
        Q = np.array(topo.pipe_state.link_flow_m3ps, np.float64)
        wt = np.zeros(n, np.float32)
    else:
        h, hu, hv = (np.array(a, np.float32) for a in (start.final_h, start.final_hu, start.final_hv))
        V = np.array(start.final_node_volume, np.float64)
        Q = np.array(start.final_link_flow, np.float64)
        wt = np.array(start.wet_time, np.float32)
        if rstore is not None and start.recharge_storage is not None:
            rstore[:] = start.recharge_storage
    st_t = np.zeros(n_snap, np.float64)
    sh = np.zeros((n_snap, n), np.float32)
    shu = np.zeros((n_snap, n), np.float32)
    shv = np.zeros((n_snap, n), np.float32)
    sv = np.zeros((n_snap, max(nn, 1)), np.float32)
    res = OrcRunResult()
    rc = lib().orc_run(C.byref(m), C.byref(d), C.byref(p), _p(h, C.c_float), _p(hu, C.c_float), _p(hv, C.c_float),
                       _p(V, C.c_double), _p(Q, C.c_double), _p(wt, C.c_float), _p(st_t, C.c_double),
                       _p(sh, C.c_float), _p(shu, C.c_float), _p(shv, C.c_float), _p(sv, C.c_float), C.byref(res))
    if rc not in (0, 1):
        raise RuntimeError(f"orc_run failed: {rc}")
    k = res.snapshot_count
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3", "unreturned_overflow_m3", "surface_capture_m3", "surface_surcharge_m3",
             "link_abs_flow_m3", "external_boundary_inflow_m3", "surface_recharge_capture_m3",
             "surface_recharge_loss_m3"]
    return OracleRun(
        step_count=res.step_count, cfl_evals=res.cfl_evals, cfl_reused=res.cfl_reused, t_end=res.t_end,
        snapshot_times_s=st_t[:k].copy(), depth=sh[:k].copy(), hu=shu[:k].copy(), hv=shv[:k].copy(),
        node_volume=sv[:k, :nn].copy(), final_h=h, final_hu=hu, final_hv=hv, final_node_volume=V,
        final_link_flow=Q, wet_time=wt, ledger=dict(zip(names, list(res.ledger))), error=res.error,
        error_step=res.error_step, recharge_storage=rstore,
        step_end=(start.step_end if start is not None else 0) + res.step_count,
        cached_dt_s=res.cached_dt_s, next_snapshot_s=res.next_snapshot_s,
    )


def num_threads() -> int:
    return int(lib().orc_num_threads())
