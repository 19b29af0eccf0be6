"""``FloodSolver``: one device-resident solver over libfloodgb's C ABI.

A solver owns the renumbered device layout of one city (mesh, drainage,
forcing fields) and its state.  ``run`` advances the reference's adaptive
loop on the device; ``step`` runs one explicit step (or a subset of its
phases) for function-level use.  State arrays are exchanged in the
reference's cell order, either as host NumPy arrays or as CUDA tensors.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import native as N
from .config import RunConfig, load_config
from .rainfall import RainfallEvent, hyetograph_arrays


def _stream_handle(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(None)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    handle = getattr(stream, "cuda_stream", None)
    if handle is None:
        raise TypeError("stream must be None, an int handle or a torch.cuda.Stream")
    return C.c_void_p(handle)


@dataclass
class Progress:
    t_s: float
    step_count: int
    cfl_eval_count: int
    cfl_reused_count: int
    snapshot_count: int
    error: int
    error_step: int
    last_dt_s: float


@dataclass
class Descriptors:
    """The C-ABI descriptors of one scenario and the host arrays they point into."""

    mesh: N.FlMeshDesc
    drain: N.FlDrainDesc | None
    forcing: N.FlForcingDesc
    params: N.FlParams
    keep: N.Keep
    duration_s: float
    max_snapshots: int
    kind: int


def forcing_desc(rainfall, infiltration_fields, infiltration_mps: float, keep) -> "N.FlForcingDesc":
    """Forcing descriptor: the hyetograph of `rainfall` and the per-cell
    Horton fields (or the scalar infiltration capacity)."""

    if rainfall is not None:
        hs, he, hr = hyetograph_arrays(rainfall)
    else:
        hs = he = hr = np.zeros(0)
    kind = 1 if infiltration_fields is not None else 0
    return N.FlForcingDesc(
        kind=kind,
        rain_multiplier=keep.f32(infiltration_fields.rainfall_multiplier if kind else None),
        horton_f0_mps=keep.f32(infiltration_fields.horton_f0_mps if kind else None),
        horton_fc_mps=keep.f32(infiltration_fields.horton_fc_mps if kind else None),
        horton_k_per_s=keep.f32(infiltration_fields.horton_k_per_s if kind else None),
        infiltration_mps=float(np.float32(infiltration_mps)),
        hyetograph_count=int(np.asarray(hs).size),
        hyeto_start_s=keep.f64(hs), hyeto_end_s=keep.f64(he), hyeto_rate_mps=keep.f64(hr),
    )


def build_descriptors(surface_topology, coupling_topology=None, pipe_topology=None, *, rainfall=None,
                      infiltration_fields=None, infiltration_mps: float = 0.0, cfg: RunConfig | None = None,
                      duration_s: float | None = None, centroids=None, boundary_stage_m: float | None = None,
                      max_snapshots: int | None = None, gravity_mps2: float = 9.80665,
                      min_depth_m: float = 1.0e-5) -> Descriptors:
    """Mesh / drainage / forcing / parameter descriptors of one scenario."""

    cfg = cfg or load_config()
    s = cfg.solver
    ph = cfg.physics
    if duration_s is None:
        if s.duration_min is not None:
            duration_s = float(s.duration_min) * 60.0
        elif rainfall is not None:
            duration_s = float(rainfall.duration_min) * 60.0
        else:
            raise ValueError("duration_s, solver.duration_min or a rainfall event is needed")
    duration_s = float(duration_s)
    if surface_topology.has_stage_boundary and boundary_stage_m is None:
        raise ValueError("dirichlet_stage triangular boundary requires boundary_stage_m.")
    keep = N.Keep()
    mesh = N.mesh_desc(surface_topology, keep, centroids, boundary_stage_m)
    drain = None
    if coupling_topology is not None and coupling_topology.node_count > 0:
        drain = N.drain_desc(coupling_topology, pipe_topology, keep, ph.inlet_capture_rule,
                             ph.inlet_orifice_area_m2, ph.inlet_orifice_coefficient,
                             ph.inlet_weir_perimeter_m, ph.inlet_weir_coefficient)
    kind = 1 if infiltration_fields is not None else 0
    forcing = forcing_desc(rainfall, infiltration_fields, infiltration_mps, keep)
    if max_snapshots is None:
        max_snapshots = int(math.ceil(duration_s / (s.snapshot_interval_min * 60.0))) + 2
    params = N.FlParams(
        gravity_mps2=gravity_mps2, min_depth_m=min_depth_m, cfl=s.cfl,
        cfl_update_interval_steps=int(s.cfl_update_interval_steps),
        cfl_reuse_safety_factor=s.cfl_reuse_safety_factor, max_dt_s=s.max_dt_s, max_speed_mps=s.max_speed_mps,
        finite_check_interval_steps=int(s.finite_check_interval_steps), duration_s=duration_s,
        snapshot_interval_s=s.snapshot_interval_min * 60.0, max_snapshots=int(max_snapshots),
        surface_step_mode=1 if s.surface_step_mode == "local_inertial" else 0,
    )
    return Descriptors(mesh, drain, forcing, params, keep, duration_s, int(max_snapshots), kind)


def city_infiltration(city, cfg: RunConfig):
    """(per-cell Horton fields or None, scalar capacity) the engine derives for a city."""

    ph = cfg.physics
    fields = city.infiltration_fields if ph.infiltration_mode == "production_horton" else None
    simple = city.simple_infiltration_mps if ph.infiltration_mode != "production_horton" else None
    if fields is None and simple is not None and np.ndim(simple) > 0:
        # per-cell constant capacity: Horton with f0 = fc = capacity, k = 0, unit rain multiplier
        from .domain import ProductionInfiltrationFields

        f = np.asarray(simple, np.float32)
        fields = ProductionInfiltrationFields(
            rainfall_multiplier=np.ones_like(f), horton_f0_mps=f, horton_fc_mps=f,
            horton_k_per_s=np.zeros_like(f), open_fraction=np.ones_like(f), active_mask=np.ones(f.shape, bool))
        simple = None
    return fields, float(simple) if simple is not None else 0.0


class FloodSolver:
    """Device solver for one city (surface mesh, optional drainage, forcing)."""

    def __init__(
        self,
        surface_topology,
        coupling_topology=None,
        pipe_topology=None,
        *,
        rainfall: RainfallEvent | None = None,
        infiltration_fields=None,
        infiltration_mps: float = 0.0,
        cfg: RunConfig | None = None,
        duration_s: float | None = None,
        centroids=None,
        boundary_stage_m: float | None = None,
        max_snapshots: int | None = None,
        device: int = 0,
        gravity_mps2: float = 9.80665,
        min_depth_m: float = 1.0e-5,
    ):
        lib = N.load()
        cfg = cfg or load_config()
        d = build_descriptors(surface_topology, coupling_topology, pipe_topology, rainfall=rainfall,
                              infiltration_fields=infiltration_fields, infiltration_mps=infiltration_mps, cfg=cfg,
                              duration_s=duration_s, centroids=centroids, boundary_stage_m=boundary_stage_m,
                              max_snapshots=max_snapshots, gravity_mps2=gravity_mps2, min_depth_m=min_depth_m)
        self.cfg = cfg
        self.duration_s = d.duration_s
        self.cell_count = surface_topology.cell_count
        self.node_count = coupling_topology.node_count if coupling_topology is not None else 0
        self.link_count = pipe_topology.link_count if pipe_topology is not None else 0
        self.kind = d.kind
        self.max_snapshots = d.max_snapshots
        handle = C.c_void_p()
        rc = lib.fl_create(C.byref(d.mesh), C.byref(d.drain) if d.drain is not None else None, C.byref(d.forcing),
                           C.byref(d.params), int(device), C.byref(handle))
        N.check(rc, "fl_create")
        self._h = handle
        self._lib = lib
        self._keep = None  # the library copied everything it needs

    # ------------------------------------------------------------- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------- state
    @staticmethod
    def _ptr(a, dtype, keep):
        if a is None:
            return None, N.FL_MEM_HOST
        if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
            if not a.is_contiguous():
                raise ValueError("device tensors must be contiguous")
            return C.c_void_p(a.data_ptr()), N.FL_MEM_DEVICE
        arr = np.ascontiguousarray(np.asarray(a), dtype=dtype)
        keep.append(arr)
        return C.c_void_p(arr.ctypes.data), N.FL_MEM_HOST

    def set_state(self, h=None, hu=None, hv=None, node_volume=None, link_flow=None, wet_time=None, stream=None):
        keep = []
        ptrs = []
        kinds = set()
        for a, dt in ((h, np.float32), (hu, np.float32), (hv, np.float32), (node_volume, np.float64),
                      (link_flow, np.float64), (wet_time, np.float32)):
            p, k = self._ptr(a, dt, keep)
            ptrs.append(p)
            if a is not None:
                kinds.add(k)
        if len(kinds) > 1:
            raise ValueError("mix of host and device arrays in one set_state call")
        mem = kinds.pop() if kinds else N.FL_MEM_HOST
        rc = self._lib.fl_set_state(self._h, *ptrs, mem, _stream_handle(stream))
        N.check(rc, "fl_set_state")

    def get_state(self, stream=None, wet_time: bool = False):
        """Host copies (reference order): h, hu, hv, node_volume, link_flow[, wet_time]."""

        c = self.cell_count
        h, hu, hv = np.empty(c, np.float32), np.empty(c, np.float32), np.empty(c, np.float32)
        V = np.empty(self.node_count, np.float64)
        Q = np.empty(self.link_count, np.float64)
        wt = np.empty(c, np.float32) if wet_time else None
        p = lambda a: C.c_void_p(a.ctypes.data) if a is not None and a.size else None  # noqa: E731
        rc = self._lib.fl_get_state(self._h, p(h), p(hu), p(hv), p(V), p(Q), p(wt), N.FL_MEM_HOST,
                                    _stream_handle(stream))
        N.check(rc, "fl_get_state")
        return (h, hu, hv, V, Q, wt) if wet_time else (h, hu, hv, V, Q)

    def get_state_device(self, h, hu, hv, node_volume=None, link_flow=None, stream=None):
        """Write the state into caller CUDA tensors (reference order)."""

        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        rc = self._lib.fl_get_state(self._h, ptr(h), ptr(hu), ptr(hv), ptr(node_volume), ptr(link_flow), None,
                                    N.FL_MEM_DEVICE, _stream_handle(stream))
        N.check(rc, "fl_get_state")

    def update_forcing(self, rain_multiplier=None, f0=None, fc=None, k=None, infiltration_mps: float = 0.0):
        keep = N.Keep()
        rc = self._lib.fl_update_forcing(self._h, keep.f32(rain_multiplier), keep.f32(f0), keep.f32(fc), keep.f32(k),
                                         float(np.float32(infiltration_mps)))
        N.check(rc, "fl_update_forcing")

    # ------------------------------------------------- inflow and recharge
    def set_boundary_inflow(self, external) -> None:
        """External boundary inflow from an ExternalBoundaryInflowSurface
        (receiver_cell_index, times_s, q_m3ps_by_receiver [times x receivers]);
        None removes it.  Reference production_event_support.py:169-196."""

        keep = N.Keep()
        if external is None or np.asarray(external.receiver_cell_index).size == 0:
            rc = self._lib.fl_set_boundary_inflow(self._h, 0, None, 0, None, None)
        else:
            cells = np.asarray(external.receiver_cell_index, np.int32)
            times = np.asarray(external.times_s, np.float64)
            q = np.asarray(external.q_m3ps_by_receiver, np.float32)
            if q.shape != (times.size, cells.size):
                raise ValueError(f"q_m3ps_by_receiver has shape {q.shape}, expected {(times.size, cells.size)}")
            rc = self._lib.fl_set_boundary_inflow(self._h, cells.size, keep.i32(cells), times.size, keep.f64(times),
                                                  keep.f32(q))
        N.check(rc, "fl_set_boundary_inflow")
        self.inflow_receivers = 0 if external is None else int(np.asarray(external.receiver_cell_index).size)

    def set_recharge(self, topo) -> None:
        """Surface recharge rows from a June5RechargeTopology (float32 rows);
        None removes it.  Reference june5_production_drainage.py:543-572."""

        keep = N.Keep()
        n = 0 if topo is None else int(np.asarray(topo.source_cell_index).size)
        if n == 0:
            rc = self._lib.fl_set_recharge(self._h, 0, None, None, None, None, None)
        else:
            rc = self._lib.fl_set_recharge(self._h, n, keep.i32(topo.source_cell_index),
                                           keep.f32(topo.storage_capacity_m3), keep.f32(topo.capture_capacity_m3ps),
                                           keep.f32(topo.recharge_capacity_m3ps), keep.f32(topo.stop_depth_m))
        N.check(rc, "fl_set_recharge")
        self.recharge_rows = n

    def recharge_storage(self, stream=None) -> np.ndarray:
        n = getattr(self, "recharge_rows", 0)
        out = np.zeros(n, np.float32)
        if n:
            rc = self._lib.fl_get_recharge_storage(self._h, C.c_void_p(out.ctypes.data), n, N.FL_MEM_HOST,
                                                   _stream_handle(stream))
            N.check(rc, "fl_get_recharge_storage")
        return out

    def set_recharge_storage(self, storage, stream=None) -> None:
        a = np.ascontiguousarray(storage, np.float32)
        rc = self._lib.fl_set_recharge_storage(self._h, C.c_void_p(a.ctypes.data), a.size, N.FL_MEM_HOST,
                                               _stream_handle(stream))
        N.check(rc, "fl_set_recharge_storage")

    # ------------------------------------------------------------- stepping
    def reset_clock(self, stream=None):
        N.check(self._lib.fl_reset_clock(self._h, _stream_handle(stream)), "fl_reset_clock")

    def run(self, t_target_s: float | None = None, max_steps: int = 0, stream=None):
        t = self.duration_s if t_target_s is None else float(t_target_s)
        N.check(self._lib.fl_run(self._h, t, int(max_steps), _stream_handle(stream)), "fl_run")

    def step(self, dt_s: float, phases: int = N.FL_PHASE_ALL, rain_rate_mps: float = 0.0, stream=None):
        N.check(self._lib.fl_step(self._h, float(dt_s), int(phases), float(rain_rate_mps), _stream_handle(stream)),
                "fl_step")

    def stable_timestep(self, stream=None) -> float:
        v = C.c_double(0.0)
        N.check(self._lib.fl_stable_timestep(self._h, C.byref(v), _stream_handle(stream)), "fl_stable_timestep")
        return float(v.value)

    def time_kernel(self, kernel: int, reps: int = 50, stream=None) -> float:
        """Mean ms per launch of one step kernel (0 surface, 1 inlets, 2 network, 3 CFL, 4 links, 5 donor
        factors), launched in chains as in the step loop."""

        v = C.c_double(0.0)
        N.check(self._lib.fl_time_kernel(self._h, int(kernel), int(reps), _stream_handle(stream), C.byref(v)),
                "fl_time_kernel")
        return float(v.value)

    def progress(self, stream=None) -> Progress:
        p = N.FlProgress()
        N.check(self._lib.fl_get_progress(self._h, C.byref(p), _stream_handle(stream)), "fl_get_progress")
        return Progress(p.t_s, p.step_count, p.cfl_eval_count, p.cfl_reused_count, p.snapshot_count, p.error,
                        p.error_step, p.last_dt_s)

    def ledger(self, stream=None) -> dict:
        out = (C.c_double * len(N.LEDGER_NAMES))()
        N.check(self._lib.fl_read_ledger(self._h, out, len(N.LEDGER_NAMES), _stream_handle(stream)), "fl_read_ledger")
        d = dict(zip(N.LEDGER_NAMES, [float(v) for v in out]))
        d["boundary_net_flux_m3"] = d["boundary_inflow_m3"] - d["boundary_outflow_m3"]
        return d

    def snapshots(self, first: int = 0, count: int | None = None, stream=None):
        """(times_s, h, hu, hv, node_volume) of snapshots [first, first+count), reference order."""

        n = self.progress(stream).snapshot_count
        count = n - first if count is None else count
        c = self.cell_count
        t = np.empty(count, np.float64)
        h = np.empty((count, c), np.float32)
        hu = np.empty((count, c), np.float32)
        hv = np.empty((count, c), np.float32)
        v = np.empty((count, self.node_count), np.float32)
        p = lambda a: C.c_void_p(a.ctypes.data) if a.size else None  # noqa: E731
        rc = self._lib.fl_get_snapshots(self._h, int(first), int(count), p(t), p(h), p(hu), p(hv), p(v),
                                        N.FL_MEM_HOST, _stream_handle(stream))
        N.check(rc, "fl_get_snapshots")
        return t, h, hu, hv, v


def solver_for_city(city, rainfall, cfg: RunConfig, duration_s: float | None = None, device: int = 0,
                    max_snapshots: int | None = None) -> FloodSolver:
    """FloodSolver for a CityDomain, with the forcing the engine would derive."""

    topo = city.topologies
    fields, simple = city_infiltration(city, cfg)
    s = FloodSolver(
        topo.surface_topology, topo.coupling_topology, topo.pipe_topology, rainfall=rainfall,
        infiltration_fields=fields, infiltration_mps=simple, cfg=cfg,
        duration_s=duration_s, centroids=city.mesh.centroids_xy, device=device, max_snapshots=max_snapshots,
    )
    s.set_state(topo.surface_state.h_m, topo.surface_state.hu_m2ps, topo.surface_state.hv_m2ps,
                topo.pipe_state.node_volume_m3 if s.node_count else None,
                topo.pipe_state.link_flow_m3ps if s.link_count else None)
    if getattr(city, "external_boundary", None) is not None:
        s.set_boundary_inflow(city.external_boundary)
    if getattr(city, "recharge_topology", None) is not None:
        s.set_recharge(city.recharge_topology)
    s.reset_clock()
    return s


class MemberSolver(FloodSolver):
    """Ensemble members on one city (fl_create_members): the same mesh,
    drainage network, infiltration fields and parameters, one rainfall event
    per member; each member its own state, adaptive dt, snapshots and ledger.
    run() advances every member to the end of the run; the other methods
    address the member chosen with select() (member 0 at first)."""

    def __init__(self, surface_topology, coupling_topology=None, pipe_topology=None, *, rainfalls,
                 infiltration_fields=None, infiltration_mps: float = 0.0, cfg: RunConfig | None = None,
                 duration_s: float | None = None, centroids=None, max_snapshots: int | None = None, device: int = 0,
                 gravity_mps2: float = 9.80665, min_depth_m: float = 1.0e-5):
        lib = N.load()
        cfg = cfg or load_config()
        rainfalls = list(rainfalls)
        if not rainfalls:
            raise ValueError("at least one member is needed")
        d = build_descriptors(surface_topology, coupling_topology, pipe_topology, rainfall=rainfalls[0],
                              infiltration_fields=infiltration_fields, infiltration_mps=infiltration_mps, cfg=cfg,
                              duration_s=duration_s, centroids=centroids, max_snapshots=max_snapshots,
                              gravity_mps2=gravity_mps2, min_depth_m=min_depth_m)
        forcings = (N.FlForcingDesc * len(rainfalls))()
        forcings[0] = d.forcing
        for m, r in enumerate(rainfalls[1:], start=1):
            forcings[m] = forcing_desc(r, infiltration_fields, infiltration_mps, d.keep)
        self.cfg = cfg
        self.duration_s = d.duration_s
        self.cell_count = surface_topology.cell_count
        self.node_count = coupling_topology.node_count if coupling_topology is not None else 0
        self.link_count = pipe_topology.link_count if pipe_topology is not None else 0
        self.kind = d.kind
        self.max_snapshots = d.max_snapshots
        self.members = len(rainfalls)
        handle = C.c_void_p()
        rc = lib.fl_create_members(C.byref(d.mesh), C.byref(d.drain) if d.drain is not None else None, forcings,
                                   len(rainfalls), C.byref(d.params), int(device), C.byref(handle))
        N.check(rc, "fl_create_members")
        self._h = handle
        self._lib = lib
        self._keep = None

    def select(self, member: int) -> "MemberSolver":
        N.check(self._lib.fl_member_select(self._h, int(member)), "fl_member_select")
        return self

    def run(self, t_target_s: float | None = None, max_steps: int = 0, stream=None):
        """Every member to the end of the run."""

        return super().run(None, 0, stream=stream)


def members_for_city(city, rainfalls, cfg: RunConfig, duration_s: float | None = None, device: int = 0,
                     max_snapshots: int | None = None) -> MemberSolver:
    """MemberSolver for a CityDomain and one rainfall event per member, each
    member starting from the city's initial state."""

    topo = city.topologies
    if getattr(city, "external_boundary", None) is not None or getattr(city, "recharge_topology", None) is not None:
        raise ValueError("ensemble members support neither external inflow nor surface recharge")
    fields, simple = city_infiltration(city, cfg)
    s = MemberSolver(topo.surface_topology, topo.coupling_topology, topo.pipe_topology, rainfalls=rainfalls,
                     infiltration_fields=fields, infiltration_mps=simple, cfg=cfg, duration_s=duration_s,
                     centroids=city.mesh.centroids_xy, device=device, max_snapshots=max_snapshots)
    for m in range(s.members):
        s.select(m).set_state(topo.surface_state.h_m, topo.surface_state.hu_m2ps, topo.surface_state.hv_m2ps,
                              topo.pipe_state.node_volume_m3 if s.node_count else None,
                              topo.pipe_state.link_flow_m3ps if s.link_count else None)
    s.select(0)
    s.reset_clock()
    return s
