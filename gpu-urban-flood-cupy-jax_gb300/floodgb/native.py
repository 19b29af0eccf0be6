"""ctypes binding of ``libfloodgb.so`` (declarations in ``include/floodgb.h``).

There is no CPU fallback: if the library is missing or no CUDA device is
visible, solver creation raises ``BackendUnavailableError`` (as the
reference's engine does when CuPy cannot start, ``engine.py:107-116``).
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .exceptions import BackendUnavailableError, NativeError, SimulationError

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfloodgb.so"

FL_OK = 0
FL_E_INVALID = -1
FL_E_CUDA = -2
FL_E_NO_DEVICE = -3
FL_E_NONFINITE = -4
FL_E_STEP_CAP = -5
FL_E_NOMEM = -6
FL_E_UNSUPPORTED = -7
FL_E_SNAPSHOTS = -8
FL_E_TIMEOUT = -9

FL_PHASE_SURFACE = 1
FL_PHASE_CLAMP = 2
FL_PHASE_DRAINAGE = 4
FL_PHASE_INFLOW = 8
FL_PHASE_RECHARGE = 16
FL_PHASE_ALL = 31
FL_MEM_HOST = 0
FL_MEM_DEVICE = 1

CAPTURE_RULES = {"capacity": 0, "head_limited_capacity": 1, "orifice": 2, "weir_orifice": 3}
LEDGER_NAMES = [
    "rainfall_input_m3", "infiltration_loss_m3", "boundary_inflow_m3", "boundary_outflow_m3",
    "surface_capture_m3", "surface_surcharge_m3", "outfall_discharge_m3", "overflow_surcharge_m3",
    "unreturned_overflow_m3", "link_abs_flow_m3", "surface_volume_m3", "node_volume_m3",
    "external_boundary_inflow_m3", "surface_recharge_capture_m3", "surface_recharge_loss_m3",
]

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)


class FlMeshDesc(C.Structure):
    _fields_ = [
        ("cell_count", C.c_int32), ("edge_count", C.c_int32),
        ("bed_elevation_m", f32p), ("manning_n", f32p), ("cell_area_m2", f32p), ("characteristic_length_m", f32p),
        ("active_mask", f32p),
        ("edge_left_cell", i32p), ("edge_right_cell", i32p), ("boundary_code", i32p),
        ("edge_normal_x", f32p), ("edge_normal_y", f32p), ("edge_length_m", f32p),
        ("centroid_x", f32p), ("centroid_y", f32p),
        ("has_stage_boundary", C.c_int32), ("boundary_stage_m", C.c_float),
    ]


class FlDrainDesc(C.Structure):
    _fields_ = [
        ("node_count", C.c_int32), ("link_count", C.c_int32), ("inlet_count", C.c_int32),
        ("inlet_cell_index", i32p), ("inlet_node_index", i32p), ("node_surface_cell_index", i32p),
        ("node_invert_elevation_m", f32p), ("node_storage_area_m2", f32p), ("node_max_depth_m", f32p),
        ("inlet_capture_capacity_m3ps", f32p), ("inlet_surcharge_capacity_m3ps", f32p),
        ("link_from_node_index", i32p), ("link_to_node_index", i32p),
        ("link_length_m", f32p), ("link_area_m2", f32p), ("link_hydraulic_radius_m", f32p), ("link_manning_n", f32p),
        ("link_flow_capacity_m3ps", f32p), ("link_invert_elevation_m", f32p), ("link_diameter_m", f32p),
        ("link_minor_loss_coefficient", f32p),
        ("link_geometry_code", i32p), ("link_rect_width_m", f32p), ("link_rect_height_m", f32p),
        ("outfall_area_m2", f32p), ("outfall_coefficient", f32p), ("outfall_tailwater_head_m", f32p),
        ("outfall_flow_capacity_m3ps", f32p),
        ("pressurized_wave_speed_mps", C.c_float),
        ("inlet_capture_rule", C.c_int32),
        ("inlet_orifice_area_m2", C.c_float), ("inlet_orifice_coefficient", C.c_float),
        ("inlet_weir_perimeter_m", C.c_float), ("inlet_weir_coefficient", C.c_float),
        ("surcharge_entry_count", C.c_int32), ("surcharge_cell_index", i32p), ("surcharge_node_index", i32p),
        ("surcharge_return_weight", f32p), ("surcharge_return_weight_is_normalized", C.c_int32),
    ]


class FlForcingDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("rain_multiplier", f32p), ("horton_f0_mps", f32p), ("horton_fc_mps", f32p), ("horton_k_per_s", f32p),
        ("infiltration_mps", C.c_float),
        ("hyetograph_count", C.c_int32),
        ("hyeto_start_s", f64p), ("hyeto_end_s", f64p), ("hyeto_rate_mps", f64p),
    ]


class FlParams(C.Structure):
    _fields_ = [
        ("gravity_mps2", C.c_double), ("min_depth_m", C.c_double),
        ("cfl", C.c_double), ("cfl_update_interval_steps", C.c_int32), ("cfl_reuse_safety_factor", C.c_double),
        ("max_dt_s", C.c_double), ("max_speed_mps", C.c_double),
        ("finite_check_interval_steps", C.c_int32),
        ("duration_s", C.c_double), ("snapshot_interval_s", C.c_double),
        ("max_snapshots", C.c_int32), ("surface_step_mode", C.c_int32),
    ]


class FlProgress(C.Structure):
    _fields_ = [
        ("t_s", C.c_double), ("step_count", C.c_int64), ("cfl_eval_count", C.c_int64),
        ("cfl_reused_count", C.c_int64), ("snapshot_count", C.c_int32), ("error", C.c_int32),
        ("error_step", C.c_int64), ("last_dt_s", C.c_double),
    ]


class FlBatchShape(C.Structure):
    _fields_ = [("tile_cells", C.c_int32), ("ctas_per_sm", C.c_int32), ("chunk_steps", C.c_int32),
                ("reserved", C.c_int32)]


class FlGemmSegment(C.Structure):
    _fields_ = [("base", C.c_void_p), ("rows", C.c_void_p), ("ld", C.c_int64), ("width", C.c_int32)]


class FlGemmDesc(C.Structure):
    _fields_ = [
        ("a", FlGemmSegment * 3), ("n_seg", C.c_int32), ("m", C.c_int32), ("n", C.c_int32),
        ("b", C.c_void_p), ("ldb", C.c_int64), ("bias", C.c_void_p), ("residual", C.c_void_p), ("ldr", C.c_int64),
        ("out_f32", C.c_void_p), ("out_bf16", C.c_void_p), ("ldo", C.c_int64), ("relu", C.c_int32),
        ("k_splits", C.c_int32), ("force_tiled", C.c_int32),
    ]


_lib = None

# symbol -> (restype, argtypes)
_SIGNATURES = {
    "fl_abi_version": (C.c_int, []),
    "fl_last_error": (C.c_char_p, []),
    "fl_device_count": (C.c_int, [i32p]),
    "fl_create": (C.c_int, [C.POINTER(FlMeshDesc), C.POINTER(FlDrainDesc), C.POINTER(FlForcingDesc),
                            C.POINTER(FlParams), C.c_int32, C.POINTER(C.c_void_p)]),
    "fl_create_members": (C.c_int, [C.POINTER(FlMeshDesc), C.POINTER(FlDrainDesc), C.POINTER(FlForcingDesc),
                                    C.c_int32, C.POINTER(FlParams), C.c_int32, C.POINTER(C.c_void_p)]),
    "fl_member_select": (C.c_int, [C.c_void_p, C.c_int32]),
    "fl_member_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "fl_destroy": (None, [C.c_void_p]),
    "fl_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_int32, C.c_void_p]),
    "fl_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_int32, C.c_void_p]),
    "fl_reset_clock": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fl_run": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_void_p]),
    "fl_step": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_void_p]),
    "fl_stable_timestep": (C.c_int, [C.c_void_p, f64p, C.c_void_p]),
    "fl_update_forcing": (C.c_int, [C.c_void_p, f32p, f32p, f32p, f32p, C.c_float]),
    "fl_get_progress": (C.c_int, [C.c_void_p, C.POINTER(FlProgress), C.c_void_p]),
    "fl_read_ledger": (C.c_int, [C.c_void_p, f64p, C.c_int32, C.c_void_p]),
    "fl_get_snapshots": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int32, C.c_void_p]),
    "fl_plan_check": (C.c_int, [C.POINTER(FlMeshDesc), C.POINTER(FlDrainDesc), C.POINTER(C.c_int64), i32p]),
    "fl_plan_tiles": (C.c_int, [C.POINTER(FlMeshDesc), C.POINTER(C.c_int64)]),
    "fl_time_kernel": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, f64p]),
    "fl_launch_count": (C.c_int64, []),
    "fl_gemm_bf16": (C.c_int, [C.POINTER(FlGemmDesc), C.c_void_p]),
    "fl_gemm_status": (C.c_int, [C.c_void_p]),
    "fl_wait_selftest": (C.c_int, [C.c_double, i32p, f64p]),
    "fl_transpose_bf16": (C.c_int, [C.POINTER(FlGemmSegment), C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                    C.c_void_p]),
    "fl_segment_sum": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                 C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]),
    "fl_relu_bwd": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                              C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]),
    "fl_colsum": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                            C.c_void_p]),
    "fl_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float,
                          C.c_float, C.c_float, C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "fl_cast_bf16": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "fl_batch_create": (C.c_int, [C.c_int32, C.POINTER(FlMeshDesc), C.POINTER(FlForcingDesc), C.POINTER(FlParams),
                                  C.POINTER(FlBatchShape), C.c_int32, C.POINTER(C.c_void_p)]),
    "fl_batch_destroy": (None, [C.c_void_p]),
    "fl_batch_set_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.c_void_p]),
    "fl_batch_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "fl_batch_progress": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(FlProgress), C.c_void_p]),
    "fl_batch_get_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.c_void_p]),
    "fl_batch_get_snapshots": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int32, C.c_void_p]),
    "fl_batch_get_snapshot_momentum": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                                 C.c_void_p, C.c_int32, C.c_void_p]),
    "fl_batch_read_ledger": (C.c_int, [C.c_void_p, C.c_int32, f64p, C.c_int32, C.c_void_p]),
    "fl_batch_info": (C.c_int, [C.c_void_p, C.POINTER(FlBatchShape), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                i32p]),
    "fl_set_boundary_inflow": (C.c_int, [C.c_void_p, C.c_int32, i32p, C.c_int32, f64p, f32p]),
    "fl_set_recharge": (C.c_int, [C.c_void_p, C.c_int32, i32p, f32p, f32p, f32p, f32p]),
    "fl_get_recharge_storage": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "fl_set_recharge_storage": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "fl_stable_timestep_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                             C.c_double, C.c_double, C.c_void_p, C.c_void_p]),
}


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def load(build_if_missing: bool = False):
    """Load libfloodgb.so (optionally building it first)."""

    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if build_if_missing or os.environ.get("FLOODGB_BUILD", "0") == "1":
            from .build import build_library

            build_library()
        if not LIB_PATH.exists():
            raise BackendUnavailableError(
                f"{LIB_PATH} is not built; run `python -m floodgb.build` (or __graft_entry__.build()) first. "
                "There is no CPU fallback."
            )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return (load().fl_last_error() or b"").decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc == FL_OK:
        return
    msg = last_error()
    text = f"{what}: {msg}" if what else msg
    if rc == FL_E_INVALID:
        raise ValueError(msg)
    if rc == FL_E_NO_DEVICE:
        raise BackendUnavailableError(text)
    if rc in (FL_E_NONFINITE, FL_E_STEP_CAP, FL_E_SNAPSHOTS, FL_E_TIMEOUT):
        raise SimulationError(msg)
    if rc == FL_E_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise NativeError(f"{text} (code {rc})")


def device_count() -> int:
    n = C.c_int32(0)
    load().fl_device_count(C.byref(n))
    return int(n.value)


class Keep:
    """Owns contiguous host copies that a descriptor points into."""

    def __init__(self):
        self.items = []

    def arr(self, a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a), dtype=dtype)
        self.items.append(a)
        return a

    def ptr(self, a, dtype, ctype):
        a = self.arr(a, dtype)
        if a is None:
            return C.cast(None, C.POINTER(ctype))
        return a.ctypes.data_as(C.POINTER(ctype))

    def f32(self, a):
        return self.ptr(a, np.float32, C.c_float)

    def i32(self, a):
        return self.ptr(a, np.int32, C.c_int32)

    def f64(self, a):
        return self.ptr(a, np.float64, C.c_double)


def mesh_desc(topo, keep: Keep, centroids=None, boundary_stage_m=None) -> FlMeshDesc:
    cx = cy = None
    if centroids is not None:
        cen = np.asarray(centroids)
        cx, cy = cen[:, 0], cen[:, 1]
    return FlMeshDesc(
        cell_count=topo.cell_count, edge_count=topo.edge_count,
        bed_elevation_m=keep.f32(topo.bed_elevation_m), manning_n=keep.f32(topo.manning_n),
        cell_area_m2=keep.f32(topo.cell_area_m2), characteristic_length_m=keep.f32(topo.characteristic_length_m),
        active_mask=keep.f32(topo.active_mask),
        edge_left_cell=keep.i32(topo.edge_left_cell), edge_right_cell=keep.i32(topo.edge_right_cell),
        boundary_code=keep.i32(topo.boundary_code),
        edge_normal_x=keep.f32(topo.edge_normal_x), edge_normal_y=keep.f32(topo.edge_normal_y),
        edge_length_m=keep.f32(topo.edge_length_m),
        centroid_x=keep.f32(cx), centroid_y=keep.f32(cy),
        has_stage_boundary=1 if topo.has_stage_boundary else 0,
        boundary_stage_m=float(boundary_stage_m) if boundary_stage_m is not None else 0.0,
    )


def drain_desc(coupling, pipe, keep: Keep, capture_rule="orifice", orifice_area=0.04, orifice_coef=0.62,
               weir_perimeter=0.0, weir_coef=0.45) -> FlDrainDesc:
    if capture_rule not in CAPTURE_RULES:
        raise ValueError("inlet_capture_rule must be 'orifice', 'weir_orifice', 'capacity', or 'head_limited_capacity'.")
    rect = pipe.link_geometry_code is not None and pipe.link_rect_width_m is not None and pipe.link_rect_height_m is not None
    d = FlDrainDesc(
        node_count=coupling.node_count, link_count=pipe.link_count, inlet_count=coupling.inlet_count,
        inlet_cell_index=keep.i32(coupling.inlet_cell_index), inlet_node_index=keep.i32(coupling.inlet_node_index),
        node_surface_cell_index=keep.i32(coupling.node_surface_cell_index),
        node_invert_elevation_m=keep.f32(coupling.node_invert_elevation_m),
        node_storage_area_m2=keep.f32(coupling.node_storage_area_m2),
        node_max_depth_m=keep.f32(coupling.node_max_depth_m),
        inlet_capture_capacity_m3ps=keep.f32(coupling.inlet_capture_capacity_m3ps),
        inlet_surcharge_capacity_m3ps=keep.f32(coupling.inlet_surcharge_capacity_m3ps),
        link_from_node_index=keep.i32(pipe.link_from_node_index), link_to_node_index=keep.i32(pipe.link_to_node_index),
        link_length_m=keep.f32(pipe.link_length_m), link_area_m2=keep.f32(pipe.link_area_m2),
        link_hydraulic_radius_m=keep.f32(pipe.link_hydraulic_radius_m), link_manning_n=keep.f32(pipe.link_manning_n),
        link_flow_capacity_m3ps=keep.f32(pipe.link_flow_capacity_m3ps),
        link_invert_elevation_m=keep.f32(pipe.link_invert_elevation_m),
        link_diameter_m=keep.f32(pipe.link_diameter_m),
        link_minor_loss_coefficient=keep.f32(pipe.link_minor_loss_coefficient),
        link_geometry_code=keep.i32(pipe.link_geometry_code if rect else None),
        link_rect_width_m=keep.f32(pipe.link_rect_width_m if rect else None),
        link_rect_height_m=keep.f32(pipe.link_rect_height_m if rect else None),
        outfall_area_m2=keep.f32(pipe.outfall_area_m2), outfall_coefficient=keep.f32(pipe.outfall_coefficient),
        outfall_tailwater_head_m=keep.f32(pipe.outfall_tailwater_head_m),
        outfall_flow_capacity_m3ps=keep.f32(pipe.outfall_flow_capacity_m3ps),
        pressurized_wave_speed_mps=float(pipe.pressurized_wave_speed_mps),
        inlet_capture_rule=CAPTURE_RULES[capture_rule],
        inlet_orifice_area_m2=float(orifice_area), inlet_orifice_coefficient=float(orifice_coef),
        inlet_weir_perimeter_m=float(weir_perimeter), inlet_weir_coefficient=float(weir_coef),
    )
    # the weighted return table is used when all three arrays are given (reference :1424-1428)
    sc, sn, sw = coupling.surcharge_cell_index, coupling.surcharge_node_index, coupling.surcharge_return_weight
    if sc is not None and sn is not None and sw is not None:
        n = int(np.asarray(sc).size)
        if np.asarray(sn).size != n or np.asarray(sw).size != n:
            raise ValueError("surcharge_cell_index, surcharge_node_index and surcharge_return_weight differ in length")
        d.surcharge_entry_count = n
        d.surcharge_cell_index = keep.i32(sc)
        d.surcharge_node_index = keep.i32(sn)
        d.surcharge_return_weight = keep.f32(sw)
        d.surcharge_return_weight_is_normalized = int(bool(coupling.surcharge_return_weight_is_normalized))
    return d


def plan_check(topo, coupling=None, pipe=None, centroids=None):
    """Host-only layout build (no GPU): stats dict and the cell permutation."""

    keep = Keep()
    m = mesh_desc(topo, keep, centroids)
    d = drain_desc(coupling, pipe, keep) if coupling is not None and coupling.node_count > 0 else None
    stats = (C.c_int64 * 8)()
    perm = np.empty(topo.cell_count, np.int32)
    rc = load().fl_plan_check(C.byref(m), C.byref(d) if d is not None else None, stats,
                              perm.ctypes.data_as(i32p))
    check(rc, "fl_plan_check")
    names = ["cells", "edges", "slots", "inlet_cells", "nodes", "links", "groups", "max_inlets_per_cell"]
    return dict(zip(names, [int(v) for v in stats])), perm


def plan_tiles(topo, centroids=None):
    """Host-only surface tiling report (no GPU): tiles, entries, halo cells,
    largest tile entry count and halo, shared memory per CTA (bytes)."""

    keep = Keep()
    m = mesh_desc(topo, keep, centroids)
    out = (C.c_int64 * 6)()
    check(load().fl_plan_tiles(C.byref(m), out), "fl_plan_tiles")
    names = ["tiles", "entries", "halo_cells", "max_entries", "max_halo", "smem_bytes"]
    return dict(zip(names, [int(v) for v in out]))
