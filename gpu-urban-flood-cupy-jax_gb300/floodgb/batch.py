"""``BatchSolver``: many surface scenarios advanced together on one GPU.

Scenarios are cities (any mesh sizes) with their own rainfall, forcing,
duration and adaptive dt.  The library concatenates their tiles and runs one
persistent surface launch plus one planning launch per lockstep step, so a
64-scenario ensemble costs about what one mesh of the combined size costs,
instead of 64 runs of launch-bound small meshes.  Each scenario follows the
single-instance step exactly (``FloodSolver.run`` gives bitwise the same
states).  Drainage is not part of the batched path.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native as N
from .config import RunConfig
from .solver import Progress, _stream_handle, build_descriptors, city_infiltration


@dataclass
class Member:
    """One member of a batch: a city, its rainfall and its run configuration."""

    city: object
    rainfall: object
    cfg: RunConfig
    duration_s: float | None = None


class BatchSolver:
    """Device solver for a batch of surface-only scenarios (see module docstring)."""

    def __init__(self, scenarios: list[Member], shape: N.FlBatchShape | dict | None = None, device: int = 0):
        lib = N.load()
        n = len(scenarios)
        if n == 0:
            raise ValueError("a batch needs at least one scenario")
        descs = []
        for sc in scenarios:
            topo = sc.city.topologies
            fields, simple = city_infiltration(sc.city, sc.cfg)
            descs.append(build_descriptors(
                topo.surface_topology, rainfall=sc.rainfall, infiltration_fields=fields, infiltration_mps=simple,
                cfg=sc.cfg, duration_s=sc.duration_s, centroids=sc.city.mesh.centroids_xy))
        meshes = (N.FlMeshDesc * n)(*[d.mesh for d in descs])
        forcings = (N.FlForcingDesc * n)(*[d.forcing for d in descs])
        params = (N.FlParams * n)(*[d.params for d in descs])
        if isinstance(shape, dict):
            shape = N.FlBatchShape(**shape)
        handle = C.c_void_p()
        rc = lib.fl_batch_create(int(n), meshes, forcings, params, C.byref(shape) if shape is not None else None,
                                 int(device), C.byref(handle))
        N.check(rc, "fl_batch_create")
        self._h = handle
        self._lib = lib
        self.n = n
        self.cell_counts = [sc.city.topologies.surface_topology.cell_count for sc in scenarios]
        self.durations_s = [d.duration_s for d in descs]
        for k, sc in enumerate(scenarios):
            st = sc.city.topologies.surface_state
            if np.any(st.h_m) or np.any(st.hu_m2ps) or np.any(st.hv_m2ps):
                self.set_state(k, st.h_m, st.hu_m2ps, st.hv_m2ps)

    # ------------------------------------------------------------- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fl_batch_destroy(self._h)
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

    # ------------------------------------------------------------- running
    def set_state(self, scen: int, h=None, hu=None, hv=None, stream=None) -> None:
        arrs = [np.ascontiguousarray(a, np.float32) if a is not None else None for a in (h, hu, hv)]
        p = [C.c_void_p(a.ctypes.data) if a is not None else None for a in arrs]
        N.check(self._lib.fl_batch_set_state(self._h, int(scen), p[0], p[1], p[2], N.FL_MEM_HOST,
                                             _stream_handle(stream)), "fl_batch_set_state")

    def run(self, max_steps: int = 0, stream=None) -> None:
        """Every scenario from t = 0 to its own duration (or max_steps lockstep steps)."""

        N.check(self._lib.fl_batch_run(self._h, int(max_steps), _stream_handle(stream)), "fl_batch_run")

    def info(self) -> dict:
        shape = N.FlBatchShape()
        cells, tiles, grid = C.c_int64(), C.c_int64(), C.c_int32()
        N.check(self._lib.fl_batch_info(self._h, C.byref(shape), C.byref(cells), C.byref(tiles), C.byref(grid)),
                "fl_batch_info")
        return {"tile_cells": shape.tile_cells, "ctas_per_sm": shape.ctas_per_sm, "chunk_steps": shape.chunk_steps,
                "smem_bytes": shape.reserved, "cells": cells.value, "tiles": tiles.value, "grid": grid.value}

    # ------------------------------------------------------------- results
    def progress(self, scen: int, stream=None) -> Progress:
        p = N.FlProgress()
        N.check(self._lib.fl_batch_progress(self._h, int(scen), C.byref(p), _stream_handle(stream)),
                "fl_batch_progress")
        return Progress(p.t_s, p.step_count, p.cfl_eval_count, p.cfl_reused_count, p.snapshot_count, p.error,
                        p.error_step, p.last_dt_s)

    def state(self, scen: int, stream=None):
        c = self.cell_counts[scen]
        h, hu, hv = (np.empty(c, np.float32) for _ in range(3))
        N.check(self._lib.fl_batch_get_state(self._h, int(scen), C.c_void_p(h.ctypes.data),
                                             C.c_void_p(hu.ctypes.data), C.c_void_p(hv.ctypes.data), N.FL_MEM_HOST,
                                             _stream_handle(stream)), "fl_batch_get_state")
        return h, hu, hv

    def snapshots(self, scen: int, stream=None, momentum: bool = False):
        """(times_s, h, hmax) of every snapshot of a scenario; hmax = maximum
        depth since the previous snapshot.  With momentum, (times_s, h, hmax,
        hu, hv)."""

        n = self.progress(scen, stream).snapshot_count
        c = self.cell_counts[scen]
        t = np.empty(n, np.float64)
        h = np.empty((n, c), np.float32)
        hm = np.empty((n, c), np.float32)
        if n:
            N.check(self._lib.fl_batch_get_snapshots(self._h, int(scen), 0, int(n), C.c_void_p(t.ctypes.data),
                                                     C.c_void_p(h.ctypes.data), C.c_void_p(hm.ctypes.data),
                                                     N.FL_MEM_HOST, _stream_handle(stream)), "fl_batch_get_snapshots")
        if not momentum:
            return t, h, hm
        hu = np.empty((n, c), np.float32)
        hv = np.empty((n, c), np.float32)
        if n:
            N.check(self._lib.fl_batch_get_snapshot_momentum(self._h, int(scen), 0, int(n), C.c_void_p(hu.ctypes.data),
                                                             C.c_void_p(hv.ctypes.data), N.FL_MEM_HOST,
                                                             _stream_handle(stream)), "fl_batch_get_snapshot_momentum")
        return t, h, hm, hu, hv

    def ledger(self, scen: int, stream=None) -> dict:
        out = (C.c_double * len(N.LEDGER_NAMES))()
        N.check(self._lib.fl_batch_read_ledger(self._h, int(scen), out, len(N.LEDGER_NAMES), _stream_handle(stream)),
                "fl_batch_read_ledger")
        d = dict(zip(N.LEDGER_NAMES[:4] + [N.LEDGER_NAMES[10]], [float(out[i]) for i in (0, 1, 2, 3, 10)]))
        d["boundary_net_flux_m3"] = d["boundary_inflow_m3"] - d["boundary_outflow_m3"]
        return d


def measure_ensemble(per_size: int = 16, duration_cap_h: float | None = None, sequential_per_size: int = 2,
                     tune_shape: bool = True, seed: int = 2) -> dict:
    """The ragged batched ensemble: per_size members at each of the four mesh
    sizes (10,082 / 49,928 / 100,352 / 250,632 triangles), seeded storms with
    peak 20-120 mm/h over 1-6 h, each member run for its storm's duration,
    all in one persistent launch per step (launch shape from the autotuner).
    The plain single-instance solver is timed on sequential_per_size members
    of each size, and its scenario-hours/s is extrapolated per size to the
    whole ensemble."""

    import time

    import torch

    from .autotune import tune
    from .solver import solver_for_city
    from .synthetic import ensemble_workload

    members = ensemble_workload(seed=seed, per_size=per_size, duration_cap_h=duration_cap_h)
    hours = sum(m.duration_s for m in members) / 3600.0
    shape = tune(members) if tune_shape else {"tile_cells": 256, "ctas_per_sm": 0}
    with BatchSolver(members, shape=shape) as b:
        torch.cuda.synchronize()
        t = time.perf_counter()
        b.run()
        torch.cuda.synchronize()
        batched_s = time.perf_counter() - t
        steps = [b.progress(k).step_count for k in range(b.n)]
        cell_steps = sum(s * c for s, c in zip(steps, b.cell_counts))
        info = b.info()
    # plain solver: per mesh size, the mean time per simulated hour of a sample
    per_hour = {}
    for k0 in range(0, len(members), per_size):
        group = members[k0:k0 + per_size]
        secs = hrs = 0.0
        for m in group[:sequential_per_size]:
            s = solver_for_city(m.city, m.rainfall, m.cfg, duration_s=m.duration_s)
            torch.cuda.synchronize()
            t = time.perf_counter()
            s.run()
            torch.cuda.synchronize()
            secs += time.perf_counter() - t
            hrs += m.duration_s / 3600.0
            s.close()
        per_hour[group[0].city.topologies.surface_topology.cell_count] = secs / hrs
    seq_s = sum(per_hour[m.city.topologies.surface_topology.cell_count] * m.duration_s / 3600.0 for m in members)
    return {
        "members": len(members), "scenario_hours": hours, "batched_s": batched_s,
        "batched_scenario_h_per_s": hours / batched_s, "batched_cell_steps_per_s": cell_steps / batched_s,
        "single_instance_scenario_h_per_s": hours / seq_s, "single_instance_s_estimated": seq_s,
        "batched_over_single": seq_s / batched_s, "shape": {k: info[k] for k in ("tile_cells", "ctas_per_sm", "grid", "tiles")},
        "single_instance_sample": f"{sequential_per_size} members per mesh size, extrapolated per size",
    }


def main():
    import argparse
    import json

    p = argparse.ArgumentParser(description="time the ragged batched ensemble against the single-instance solver")
    p.add_argument("--per-size", type=int, default=16)
    p.add_argument("--cap-h", type=float, default=None)
    p.add_argument("--sequential-per-size", type=int, default=2)
    p.add_argument("--no-tune", action="store_true")
    a = p.parse_args()
    print(json.dumps(measure_ensemble(a.per_size, a.cap_h, a.sequential_per_size, not a.no_tune)))


if __name__ == "__main__":
    main()
