#!/usr/bin/env python
"""Benchmark: cell-steps/s of the production-shaped coupled 60-minute run.

One bench step is one full 60-minute simulated run of the 981,880-triangle
coupled city (seeded synthetic inputs with the production counts: 1,490,015
edges, 817,573 active cells, 118,768 nodes, 139,798 links, 61,317 inlets, 46
outfalls; Horton infiltration; hour 1 of a 160 mm / 24 h front-loaded
hyetograph), exactly the workload the reference's headline benchmark runs.
The adaptive loop runs on the device (CUDA-graph chunks); each run starts
from the same initial state with L2 flushed (512 MB write) beforehand.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  With --impl reference the C oracle (the
CPU restatement of the reference's step, all host threads) is timed on a
bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "gpu-urban-flood-cupy-jax_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "cell-steps/s, 1M-tri coupled SWE on 1 GB300"
UNIT = "cell-steps/s"
REFERENCE_PUBLISHED = 7.447e8  # reference CuPy, RTX PRO 4000 Blackwell, real 981,880-tri city (derived)
# the reference arm's sample: adaptive steps continued from the state half
# way through the run (step 1,995 of 3,990), a wet mid-run state
MID_RUN_STEP = 1995
WORKLOAD = ("production-shaped coupled 60-min run: 981,880 triangles, 1,490,015 edges, 817,573 active, "
            "118,768 nodes, 139,798 links, 61,317 inlets, 46 outfalls, Horton infiltration, hour 1 of a "
            "160 mm/24 h front-loaded hyetograph")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ensemble", action="store_true", help="skip the ensemble / surrogate screening measurement")
    p.add_argument("--no-long-run", action="store_true", help="skip the 24 h single-instance run")
    p.add_argument("--cpu-seconds", type=float, default=60.0,
                   help="reference arm: CPU seconds spread over the timed samples")
    p.add_argument("--mid-run-step", type=int, default=MID_RUN_STEP,
                   help="reference arm: the step of the 60-min run its samples continue from")
    p.add_argument("--profile", choices=["loop", "kernels", "surrogate"], default=None,
                   help="ncu helper: open a profiler range around 64 solver steps of a wet run (loop) or "
                        "around 2 isolated launches of each step kernel (kernels); prints nothing else")
    p.add_argument("--profile-start-s", type=float, default=900.0)
    p.add_argument("--surface-mode", choices=["full_swe", "local_inertial"], default="full_swe",
                   help="solver.surface_step_mode of the measured run (the headline is full_swe)")
    p.add_argument("--long", action="store_true",
                   help="the 24 h production-shaped run with hourly ledger checks, then 8 concurrent members")
    p.add_argument("--long-hours", type=float, default=24.0)
    p.add_argument("--long-members", type=int, default=8)
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def aggregate_ranks(total_ms: float, cell_steps: float, device=None):
    """Whole-job figures of N replicas: the slowest rank's timed milliseconds
    and the cell-steps of all ranks (each rank solves its own copy of the
    city; there is no data exchange).  One process without a process group
    returns its own figures."""

    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(total_ms), float(cell_steps)
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    cs = torch.tensor([float(cell_steps)], dtype=torch.float64, device=device)
    dist.all_reduce(cs)
    return float(t.item()), float(cs.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# DRAM traffic of one k_surface launch (dram__bytes_read.sum + dram__bytes_write.sum)
# from an ncu capture, keyed by the digest of the sources the kernel is built
# from; a kernel whose sources changed since its capture reports null.
SURFACE_SOURCES = ("fl_surface.cu", "fl_device.cuh", "fl_internal.h")
SURFACE_TRAFFIC_CAPTURES = {
    # two launches at the wet state after 900 s: 74.78 + 2.93 MB and 74.78 + 2.50 MB (549-CTA grid)
    "8643f7e5e23436c8": 77_498_240,
    # the same with the grid over every CTA slot: 74.80 + 2.54 MB and 74.80 + 2.83 MB
    "c4a68efc35e9b1cd": 77_481_984,
    # helper kernels sized from the SM count (k_surface unchanged): 74.80 + 2.55 MB and 74.80 + 2.82 MB
    "f8cff34baccfde73": 77_484_672,
}


def surface_source_digest() -> str:
    import hashlib

    h = hashlib.sha256()
    for name in SURFACE_SOURCES:
        h.update((ROOT / "gpu-urban-flood-cupy-jax_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def surface_traffic_per_launch():
    return SURFACE_TRAFFIC_CAPTURES.get(surface_source_digest())


def workload_config(world: int, surface_mode: str = "full_swe") -> dict:
    """The workload both arms measure (identical in both JSON lines)."""

    return {
        "workload": WORKLOAD, "cells": 981_880, "edges": 1_490_015,
        "step": "one 60-min simulated run (adaptive dt, CFL every 32 steps)",
        "surface_step_mode": surface_mode,
        "l2": "flushed before every run (512 MB write); state reset outside the events",
        "parallelism": f"replicas x{world}",
    }


def cpu_baseline_and_parity(sc, cfg, gpu):
    """The C oracle (all host threads) runs the whole 60-minute workload; its
    wall time is the CPU baseline and its hourly snapshots and final drainage
    state are this line's parity reference for the GPU run ``gpu`` (the
    snapshots, final node volumes and link flows of the last timed run)."""

    import numpy as np

    import oracle
    from floodgb.parity import compare_runs

    oracle.build()
    c = sc.cell_count
    t0 = time.perf_counter()
    r = oracle.run(sc, cfg)
    wall = time.perf_counter() - t0
    base = {
        "value": c * r.step_count / wall, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
        "sample": f"the whole 60-min run ({r.step_count} adaptive steps, {wall:.1f} s, C oracle, OpenMP); "
                  f"the same run is this line's parity reference",
    }
    topo = sc.city.topologies
    mesh = sc.city.mesh
    valid = np.asarray(mesh.active_mask, bool) & ~np.asarray(mesh.building_mask, bool)
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    cmp = compare_runs(r.snapshot_times_s, r.depth, gpu["times"], gpu["depth"], valid, area,
                       ref_node_volume=r.final_node_volume, cand_node_volume=gpu["node_volume"],
                       ref_link_flow=r.final_link_flow, cand_link_flow=gpu["link_flow"])
    parity = {
        "reference": "C oracle (CPU restatement of the reference step), same seeded inputs, whole 60-min run",
        "cells": c, "snapshot_times_s": [round(x["candidate_time_s"], 3) for x in cmp["snapshots"]],
        "steps": {"gpu": gpu["steps"], "oracle": r.step_count},
        "depth_rmse_m": [x["valid_depth_rmse_m"] for x in cmp["snapshots"]],
        "csi_0_05m": [x["extent_agreement_csi"] for x in cmp["snapshots"]],
        "wet_cells_0_05m": {"gpu": [x["candidate_wet_triangle_count"] for x in cmp["snapshots"]],
                            "oracle": [x["reference_wet_triangle_count"] for x in cmp["snapshots"]]},
        "surface_volume_error": [x["surface_volume_error_fraction"] for x in cmp["snapshots"]],
        "max_abs_depth_error_m": [x["max_absolute_error_m"] for x in cmp["snapshots"]],
        "drainage_state": cmp["drainage_state"],
        "gates": cmp["drop_in_gates"], "passed": cmp["passed"],
    }
    return base, parity


def reference_arm(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from floodgb.config import load_config
    from floodgb.synthetic import production_workload

    sc = production_workload()
    cfg = load_config(None, sc.overrides)
    import oracle

    oracle.build()
    c = sc.cell_count
    mid = oracle.run(sc, cfg, max_steps=args.mid_run_step)  # untimed: the wet mid-run state
    per_step = None
    per = []
    n_steps = 8
    for i in range(args.warmup + args.steps):
        if per_step is not None:
            secs = max(2.0, args.cpu_seconds / max(args.steps, 1)) if i >= args.warmup else 1.0
            n_steps = int(max(4, min(2000, secs / max(per_step, 1e-6))))
        t0 = time.perf_counter()
        r = oracle.run(sc, cfg, max_steps=n_steps, start=mid)
        wall = time.perf_counter() - t0
        per_step = wall / max(r.step_count, 1)
        if i >= args.warmup:
            per.append((c * r.step_count / wall, r.step_count, wall))
    value = statistics.median(v for v, _, _ in per)
    n, w = per[-1][1], per[-1][2]
    sample = (f"{n} adaptive steps continued from step {mid.step_end} of the same 60-min run "
              f"(t = {mid.t_end:.0f} s, wet mid-run state; {w:.1f} s per sample, C oracle, OpenMP)")
    base = {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port", "sample": sample}
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world),
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


SURROGATE_WEIGHTS = ROOT / "gpu-urban-flood-cupy-jax_gb300" / "floodgb" / "surrogate" / "weights" / "mpnn_grid224.npz"


def ensemble_measure(screen_members: int = 1024):
    """Second metric, ensemble scenario-hours/s.  The ragged batched ensemble:
    64 members, 16 each of 10,082 / 49,928 / 100,352 / 250,632-triangle
    meshes, seeded storms of peak 20-120 mm/h over 1-6 h, each member run for
    its storm's duration in one persistent launch per step, launch shape from
    the autotuner; against the plain single-instance solver (two members per
    mesh size timed, extrapolated per size).  Then, with the trained
    surrogate, screening of the held-out storms on its 100,352-triangle mesh
    (rollouts + solver re-runs of flagged and audited members) against the
    plain single-instance solver."""

    from floodgb.batch import measure_ensemble

    e = measure_ensemble(per_size=16, duration_cap_h=None, sequential_per_size=2, tune_shape=True)
    out = {
        "metric": "scenario-h/s",
        "workload": f"{e['members']} members (16 each of 10,082 / 49,928 / 100,352 / 250,632 triangles), "
                    f"seeded storms of 1-6 h, {e['scenario_hours']:.1f} scenario-hours",
        "batched": e["batched_scenario_h_per_s"], "sequential_single_instance": e["single_instance_scenario_h_per_s"],
        "batched_over_single": e["batched_over_single"], "batched_cell_steps_per_s": e["batched_cell_steps_per_s"],
        "batch_shape": dict(e["shape"], source="autotuner"), "single_instance_sample": e["single_instance_sample"],
    }
    if SURROGATE_WEIGHTS.exists():
        from floodgb.surrogate.experiment import screen_saved

        r = screen_saved(SURROGATE_WEIGHTS, n_eval=screen_members, plain_sample=2, score_all=False)
        out["surrogate_screening"] = {
            "members": r["members"], "mesh_cells": r["mesh_cells"], "scenario_hours": r["scenario_hours"],
            "ensemble_networks": r["ensemble_networks"], "flag_threshold_m": r["flag_threshold_m"],
            "flagged": r["flagged"], "audited": r["audited"], "re_solved": r["re_solved"], "scored": r["scored"],
            "flagged_scores": r["surrogate_flagged"], "audit_scores": r["audit_scores"],
            "calibration": r["calibration"], "throughput_scenario_h_per_s": r["throughput_scenario_h_per_s"],
        }
    return out


def our_arm(args):
    import numpy as np
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from floodgb import native
    from floodgb.build import build_library
    from floodgb.config import load_config
    from floodgb.solver import solver_for_city
    from floodgb.synthetic import production_workload

    build_library()
    native.load()
    sc = production_workload()
    cfg = load_config(None, dict(sc.overrides, **{"solver.surface_step_mode": args.surface_mode}))
    topo = sc.city.topologies
    st = topo.surface_topology
    C, E = st.cell_count, st.edge_count
    Nn, L = topo.coupling_topology.node_count, topo.pipe_topology.link_count
    solver = solver_for_city(sc.city, sc.rainfall, cfg, device=local)
    stream = torch.cuda.Stream(local)

    def pinned(a, dtype):
        t = torch.empty(len(a), dtype=dtype, pin_memory=True)
        t.numpy()[:] = a
        return t

    h0 = pinned(np.asarray(topo.surface_state.h_m, np.float32), torch.float32)
    hu0 = pinned(np.asarray(topo.surface_state.hu_m2ps, np.float32), torch.float32)
    hv0 = pinned(np.asarray(topo.surface_state.hv_m2ps, np.float32), torch.float32)
    v0 = pinned(np.asarray(topo.pipe_state.node_volume_m3, np.float64), torch.float64)
    q0 = pinned(np.asarray(topo.pipe_state.link_flow_m3ps, np.float64), torch.float64)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def reset():
        solver.set_state(h0.numpy(), hu0.numpy(), hv0.numpy(), v0.numpy(), q0.numpy(), stream=stream)
        solver.reset_clock(stream=stream)
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()

    def timed_run():
        reset()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.run(stream=stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), solver.progress(stream=stream).step_count

    for _ in range(args.warmup):
        timed_run()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = native.load().fl_launch_count()
    wall0 = time.perf_counter()
    ms, steps = [], []
    for _ in range(args.steps):
        m, s = timed_run()
        ms.append(m)
        steps.append(s)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = native.load().fl_launch_count() - launches0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_ms, cell_steps = aggregate_ranks(float(sum(ms)), float(C) * float(sum(steps)), device=f"cuda:{local}")
    value = cell_steps / (total_ms / 1000.0)

    # end to end through the C ABI with host buffers (pinned H2D in, D2H of snapshots + final state)
    n_snap = None
    e2e_s = []
    out_h = torch.empty(C, dtype=torch.float32, pin_memory=True)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        solver.set_state(h0.numpy(), hu0.numpy(), hv0.numpy(), v0.numpy(), q0.numpy(), stream=stream)
        solver.reset_clock(stream=stream)
        solver.run(stream=stream)
        snaps = solver.snapshots(stream=stream)
        final = solver.get_state(stream=stream)
        out_h.numpy()[:] = final[0]
        e2e_s.append(time.perf_counter() - t0)
        n_snap = len(snaps[0])
    # the last run's hourly snapshots and final drainage state: the parity candidate
    gpu_run = {"times": snaps[0], "depth": snaps[1], "node_volume": final[3], "link_flow": final[4],
               "steps": solver.progress(stream=stream).step_count}
    e2e_value = float(C) * float(steps[-1]) * len(e2e_s) / sum(e2e_s)
    h2d = C * 12 + Nn * 8 + L * 8
    d2h = n_snap * (C * 12 + Nn * 4 + 8) + C * 12 + Nn * 8 + L * 8

    # roofline of the dominant kernel (k_surface) at a wet mid-run state
    reset()
    solver.run(1800.0, stream=stream)
    surf_ms = solver.time_kernel(0, reps=224, stream=stream)
    inlet_ms = solver.time_kernel(1, reps=224, stream=stream)
    net_ms = solver.time_kernel(2, reps=224, stream=stream)
    dt_ms = solver.time_kernel(3, reps=224, stream=stream)
    link_ms = solver.time_kernel(4, reps=224, stream=stream)
    donor_ms = solver.time_kernel(5, reps=224, stream=stream)
    alg_surface = C * (24 + 20 + 16 + 8) + E * 24
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_surface / (surf_ms * 1e-3) / 1e9
    alg_step = C * (24 + 20 + 16 + 8) + E * 24 + L * 68 + Nn * 48 + topo.coupling_topology.inlet_count * 16
    solver.close()

    if rank != 0:
        return
    base = parity = None
    if world == 1 and not args.no_cpu_baseline:
        base, parity = cpu_baseline_and_parity(sc, cfg, gpu_run)
    ensemble = None
    if world == 1 and not args.no_ensemble:
        ensemble = ensemble_measure()
    long_run = members = None
    if world == 1 and not args.no_long_run:
        long_run = long_single(24.0)
        members = members_measure(3.0, 8)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / len(ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / REFERENCE_PUBLISHED, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world, args.surface_mode),
        "detail": {
            "cells": C, "edges": E, "nodes": Nn, "links": L, "solver_steps_per_run": steps[-1],
            "vs_baseline_ref": "7.447e8 cell-steps/s: reference CuPy on RTX PRO 4000, real 981,880-tri city",
            "algorithmic_bytes_per_solver_step": alg_step,
            "whole_step_hbm_frac": alg_step / (total_ms / len(ms) / steps[-1] * 1e-3) / 1e9 / peak,
            "kernel_ms": {"k_surface": surf_ms, "k_nodes": inlet_ms, "k_links": link_ms, "k_donor": donor_ms,
                          "k_network": net_ms, "k_dt": dt_ms},
            "kernel_timing": "224 launches per kernel in chains of 32 per CUDA graph (as in the step loop), "
                             "wet state at t = 1800 s",
            "solver_step_us": total_ms / len(ms) / steps[-1] * 1000.0,
            "wall_s_timed_region": wall,
        },
        "roofline": {
            "bound": "hbm", "kernel": "k_surface", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": surface_traffic_per_launch(),
            "algorithmic_bytes_per_launch": alg_surface, "kernel_source_digest": surface_source_digest(),
        },
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk,
        "cpu_baseline": base,
        "parity": parity,
        "ensemble": ensemble,
        "long_run_24h": long_run,
        "members_config4": members,
    }
    print(json.dumps(line), flush=True)


def profile_surrogate():
    """One surrogate forward pass over 19 replicated 100,352-cell graphs (1.9 M
    nodes, 5.7 M directed edges) with the committed weights, inside the
    profiler range; prints the mean time of 10 unprofiled passes first."""

    import torch

    from floodgb import native
    from floodgb.build import build_library
    from floodgb.surrogate.experiment import _mesh, load
    from floodgb.surrogate.pipeline import MeshFeatures

    build_library()
    native.load()
    models, _, meta = load(SURROGATE_WEIGHTS)
    model = models[0]
    city, _ = _mesh(int(meta["grid_n"]), int(meta["seed"]))
    mf = MeshFeatures(city.topologies.surface_topology)
    g = mf.graph.replicate(19)
    x = mf.static.repeat(19, 1).to(torch.bfloat16).contiguous()
    for _ in range(3):
        model.forward(g, x, train=False)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(10):
        model.forward(g, x, train=False)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t) / 10 * 1000.0
    torch.cuda.profiler.start()
    model.forward(g, x, train=False)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile": "surrogate", "nodes": g.C, "edges": g.E, "forward_ms": ms}))


def profile_arm(args):
    """Small, bounded workloads for ncu (use with --profile-from-start off)."""

    import torch

    if args.profile == "surrogate":
        profile_surrogate()
        return

    from floodgb import native
    from floodgb.build import build_library
    from floodgb.config import load_config
    from floodgb.exceptions import SimulationError
    from floodgb.solver import solver_for_city
    from floodgb.synthetic import production_workload

    build_library()
    native.load()
    sc = production_workload()
    cfg = load_config(None, dict(sc.overrides, **{"solver.surface_step_mode": args.surface_mode}))
    solver = solver_for_city(sc.city, sc.rainfall, cfg)
    solver.run(args.profile_start_s)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    if args.profile == "loop":
        try:
            solver.run(max_steps=64)
        except SimulationError:
            pass  # the step cap ends the slice
    else:
        for k in range(6):
            solver.time_kernel(k, reps=1)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    p = solver.progress()
    print(json.dumps({"profile": args.profile, "t_s": p.t_s, "steps": p.step_count}))
    solver.close()


def long_single(hours: float = 24.0) -> dict:
    """The whole 160.09 mm / 24 h front-loaded event on the production-shaped
    coupled city, one instance, the float64 ledger closed after every
    simulated hour (its residual against the inflow)."""

    import numpy as np
    import torch

    from floodgb.config import load_config
    from floodgb.solver import solver_for_city
    from floodgb.synthetic import production_workload

    sc = production_workload()
    dur_s = hours * 3600.0
    cfg = load_config(None, dict(sc.overrides, **{"solver.duration_min": hours * 60.0}))
    topo = sc.city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    C = topo.surface_topology.cell_count
    v0 = float(np.sum(np.asarray(topo.surface_state.h_m, np.float64) * area)) + float(
        np.sum(topo.pipe_state.node_volume_m3))
    s = solver_for_city(sc.city, sc.rainfall, cfg, duration_s=dur_s)
    worst = 0.0
    solve_s = 0.0
    for k in range(1, int(np.ceil(hours)) + 1):
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.run(min(k * 3600.0, dur_s))
        torch.cuda.synchronize()
        solve_s += time.perf_counter() - t
        led = s.ledger()
        lhs = v0 + led["rainfall_input_m3"]
        rhs = (led["surface_volume_m3"] + led["node_volume_m3"] + led["infiltration_loss_m3"]
               + led["outfall_discharge_m3"] + led["unreturned_overflow_m3"] - led["boundary_net_flux_m3"])
        worst = max(worst, abs(lhs - rhs) / max(abs(lhs), 1.0))
    p = s.progress()
    led = s.ledger()
    s.close()
    return {"hours": hours, "solver_s": solve_s, "steps": p.step_count, "cell_steps_per_s": C * p.step_count / solve_s,
            "snapshots": p.snapshot_count, "worst_hourly_ledger_residual_ratio": worst,
            "rainfall_input_m3": led["rainfall_input_m3"], "outfall_discharge_m3": led["outfall_discharge_m3"],
            "timing": "wall clock around each simulated hour's fl_run (device loop), synchronised",
            "reference_24h_cupy_s": 430.467,
            "reference_hardware": "RTX PRO 4000 Blackwell, real 981,880-tri city, 321,645 steps"}


def members_measure(hours: float = 3.0, members: int = 8) -> dict:
    """Config-4 ensemble: `members` production-sized coupled members on the
    981,880-triangle city with seeded variants of the 160 mm / 24 h event
    (intensity x U(0.7, 1.3), peak shifted by up to +-3 h), run for `hours`
    simulated hours as one member solver (the surface kernel once per member
    and each drainage kernel once for all members per step), against the
    same members run one after another by the single-instance solver."""

    import numpy as np
    import torch

    from floodgb.config import load_config
    from floodgb.rainfall import hourly_rainfall
    from floodgb.solver import members_for_city, solver_for_city
    from floodgb.synthetic import FRONT_LOADED_24H_MMHR, production_workload

    sc = production_workload()
    cfg = load_config(None, dict(sc.overrides, **{"solver.duration_min": hours * 60.0}))
    C = sc.city.topologies.surface_topology.cell_count
    rng = np.random.default_rng(24)
    rains = [hourly_rainfall(np.roll(FRONT_LOADED_24H_MMHR * rng.uniform(0.7, 1.3), int(rng.integers(-3, 4))))
             for _ in range(members)]
    seq_s, seq_steps = 0.0, []
    for r in rains:
        s = solver_for_city(sc.city, r, cfg)
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.run()
        torch.cuda.synchronize()
        seq_s += time.perf_counter() - t
        seq_steps.append(s.progress().step_count)
        s.close()
    ens = members_for_city(sc.city, rains, cfg)
    try:
        torch.cuda.synchronize()
        t = time.perf_counter()
        ens.run()
        torch.cuda.synchronize()
        batched_s = time.perf_counter() - t
        steps = [ens.select(m).progress().step_count for m in range(members)]
    finally:
        ens.close()
    return {"members": members, "hours_each": hours, "cells": C, "steps": steps,
            "steps_match_single_runs": steps == seq_steps,
            "batched_s": batched_s, "batched_scenario_h_per_s": members * hours / batched_s,
            "batched_cell_steps_per_s": C * sum(steps) / batched_s,
            "single_instance_s": seq_s, "single_instance_scenario_h_per_s": members * hours / seq_s,
            "batched_over_single": seq_s / batched_s,
            "workload": "production-shaped coupled city, seeded variants of the 160 mm / 24 h front-loaded event, "
                        f"hours 0-{hours:g}"}


def long_arm(args):
    """The 24 h single instance (long_single), then `long_members` members
    with seeded variants of the event (intensity x U(0.7, 1.3), peak shifted
    by up to +-3 h) run concurrently, one host thread and CUDA stream each
    (replicas on one GPU)."""

    import threading

    import numpy as np
    import torch

    from floodgb import native
    from floodgb.build import build_library
    from floodgb.config import load_config
    from floodgb.rainfall import hourly_rainfall
    from floodgb.solver import solver_for_city
    from floodgb.synthetic import FRONT_LOADED_24H_MMHR, production_workload

    build_library()
    native.load()
    single = long_single(args.long_hours)
    sc = production_workload()
    dur_s = args.long_hours * 3600.0
    cfg = load_config(None, dict(sc.overrides, **{"solver.duration_min": args.long_hours * 60.0}))
    C = sc.city.topologies.surface_topology.cell_count
    solve_s = single["solver_s"]
    rng = np.random.default_rng(24)
    solvers, streams = [], []
    for m in range(args.long_members):
        hourly = np.roll(FRONT_LOADED_24H_MMHR * rng.uniform(0.7, 1.3), int(rng.integers(-3, 4)))
        s = solver_for_city(sc.city, hourly_rainfall(hourly), cfg, duration_s=dur_s)
        solvers.append(s)
        streams.append(torch.cuda.Stream())
    errors = []

    def go(k):
        try:
            solvers[k].run(stream=streams[k])
        except Exception as e:  # reported below
            errors.append(repr(e))

    torch.cuda.synchronize()
    t = time.perf_counter()
    threads = [threading.Thread(target=go, args=(k,)) for k in range(len(solvers))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    torch.cuda.synchronize()
    ens_s = time.perf_counter() - t
    steps = [sv.progress().step_count for sv in solvers]
    for sv in solvers:
        sv.close()
    ensemble = {"members": len(solvers), "wall_s": ens_s, "scenario_hours": len(solvers) * args.long_hours,
                "scenario_h_per_s": len(solvers) * args.long_hours / ens_s, "steps": steps,
                "cell_steps_per_s": C * sum(steps) / ens_s, "errors": errors,
                "single_instance_scenario_h_per_s": args.long_hours / solve_s}
    batched = members_measure(args.long_hours, args.long_members)
    print(json.dumps({"long_run": single, "concurrent_members": ensemble, "batched_members": batched}))


def main():
    args = parse_args()
    if args.long:
        long_arm(args)
        return
    if args.profile:
        profile_arm(args)
        return
    if args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
