"""Surrogate screening of a rainfall ensemble with the plain solver as judge.

One mesh (a jittered grid with a seeded random-field bed), seeded storms
(peak 20-120 mm/h, duration 1-6 h): the batched solver generates training
trajectories, an ensemble of networks is trained on the GPU (a few training
storms held out), the flag threshold on the networks' disagreement is
calibrated on the held-out storms, then a held-out ensemble is screened --
ensemble rollouts for every member, flags where the networks disagree, a
random audit -- and the solver re-runs the flagged and audited members and
scores the surrogate on them (or on every member).  The re-runs follow the
rollouts as one set of batches, or the audit (drawn before the rollouts) runs
on a second stream beside them.  Throughput is
scenario-hours per second of the whole screening (surrogate + re-runs)
against the plain single-instance solver (one FloodSolver run per member,
sequentially) and the batched solver.

    python -m floodgb.surrogate.experiment [--grid-n 224] [--train 512] [--eval 1024]
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np


def _storms(n: int, seed: int, duration_cap_h=None):
    from ..synthetic import storm_hyetograph

    r = np.random.default_rng(seed)
    out = [storm_hyetograph(r) for _ in range(n)]
    dur = [min(e.duration_min * 60.0, duration_cap_h * 3600.0) if duration_cap_h else e.duration_min * 60.0
           for e in out]
    return out, dur


def _mesh(grid_n: int, seed: int):
    from ..config import load_config
    from ..synthetic import make_grid_city

    sc = make_grid_city(n=grid_n, size_m=1000.0, seed=seed)
    cfg = load_config(None, dict(sc.overrides, **{"solver.duration_min": None}))
    return sc.city, cfg


def screen(models, mf, city, cfg, threshold: float, storms, durations, *, audit: float = 0.05, seed: int = 0,
           plain_sample: int = 8, batch_size: int = 64, baselines: bool = False, n_layers: int = 8,
           score_all: bool = True, rerun: str = "after", rerun_batch: int = 128,
           extent_threshold: float | None = None) -> dict:
    """Screen an ensemble: a random audit, ensemble rollouts of every member,
    flags where the networks disagree, solver re-runs of the flagged and
    audited members; the solver judges the re-run members (or, with
    score_all, every member); the plain single-instance solver is timed on a
    sample.

    rerun="after": the rollouts first, then the flagged and audited members
    in batches of up to `rerun_batch`.  rerun="overlap": the audit re-runs on
    a second stream while the rollouts run, then the flagged members that
    were not audited.  `extent_threshold` (calibrate_extent) adds each
    member's CSI of the surrogate's envelope at that depth."""

    if rerun not in ("after", "overlap"):
        raise ValueError(f"rerun must be 'after' or 'overlap', not {rerun!r}")

    import threading

    import torch

    from ..solver import solver_for_city
    from . import ops
    from .model import MPNN
    from .pipeline import ensemble_rollouts, flags, rollout_batch, score, solve_members

    rng = np.random.default_rng(seed)
    n = len(storms)
    copies = max(1, min(64, 2_000_000 // mf.C))
    audited = np.zeros(n, bool)
    audited[rng.choice(n, size=min(int(np.ceil(audit * n)), n), replace=False)] = True
    a_idx = np.flatnonzero(audited)
    # warm-up, not timed (as the solvers are warmed up): the first pass of a
    # batch shape loads the kernels and grows the allocator's pool
    ensemble_rollouts(models, mf, storms[:copies], [min(float(d), 3600.0) for d in durations[:copies]], copies=copies)
    torch.cuda.synchronize()
    audit_out = {}

    def run_audit():
        side = torch.cuda.Stream()
        audit_out["r"] = solve_members(city, cfg, [storms[i] for i in a_idx], [durations[i] for i in a_idx],
                                       batch_size, stream=side, device="cpu")

    t = time.perf_counter()
    worker = threading.Thread(target=run_audit) if rerun == "overlap" else None
    if worker is not None:
        worker.start()
    main = torch.cuda.Stream()
    with torch.cuda.stream(main):
        preds, spread = ensemble_rollouts(models, mf, storms, durations, copies=copies)
    main.synchronize()
    surr_s = time.perf_counter() - t
    audit_trajs, audit_solver_s = [], None
    if worker is not None:
        worker.join()
        audit_trajs, audit_solver_s, _ = audit_out["r"]
    overlap_s = time.perf_counter() - t
    ops.status()
    hours = float(sum(durations)) / 3600.0
    flagged = flags(spread, threshold)
    # the members the solver re-runs now: with the audit already re-run, the flagged rest
    # (re-run trajectories stay in host memory: they are only scored)
    f_idx = np.flatnonzero(flagged & ~audited) if worker is not None else np.flatnonzero(flagged | audited)
    t = time.perf_counter()
    flag_trajs, flag_solver_s = [], 0.0
    if f_idx.size:
        flag_trajs, flag_solver_s, _ = solve_members(city, cfg, [storms[i] for i in f_idx],
                                                     [durations[i] for i in f_idx],
                                                     batch_size if worker is not None else rerun_batch, device="cpu")
    torch.cuda.synchronize()
    flag_s = time.perf_counter() - t
    re_solved = {int(i): tr for i, tr in zip(a_idx, audit_trajs)}
    re_solved.update({int(i): tr for i, tr in zip(f_idx, flag_trajs)})
    rerun_h = float(sum(durations[i] for i in re_solved)) / 3600.0
    if score_all:
        truth, batched_s, _ = solve_members(city, cfg, storms, durations, batch_size, device="cpu")
        scores = [score(mf, p, tr, extent_threshold=extent_threshold) for p, tr in zip(preds, truth)]
        scored = np.ones(n, bool)
    else:
        truth, batched_s = None, None
        scores = [None] * n
        for i, tr in re_solved.items():
            scores[i] = score(mf, preds[i], tr, extent_threshold=extent_threshold)
        scored = flagged | audited
    del re_solved, audit_trajs, flag_trajs

    def agg(mask):
        mask = mask & scored
        if not mask.any():
            return None
        sel = [scores[i] for i in np.flatnonzero(mask)]
        return {k: float(np.mean([s[k] for s in sel])) for k in sel[0]} | {
            "max_rmse_hmax_m": float(np.max([s["rmse_hmax_m"] for s in sel])), "members": int(mask.sum())}

    res = {"members": n, "scenario_hours": hours, "ensemble_networks": len(models),
           "flag_threshold_m": float(threshold), "flagged": int(flagged.sum()), "audited": int(audited.sum()),
           "re_solved": int(flagged.sum() + audited.sum() - (flagged & audited).sum()),
           "scored": "all members" if score_all else "flagged and audited members (solver re-runs)",
           "surrogate_accepted": agg(~flagged), "surrogate_flagged": agg(flagged), "audit_scores": agg(audited),
           "spread_m": {"mean": float(np.mean(spread)), "max": float(np.max(spread))}}
    if baselines and truth is not None:
        # what the trained networks gain: an untrained network and "the depth does not change"
        p0 = rollout_batch(MPNN(n_layers=n_layers, seed=seed + 99), mf, storms, durations, copies=copies)
        zero = [(p[0], np.zeros_like(p[1]), np.zeros_like(p[2])) for p in preds]
        res["untrained"] = float(np.mean([score(mf, p, tr)["rmse_hmax_m"] for p, tr in zip(p0, truth)]))
        res["no_change"] = float(np.mean([score(mf, p, tr)["rmse_hmax_m"] for p, tr in zip(zero, truth)]))
    plain_s, plain_h = 0.0, 0.0
    for i in range(min(plain_sample, n)):
        s = solver_for_city(city, storms[i], cfg, duration_s=durations[i])
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.run()
        torch.cuda.synchronize()
        plain_s += time.perf_counter() - t
        plain_h += durations[i] / 3600.0
        s.close()
    plain_rate = plain_h / plain_s
    screen_s = overlap_s + flag_s
    res["throughput_scenario_h_per_s"] = {
        "plain_single_instance": plain_rate,
        "batched_solver": hours / batched_s if batched_s else None,
        "surrogate_only": hours / surr_s,
        "screening": hours / screen_s,
        "screening_over_plain": (hours / screen_s) / plain_rate,
        "surrogate_s": surr_s, "audit_rerun_solver_s": audit_solver_s, "rollout_wall_s": overlap_s,
        "rerun_wall_s": flag_s, "rerun_solver_s": flag_solver_s, "rerun_scenario_h": rerun_h,
        "rerun": rerun, "rerun_batch": rerun_batch if rerun == "after" else batch_size,
    }
    return res


def run(grid_n: int = 224, n_train: int = 512, n_eval: int = 1024, seed: int = 11, epochs: int = 8,
        lr: float = 1e-3, audit: float = 0.05, n_layers: int = 8, plain_sample: int = 8, batch_size: int = 64,
        duration_cap_h: float | None = None, train_seconds: float | None = None, log=print, weights_out=None,
        baselines: bool = False, n_models: int = 2, n_val: int = 32, flag_fraction: float = 0.04,
        extent_weight: float = 3.0, pushforward: float = 0.5, train_batch: int = 1, score_all: bool = True):
    """Train an ensemble of n_models networks on n_train - n_val solver
    trajectories, calibrate the flag threshold on the other n_val, then screen
    n_eval held-out storms."""

    import torch

    from .model import MPNN
    from .pipeline import (MeshFeatures, calibrate_extent, calibrate_flags, ensemble_rollouts, score, solve_members,
                           train)

    city, cfg = _mesh(grid_n, seed)
    mf = MeshFeatures(city.topologies.surface_topology)
    tr_storms, tr_dur = _storms(n_train, seed + 1, duration_cap_h)
    ev_storms, ev_dur = _storms(n_eval, seed + 2, duration_cap_h)
    res = {"mesh_cells": mf.C, "dual_edges": mf.graph.E, "train_members": n_train - n_val, "validation_members": n_val,
           "eval_members": n_eval, "layers": n_layers, "hidden": 128, "ensemble_networks": n_models,
           "extent_weight": extent_weight, "pushforward": pushforward, "train_batch": train_batch, "lr": lr}
    t = time.perf_counter()
    trajs, solve_s, tr_hours = solve_members(city, cfg, tr_storms, tr_dur, batch_size)
    res["train_data"] = {"solver_s": solve_s, "scenario_hours": tr_hours, "wall_s": time.perf_counter() - t}
    log(f"training trajectories: {tr_hours:.1f} scenario-h in {solve_s:.1f} s")
    fit, val = trajs[:n_train - n_val], trajs[n_train - n_val:]
    models, hists, forced = [], [], []
    torch.cuda.synchronize()
    t = time.perf_counter()
    for k in range(n_models):
        m = MPNN(n_layers=n_layers, seed=seed + 1000 * k)
        forced.append([])
        hists.append(train(m, mf, fit, epochs=epochs, lr=lr, seed=seed + k, log=log, max_seconds=train_seconds,
                           extent_weight=extent_weight, pushforward=pushforward, teacher=forced[-1],
                           batch=train_batch))
        models.append(m)
    torch.cuda.synchronize()
    res["train"] = {"seconds": time.perf_counter() - t, "epochs": [len(h) for h in hists], "loss": hists,
                    "teacher_forced_loss": forced,
                    "windows": sum(len(tr.times_s) - 1 for tr in fit)}
    # flag threshold: the networks' disagreement on the held-out training storms
    preds, spread = ensemble_rollouts(models, mf, tr_storms[n_train - n_val:], tr_dur[n_train - n_val:])
    errors = [score(mf, p, tr)["rmse_hmax_m"] for p, tr in zip(preds, val)]
    cal = calibrate_flags(spread, np.asarray(errors), flag_fraction)
    cal.update(calibrate_extent(mf, preds, val))
    res["calibration"] = cal
    log(f"calibration: {cal}")
    depth = lambda e: float(np.sum(e.intensity_mmhr * (e.end_min - e.start_min)) / 60.0)  # noqa: E731
    limits = {"peak_mmhr": max(float(e.intensity_mmhr.max()) for e in tr_storms),
              "depth_mm": max(depth(e) for e in tr_storms)}
    res["limits"] = limits
    del trajs, fit, val
    res.update(screen(models, mf, city, cfg, cal["threshold_m"], ev_storms, ev_dur, audit=audit, seed=seed,
                      plain_sample=plain_sample, batch_size=batch_size, baselines=baselines, n_layers=n_layers,
                      extent_threshold=cal["extent_threshold_m"], score_all=score_all))
    if weights_out:
        save(weights_out, models, cal, limits, {"grid_n": grid_n, "seed": seed, "n_layers": n_layers,
                                                "n_train": n_train, "n_val": n_val})
    log(json.dumps(res["throughput_scenario_h_per_s"]))
    return res


def save(path, models, calibration: dict, limits: dict, meta: dict):
    arrays = {}
    for j, model in enumerate(models):
        for k, d in enumerate(model.state()):
            arrays[f"m{j}_w{k}"] = d["w"]
            arrays[f"m{j}_b{k}"] = d["b"]
    np.savez_compressed(path, **arrays, calibration=json.dumps(calibration), limits=json.dumps(limits),
                        meta=json.dumps(dict(meta, networks=len(models))))


def load(path):
    """(networks, calibration, meta) from a file written by save()."""

    from .model import MPNN

    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    models = []
    for j in range(int(meta["networks"])):
        model = MPNN(n_layers=int(meta["n_layers"]), seed=0)
        n = len(model.layers())
        model.load([{"w": z[f"m{j}_w{k}"], "b": z[f"m{j}_b{k}"]} for k in range(n)])
        models.append(model)
    return models, json.loads(str(z["calibration"])), meta


def screen_saved(path, n_eval: int = 64, plain_sample: int = 2, audit: float = 0.05, duration_cap_h=None,
                 score_all: bool = True, rerun: str = "after", rerun_batch: int = 128) -> dict:
    """Screen the first n_eval held-out storms of the saved ensemble's mesh and seed."""

    from .pipeline import MeshFeatures

    models, cal, meta = load(path)
    city, cfg = _mesh(int(meta["grid_n"]), int(meta["seed"]))
    mf = MeshFeatures(city.topologies.surface_topology)
    storms, dur = _storms(n_eval, int(meta["seed"]) + 2, duration_cap_h)
    res = screen(models, mf, city, cfg, float(cal["threshold_m"]), storms, dur, audit=audit, seed=int(meta["seed"]),
                 plain_sample=plain_sample, score_all=score_all, rerun=rerun, rerun_batch=rerun_batch,
                 extent_threshold=cal.get("extent_threshold_m"))
    res["mesh_cells"] = mf.C
    res["calibration"] = cal
    return res


def recalibrate(path, batch_size: int = 64) -> dict:
    """Recompute the extent threshold of a saved ensemble on its held-out
    training storms (the last n_val of the n_train seeded training storms)
    and write it into the file's calibration; returns the calibration."""

    from .pipeline import MeshFeatures, calibrate_extent, ensemble_rollouts, solve_members

    models, cal, meta = load(path)
    n_train = int(meta.get("n_train", 512))
    n_val = int(meta.get("n_val", cal["validation_members"]))
    city, cfg = _mesh(int(meta["grid_n"]), int(meta["seed"]))
    mf = MeshFeatures(city.topologies.surface_topology)
    storms, dur = _storms(n_train, int(meta["seed"]) + 1)
    storms, dur = storms[n_train - n_val:], dur[n_train - n_val:]
    val, _, _ = solve_members(city, cfg, storms, dur, batch_size)
    preds, _ = ensemble_rollouts(models, mf, storms, dur)
    cal.update(calibrate_extent(mf, preds, val))
    with np.load(path) as z:
        limits = json.loads(str(z["limits"]))
    save(path, models, cal, limits, dict(meta, n_train=n_train, n_val=n_val))
    return cal


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--grid-n", type=int, default=224)
    p.add_argument("--train", type=int, default=512)
    p.add_argument("--eval", type=int, default=1024)
    p.add_argument("--epochs", type=int, default=8)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--train-batch", type=int, default=1, help="windows per optimizer step")
    p.add_argument("--layers", type=int, default=8)
    p.add_argument("--seed", type=int, default=11)
    p.add_argument("--duration-cap-h", type=float, default=None)
    p.add_argument("--train-seconds", type=float, default=None)
    p.add_argument("--out", default=None)
    p.add_argument("--weights", default=None)
    p.add_argument("--networks", type=int, default=2)
    p.add_argument("--flag-fraction", type=float, default=0.04)
    p.add_argument("--screen-only", default=None, help="screen with saved weights (no training)")
    p.add_argument("--rerun", choices=("after", "overlap"), default="after")
    p.add_argument("--rerun-batch", type=int, default=128)
    p.add_argument("--score-all", action="store_true", help="with --screen-only: solve and score every member")
    p.add_argument("--rerun-scores-only", action="store_true",
                   help="training run: score only the re-solved (flagged and audited) members")
    p.add_argument("--plain-sample", type=int, default=8)
    p.add_argument("--recalibrate", default=None, help="recompute a saved ensemble's extent threshold in place")
    a = p.parse_args()
    if a.recalibrate:
        print(json.dumps(recalibrate(a.recalibrate), indent=1))
        return
    if a.screen_only:
        res = screen_saved(a.screen_only, n_eval=a.eval, plain_sample=8, duration_cap_h=a.duration_cap_h,
                           score_all=a.score_all, rerun=a.rerun, rerun_batch=a.rerun_batch)
        text = json.dumps(res, indent=1)
        if a.out:
            with open(a.out, "w") as f:
                f.write(text)
        print(text)
        return
    res = run(a.grid_n, a.train, a.eval, a.seed, a.epochs, lr=a.lr, n_layers=a.layers,
              duration_cap_h=a.duration_cap_h, train_seconds=a.train_seconds, weights_out=a.weights,
              n_models=a.networks, flag_fraction=a.flag_fraction, train_batch=a.train_batch,
              score_all=not a.rerun_scores_only, plain_sample=a.plain_sample)
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
