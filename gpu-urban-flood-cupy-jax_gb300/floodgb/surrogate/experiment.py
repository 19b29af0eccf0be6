"""Surrogate screening of a rainfall ensemble with the plain solver as judge.

One mesh (a jittered grid with a seeded random-field bed), seeded storms
(peak 20-120 mm/h, duration 1-6 h): the batched solver generates training
trajectories, the network is trained on the GPU, then a held-out ensemble is
screened -- surrogate rollouts for every member, flags for members outside
the training range, a random audit -- and the solver re-runs the flagged and
audited members and scores the surrogate on every member.  Throughput is
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


def screen(model, mf, city, cfg, limits: dict, storms, durations, *, audit: float = 0.05, seed: int = 0,
           plain_sample: int = 8, batch_size: int = 64, baselines: bool = False, n_layers: int = 8,
           score_all: bool = True) -> dict:
    """Screen an ensemble: surrogate rollouts of every member, flags, a random
    audit; the solver re-runs flagged + audited members (timed) and judges
    every member (or, with score_all False, the re-run members only); the
    plain single-instance solver is timed on a sample."""

    import torch

    from ..solver import solver_for_city
    from . import ops
    from .model import MPNN
    from .pipeline import flags, rollout_batch, score, solve_members

    rng = np.random.default_rng(seed)
    n = len(storms)
    copies = max(1, min(64, 2_000_000 // mf.C))
    # warm-up, not timed (as the solvers are warmed up): the first pass of a
    # batch shape loads the kernels and grows the allocator's pool
    rollout_batch(model, mf, storms[:copies], [min(float(d), 3600.0) for d in durations[:copies]], copies=copies)
    torch.cuda.synchronize()
    t = time.perf_counter()
    preds = rollout_batch(model, mf, storms, durations, copies=copies)
    torch.cuda.synchronize()
    surr_s = time.perf_counter() - t
    ops.status()
    hours = float(sum(durations)) / 3600.0
    flagged = np.array([flags(mf, s, p, limits) for s, p in zip(storms, preds)])
    audited = np.zeros(n, bool)
    cand = np.flatnonzero(~flagged)
    if cand.size:
        audited[rng.choice(cand, size=min(int(np.ceil(audit * n)), cand.size), replace=False)] = True
    idx = np.flatnonzero(flagged | audited)
    rerun_s, rerun_h = 0.0, 0.0
    reruns = []
    if idx.size:
        reruns, rerun_s, rerun_h = solve_members(city, cfg, [storms[i] for i in idx], [durations[i] for i in idx],
                                                 batch_size)
    if score_all:
        truth, batched_s, _ = solve_members(city, cfg, storms, durations, batch_size)
        scores = [score(mf, p, tr) for p, tr in zip(preds, truth)]
        scored = np.ones(n, bool)
    else:
        truth, batched_s = None, None
        scores = [None] * n
        for j, i in enumerate(idx):
            scores[i] = score(mf, preds[i], reruns[j])
        scored = flagged | audited
    del reruns

    def agg(mask):
        mask = mask & scored
        if not mask.any():
            return None
        sel = [scores[i] for i in np.flatnonzero(mask)]
        return {k: float(np.mean([s[k] for s in sel])) for k in sel[0]} | {
            "max_rmse_hmax_m": float(np.max([s["rmse_hmax_m"] for s in sel])), "members": int(mask.sum())}

    res = {"members": n, "scenario_hours": hours, "flagged": int(flagged.sum()), "audited": int(audited.sum()),
           "scored": "all members" if score_all else "flagged and audited members (solver re-runs)",
           "surrogate_accepted": agg(~flagged), "surrogate_flagged": agg(flagged), "audit_scores": agg(audited)}
    if baselines and truth is not None:
        # what the trained network gains: an untrained network and "the depth does not change"
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
    screen_s = surr_s + rerun_s
    res["throughput_scenario_h_per_s"] = {
        "plain_single_instance": plain_rate,
        "batched_solver": hours / batched_s if batched_s else (rerun_h / rerun_s if rerun_s else None),
        "surrogate_only": hours / surr_s,
        "screening": hours / screen_s,
        "screening_over_plain": (hours / screen_s) / plain_rate,
        "surrogate_s": surr_s, "rerun_s": rerun_s, "rerun_scenario_h": rerun_h,
    }
    return res


def run(grid_n: int = 224, n_train: int = 512, n_eval: int = 1024, seed: int = 11, epochs: int = 8,
        lr: float = 1e-3, audit: float = 0.05, n_layers: int = 8, plain_sample: int = 8, batch_size: int = 64,
        duration_cap_h: float | None = None, train_seconds: float | None = None, log=print, weights_out=None,
        baselines: bool = False):
    """Train on n_train solver trajectories, then screen n_eval held-out storms."""

    import torch

    from .model import MPNN
    from .pipeline import MeshFeatures, solve_members, train

    city, cfg = _mesh(grid_n, seed)
    mf = MeshFeatures(city.topologies.surface_topology)
    tr_storms, tr_dur = _storms(n_train, seed + 1, duration_cap_h)
    ev_storms, ev_dur = _storms(n_eval, seed + 2, duration_cap_h)
    res = {"mesh_cells": mf.C, "dual_edges": mf.graph.E, "train_members": n_train, "eval_members": n_eval,
           "layers": n_layers, "hidden": 128}
    t = time.perf_counter()
    trajs, solve_s, tr_hours = solve_members(city, cfg, tr_storms, tr_dur, batch_size)
    res["train_data"] = {"solver_s": solve_s, "scenario_hours": tr_hours, "wall_s": time.perf_counter() - t}
    log(f"training trajectories: {tr_hours:.1f} scenario-h in {solve_s:.1f} s")
    model = MPNN(n_layers=n_layers, seed=seed)
    torch.cuda.synchronize()
    t = time.perf_counter()
    hist = train(model, mf, trajs, epochs=epochs, lr=lr, seed=seed, log=log, max_seconds=train_seconds)
    torch.cuda.synchronize()
    res["train"] = {"seconds": time.perf_counter() - t, "epochs": len(hist), "loss": hist,
                    "windows": sum(len(tr.times_s) - 1 for tr in trajs)}
    depth = lambda e: float(np.sum(e.intensity_mmhr * (e.end_min - e.start_min)) / 60.0)  # noqa: E731
    limits = {"peak_mmhr": max(float(e.intensity_mmhr.max()) for e in tr_storms),
              "depth_mm": max(depth(e) for e in tr_storms),
              "max_depth_m": 1.2 * max(float(tr.hmax.max().item()) for tr in trajs)}
    res["limits"] = limits
    del trajs
    res.update(screen(model, mf, city, cfg, limits, ev_storms, ev_dur, audit=audit, seed=seed,
                      plain_sample=plain_sample, batch_size=batch_size, baselines=baselines, n_layers=n_layers))
    if weights_out:
        save(weights_out, model, limits, {"grid_n": grid_n, "seed": seed, "n_layers": n_layers})
    log(json.dumps(res["throughput_scenario_h_per_s"]))
    return res


def save(path, model, limits: dict, meta: dict):
    st = model.state()
    np.savez_compressed(path, **{f"w{k}": d["w"] for k, d in enumerate(st)}, **{f"b{k}": d["b"] for k, d in enumerate(st)},
                        limits=json.dumps(limits), meta=json.dumps(meta))


def load(path):
    """(model, limits, meta) from a file written by save()."""

    from .model import MPNN

    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    model = MPNN(n_layers=int(meta["n_layers"]), seed=0)
    n = len(model.layers())
    model.load([{"w": z[f"w{k}"], "b": z[f"b{k}"]} for k in range(n)])
    return model, json.loads(str(z["limits"])), meta


def screen_saved(path, n_eval: int = 64, plain_sample: int = 2, audit: float = 0.05, duration_cap_h=None,
                 score_all: bool = True) -> dict:
    """Screen the first n_eval held-out storms of the saved model's mesh and seed."""

    from .pipeline import MeshFeatures

    model, limits, meta = load(path)
    city, cfg = _mesh(int(meta["grid_n"]), int(meta["seed"]))
    mf = MeshFeatures(city.topologies.surface_topology)
    storms, dur = _storms(n_eval, int(meta["seed"]) + 2, duration_cap_h)
    res = screen(model, mf, city, cfg, limits, storms, dur, audit=audit, seed=int(meta["seed"]),
                 plain_sample=plain_sample, score_all=score_all)
    res["mesh_cells"] = mf.C
    return res


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--grid-n", type=int, default=224)
    p.add_argument("--train", type=int, default=512)
    p.add_argument("--eval", type=int, default=1024)
    p.add_argument("--epochs", type=int, default=8)
    p.add_argument("--layers", type=int, default=8)
    p.add_argument("--seed", type=int, default=11)
    p.add_argument("--duration-cap-h", type=float, default=None)
    p.add_argument("--train-seconds", type=float, default=None)
    p.add_argument("--out", default=None)
    p.add_argument("--weights", default=None)
    p.add_argument("--screen-only", default=None, help="screen with saved weights (no training)")
    a = p.parse_args()
    if a.screen_only:
        res = screen_saved(a.screen_only, n_eval=a.eval, plain_sample=8, duration_cap_h=a.duration_cap_h)
        text = json.dumps(res, indent=1)
        if a.out:
            with open(a.out, "w") as f:
                f.write(text)
        print(text)
        return
    res = run(a.grid_n, a.train, a.eval, a.seed, a.epochs, n_layers=a.layers, duration_cap_h=a.duration_cap_h,
              train_seconds=a.train_seconds, weights_out=a.weights)
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
