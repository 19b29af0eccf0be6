"""Autotuner for the batched surface kernel's launch shape.

The batch kernel's tile size (cells per CTA: 128 or 256) and the number of
persistent CTAs per SM trade shared-memory staging per CTA, halo overhead
(smaller tiles re-read more neighbour states) and latency hiding (more CTAs
per SM).  ``tune`` times a bounded number of lockstep steps of the actual
batch for each candidate shape and returns the fastest; results are cached
per (device, scenario sizes) in a JSON file so a workload is tuned once.
"""

from __future__ import annotations

import hashlib
import json
import os
import time
from pathlib import Path

from . import native as N

CANDIDATES = [
    {"tile_cells": 256, "ctas_per_sm": 2},
    {"tile_cells": 256, "ctas_per_sm": 3},
    {"tile_cells": 256, "ctas_per_sm": 4},
    {"tile_cells": 128, "ctas_per_sm": 4},
    {"tile_cells": 128, "ctas_per_sm": 6},
    {"tile_cells": 128, "ctas_per_sm": 8},
]


def cache_path() -> Path:
    base = os.environ.get("FLOODGB_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "floodgb")
    return Path(base) / "autotune.json"


def workload_key(device_name: str, cell_counts: list[int], kinds: list[int]) -> str:
    sig = f"{device_name}|{sorted(cell_counts)}|{sorted(kinds)}"
    return hashlib.sha1(sig.encode()).hexdigest()[:16]


def load_cache() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def store_cache(key: str, entry: dict) -> None:
    p = cache_path()
    data = load_cache()
    data[key] = entry
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass  # a read-only home still tunes, it just does not remember


def pick(timings: dict) -> dict:
    """The fastest candidate of {shape-json: seconds}."""

    best = min(timings.items(), key=lambda kv: kv[1])[0]
    return json.loads(best)


def tune(scenarios, steps: int = 64, candidates=None, device: int = 0, use_cache: bool = True,
         chunk_steps: int = 32) -> dict:
    """Fastest launch shape {tile_cells, ctas_per_sm, chunk_steps} for a batch."""

    import torch

    from .batch import BatchSolver

    name = torch.cuda.get_device_name(device)
    cells = [sc.city.topologies.surface_topology.cell_count for sc in scenarios]
    kinds = [1 if sc.cfg.physics.infiltration_mode == "production_horton" else 0 for sc in scenarios]
    key = workload_key(name, cells, kinds)
    if use_cache:
        hit = load_cache().get(key)
        if hit:
            return dict(hit["shape"])
    timings = {}
    for cand in candidates or CANDIDATES:
        shape = dict(cand, chunk_steps=chunk_steps)
        with BatchSolver(scenarios, shape=shape, device=device) as b:
            b.run(max_steps=steps)  # warm-up: graph capture, first touch
            t0 = time.perf_counter()
            b.run(max_steps=steps)
            timings[json.dumps(shape, sort_keys=True)] = time.perf_counter() - t0
    best = pick(timings)
    store_cache(key, {"shape": best, "timings_s": timings, "steps": steps})
    return best
