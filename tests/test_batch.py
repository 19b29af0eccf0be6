"""Batched ensemble (several scenarios per launch) and its autotuner.

GPU tests: every batched scenario must reproduce the single-instance solver
bit-for-bit (same steps, dts, snapshot times and states), for both tile
sizes; snapshot maxima bound the snapshot depths; the autotuner returns one
of its candidates.  CPU tests: autotuner selection and cache, the ensemble
generator, and creation without a device failing loudly.
"""

import json

import numpy as np
import pytest

from floodgb import autotune, native
from floodgb.batch import BatchSolver, Member
from floodgb.config import load_config
from floodgb.exceptions import BackendUnavailableError
from floodgb.rainfall import rainfall_event
from floodgb.solver import solver_for_city
from floodgb.synthetic import ensemble_workload, make_grid_city, storm_hyetograph


def small_members():
    out = []
    specs = [(14, 11, [0.0, 5.0, 15.0], [5.0, 15.0, 25.0], [40.0, 110.0, 20.0], 25.0),
             (22, 12, [0.0, 10.0], [10.0, 20.0], [80.0, 30.0], 20.0),
             (9, 13, [0.0], [30.0], [60.0], 30.0)]
    for n, seed, s, e, i, dur in specs:
        rain = rainfall_event(s, e, i)
        sc = make_grid_city(n=n, size_m=200.0, seed=seed, hyetograph=rain, duration_min=dur)
        cfg = load_config(None, dict(sc.overrides, **{"solver.snapshot_interval_min": 10.0}))
        out.append((sc, Member(sc.city, sc.rainfall, cfg, dur * 60.0)))
    return out


# ------------------------------------------------------------------ CPU
def test_autotune_pick_and_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("FLOODGB_CACHE", str(tmp_path))
    timings = {json.dumps({"tile_cells": 256, "ctas_per_sm": 3}): 2.0,
               json.dumps({"tile_cells": 128, "ctas_per_sm": 6}): 1.5}
    assert autotune.pick(timings) == {"tile_cells": 128, "ctas_per_sm": 6}
    key = autotune.workload_key("GB300", [300, 100], [0, 0])
    assert key == autotune.workload_key("GB300", [100, 300], [0, 0])
    assert key != autotune.workload_key("GB300", [100, 301], [0, 0])
    autotune.store_cache(key, {"shape": {"tile_cells": 128, "ctas_per_sm": 6}})
    assert autotune.load_cache()[key]["shape"]["tile_cells"] == 128


def test_storm_hyetograph_ranges():
    rng = np.random.default_rng(5)
    for _ in range(50):
        ev = storm_hyetograph(rng)
        assert 60.0 <= ev.duration_min <= 360.0
        assert 0.0 <= ev.intensity_mmhr.max() <= 120.0 and ev.intensity_mmhr.max() >= 10.0


def test_ensemble_generator_sizes():
    members = ensemble_workload(seed=3, grid_n=(5, 7), per_size=2, size_m=100.0, duration_cap_h=1.0)
    assert [m.city.topologies.surface_topology.cell_count for m in members] == [50, 50, 98, 98]
    assert all(m.duration_s <= 3600.0 for m in members)


def test_batch_without_device_fails_loudly():
    if native.device_count() > 0:
        pytest.skip("a GPU is visible")
    members = [m for _, m in small_members()]
    with pytest.raises(BackendUnavailableError):
        BatchSolver(members)


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("tile", [128, 256])
def test_batch_matches_single_instance_bitwise(tile):
    pairs = small_members()
    singles = []
    for sc, m in pairs:
        s = solver_for_city(sc.city, sc.rainfall, m.cfg, duration_s=m.duration_s)
        s.run()
        singles.append((s.get_state(), s.progress(), s.snapshots()))
        s.close()
    with BatchSolver([m for _, m in pairs], shape={"tile_cells": tile, "ctas_per_sm": 0}) as b:
        assert b.info()["tile_cells"] == tile
        b.run()
        for k, (state, prog, snaps) in enumerate(singles):
            p = b.progress(k)
            assert p.error == 0
            assert p.step_count == prog.step_count and p.t_s == prog.t_s and p.last_dt_s == prog.last_dt_s
            h, hu, hv = b.state(k)
            assert np.array_equal(h, state[0]) and np.array_equal(hu, state[1]) and np.array_equal(hv, state[2])
            t, sh, smax, shu, shv = b.snapshots(k, momentum=True)
            assert np.array_equal(t, snaps[0])
            assert np.array_equal(sh, snaps[1])
            assert np.array_equal(shu, snaps[2]) and np.array_equal(shv, snaps[3])
            assert np.all(smax >= sh)
            led = b.ledger(k)
            assert led["rainfall_input_m3"] > 0.0


@pytest.mark.gpu
def test_batch_ledger_closes():
    pairs = small_members()
    with BatchSolver([m for _, m in pairs]) as b:
        b.run()
        for k in range(b.n):
            led = b.ledger(k)
            resid = led["rainfall_input_m3"] - led["infiltration_loss_m3"] + led["boundary_net_flux_m3"] - \
                led["surface_volume_m3"]
            assert abs(resid) <= 1e-5 * max(led["rainfall_input_m3"], 1.0)


@pytest.mark.gpu
def test_batch_step_cap_and_restart():
    pairs = small_members()
    with BatchSolver([m for _, m in pairs]) as b:
        b.run(max_steps=10)
        assert all(b.progress(k).step_count == 10 for k in range(b.n))
        b.run()
        full = [b.state(k)[0].copy() for k in range(b.n)]
        b.run()
        assert all(np.array_equal(full[k], b.state(k)[0]) for k in range(b.n))


@pytest.mark.gpu
def test_autotune_returns_a_candidate(tmp_path, monkeypatch):
    monkeypatch.setenv("FLOODGB_CACHE", str(tmp_path))
    members = [m for _, m in small_members()]
    cands = [{"tile_cells": 256, "ctas_per_sm": 2}, {"tile_cells": 128, "ctas_per_sm": 4}]
    best = autotune.tune(members, steps=8, candidates=cands, use_cache=True)
    assert {k: best[k] for k in ("tile_cells", "ctas_per_sm")} in cands
    assert autotune.tune(members, steps=8, candidates=cands, use_cache=True) == best  # from the cache
