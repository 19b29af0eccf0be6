"""Ensemble members on one mesh (fl_create_members): several coupled runs of
the same city with different rainfall, advanced together (the surface kernel
once per member, each drainage kernel once for all members), each equal bit
for bit to the same run made alone."""

import numpy as np
import pytest

from floodgb import native
from floodgb.config import load_config
from floodgb.exceptions import BackendUnavailableError
from floodgb.rainfall import rainfall_event
from floodgb.solver import members_for_city, solver_for_city
from floodgb.synthetic import coupled_test_city


def variants(rain, n):
    """n seeded variants of a storm: intensity x U(0.7, 1.3), start shifted by up to 10 min."""

    rng = np.random.default_rng(8)
    out = [rain]
    for _ in range(n - 1):
        shift = float(rng.integers(0, 3)) * 5.0
        out.append(rainfall_event(np.asarray(rain.start_min) + shift, np.asarray(rain.end_min) + shift,
                                  np.asarray(rain.intensity_mmhr) * rng.uniform(0.7, 1.3)))
    return out


def test_members_without_device_fail_loudly():
    if native.device_count() > 0:
        pytest.skip("a GPU is visible")
    sc = coupled_test_city(scale=1, seed=4, duration_min=5.0)
    with pytest.raises(BackendUnavailableError):
        members_for_city(sc.city, variants(sc.rainfall, 2), load_config(None, sc.overrides))


@pytest.mark.gpu
def test_members_equal_their_single_runs_bitwise():
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    sc = coupled_test_city(scale=1, seed=4, duration_min=20.0)
    # at the default 1 s cap every variant of this storm steps at the cap (1,200
    # steps each); at 5 s the CFL limit decides dt and the counts differ
    # (346, 295 and 348 steps in the oracle)
    cfg = load_config(None, dict(sc.overrides, **{"solver.snapshot_interval_min": 5.0, "solver.max_dt_s": 5.0}))
    rains = variants(sc.rainfall, 3)
    singles = []
    for r in rains:
        s = solver_for_city(sc.city, r, cfg)
        try:
            s.run()
            singles.append((s.progress(), s.get_state(), s.snapshots(), s.ledger()))
        finally:
            s.close()
    # the members' step counts differ (their rain differs), so some end before the others
    assert len({p.step_count for p, _, _, _ in singles}) > 1
    ens = members_for_city(sc.city, rains, cfg)
    try:
        assert ens.members == 3
        ens.run()
        for m, (prog, state, snaps, led) in enumerate(singles):
            ens.select(m)
            p = ens.progress()
            assert p.error == 0
            assert (p.step_count, p.t_s, p.last_dt_s, p.cfl_eval_count) == \
                (prog.step_count, prog.t_s, prog.last_dt_s, prog.cfl_eval_count), m
            for got, want in zip(ens.get_state(), state):
                assert np.array_equal(got, want), m
            for got, want in zip(ens.snapshots(), snaps):
                assert np.array_equal(got, want), m
            got = ens.ledger()
            for k, v in led.items():
                assert got[k] == v, (m, k, got[k], v)
        # single-member entry points refuse a member solver
        with pytest.raises(Exception):
            ens.step(0.5)
    finally:
        ens.close()
