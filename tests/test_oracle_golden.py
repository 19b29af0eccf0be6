"""The C oracle against golden vectors produced by the reference's own code.

The fixtures under ``tests/golden`` were generated by ``make_golden.py`` from
the reference's NumPy path (``gurugram_flood.kernels.triangular_backend`` and
friends).  These tests pin the oracle before it is used to check the GPU.
Surface depth agrees bit-for-bit; momentum can differ by an ulp where NumPy's
SIMD ``power`` and libm ``powf`` round differently; drainage differs at the
1e-7 relative level because the oracle follows the reference's CuPy kernels
(float32 orifice coefficient products, float32 surface accumulation) where
the NumPy path promotes to float64.
"""

import numpy as np
import pytest

import fixtures as F
import oracle as O


SURFACE = F.load("surface_cases.npz")
PIPE = F.load("pipe_cases.npz")
RUNS = F.load("run_cases.npz")


@pytest.mark.parametrize("name", [str(n) for n in SURFACE["cases"]])
def test_surface_step_matches_reference(name):
    d = SURFACE
    p = f"{name}/"
    st = F.surface_topology(d, p)
    stage = float(d[p + "stage"])
    stage = None if np.isnan(stage) else stage
    h, hu, hv, diag = O.surface_step(st, d[p + "h"], d[p + "hu"], d[p + "hv"], float(d[p + "dt"]),
                                     d[p + "rain"], d[p + "infil"], stage)
    np.testing.assert_array_equal(h, d[p + "h_out"])
    np.testing.assert_allclose(hu, d[p + "hu_out"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(hv, d[p + "hv_out"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(diag, d[p + "diag"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name", [str(n) for n in SURFACE["cases"]])
def test_clamp_and_dt_match_reference_exactly(name):
    d = SURFACE
    p = f"{name}/"
    hu, hv = O.clamp_velocity(d[p + "h_out"], d[p + "hu_out"], d[p + "hv_out"], 5.0)
    np.testing.assert_array_equal(hu, d[p + "hu_clamped"])
    np.testing.assert_array_equal(hv, d[p + "hv_clamped"])
    st = F.surface_topology(d, p)
    assert O.stable_dt(st.characteristic_length_m, d[p + "h"], d[p + "hu"], d[p + "hv"]) == float(d[p + "dt_cfl"])


@pytest.mark.parametrize("name", [str(n) for n in PIPE["cases"]])
def test_pipe_step_matches_reference(name):
    d = PIPE
    p = f"{name}/"
    st = F.surface_topology(d, "mesh/")
    cp, pp = F.coupling_pipe(d, p)
    h, V, Q, diag = O.pipe_step(st, cp, pp, d[p + "h"], d[p + "V"], d[p + "Q"], float(d[p + "dt"]),
                                capture_rule=str(d[p + "rule"]))
    np.testing.assert_allclose(h, d[p + "h_out"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(V, d[p + "V_out"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(Q, d[p + "Q_out"], rtol=1e-6, atol=1e-6)
    # capture, surcharge, link |transfer|, outfall, overflow, unreturned, final volume
    np.testing.assert_allclose(diag, d[p + "diag"], rtol=1e-6, atol=1e-5)


@pytest.mark.parametrize("prefix", ["coupled/", "grid/"])
def test_run_loop_matches_reference(prefix):
    d = RUNS
    sc = F.scenario(d, prefix)
    r = O.run(sc, max_steps=int(d[prefix + "step_count"]))
    assert r.step_count == int(d[prefix + "step_count"])
    assert r.t_end == float(d[prefix + "t_end"])
    np.testing.assert_array_equal(r.snapshot_times_s, d[prefix + "snap_t"])
    for k in range(len(r.snapshot_times_s)):
        diff = r.depth[k].astype(np.float64) - d[prefix + "snap_h"][k]
        assert np.abs(diff).max() <= 2e-5
        assert np.sqrt(np.mean(diff ** 2)) <= 2e-6
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3", "unreturned_overflow_m3"]
    got = np.array([r.ledger[n] for n in names])
    np.testing.assert_allclose(got, d[prefix + "ledger"], rtol=1e-6, atol=2e-3)


def test_resumed_run_continues_the_run_bitwise():
    """A run stopped by a step cap and resumed from its result (state, time,
    step count, cached CFL dt, snapshot schedule) equals the uninterrupted run:
    the bench's reference arm times samples continued from a mid-run state."""

    from floodgb.config import load_config
    from floodgb.synthetic import coupled_test_city

    sc = coupled_test_city(scale=1, seed=7, duration_min=10.0)
    cfg = load_config(None, dict(sc.overrides, **{"solver.snapshot_interval_min": 2.0}))
    full = O.run(sc, cfg)
    a = O.run(sc, cfg, max_steps=77)  # 77: not a multiple of the 32-step CFL cycle
    b = O.run(sc, cfg, start=a)
    assert (a.step_count, a.step_end) == (77, 77)
    assert b.step_end == full.step_count and b.t_end == full.t_end
    for x, y in ((b.final_h, full.final_h), (b.final_hu, full.final_hu), (b.final_hv, full.final_hv),
                 (b.final_node_volume, full.final_node_volume), (b.final_link_flow, full.final_link_flow),
                 (b.wet_time, full.wet_time)):
        np.testing.assert_array_equal(x, y)
    k = len(a.snapshot_times_s)
    np.testing.assert_array_equal(np.concatenate([a.snapshot_times_s, b.snapshot_times_s]), full.snapshot_times_s)
    np.testing.assert_array_equal(b.depth, full.depth[k:])
    for name, v in full.ledger.items():
        assert abs(a.ledger[name] + b.ledger[name] - v) <= 1e-12 * max(abs(v), 1.0), name
