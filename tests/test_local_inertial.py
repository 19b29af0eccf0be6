"""Local-inertial surface mode (solver.surface_step_mode = "local_inertial").

The oracle restates the reference's fused CUDA path
(``triangular_local_inertial_cuda_kernels.py``: discharge per edge, donor
scale per cell, gather per cell) and ``_apply_sources``.  The golden
fixtures (``li_cases.npz``) come from the reference's NumPy path
(``step_triangular_surface_local_inertial``), which differs from its CUDA
path in two documented ways: boundary outflow is limited by the volume left
after the interior transfers (the CUDA path clips the depth at zero
instead, so only the boundary-outflow ledger differs), and per-cell sums run
in scatter order rather than slot order (rounding).  Single steps therefore
agree to float32 rounding, the timestep bit-for-bit, and multi-step runs to
the run tolerances below.
"""

import numpy as np
import pytest

import fixtures as F
import oracle as O

LI = F.load("li_cases.npz")
CASES = [str(n) for n in LI["cases"]]


def within(a, b, abs_tol=1e-6, rel_tol=1e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    bad = np.abs(a - b) > np.maximum(abs_tol, rel_tol * np.abs(b))
    assert not bad.any(), f"{bad.sum()} values outside {abs_tol} abs / {rel_tol} rel; worst {np.abs(a - b).max():.3e}"


@pytest.mark.parametrize("name", CASES)
def test_li_step_matches_reference(name):
    d = LI
    p = f"{name}/"
    st = F.surface_topology(d, p)
    h, hu, hv, diag = O.li_step(st, d[p + "h"], d[p + "hu"], d[p + "hv"], float(d[p + "dt"]), d[p + "rain"],
                                d[p + "infil"])
    within(h, d[p + "h_out"])
    within(hu, d[p + "hu_out"])
    within(hv, d[p + "hv_out"])
    ref = d[p + "diag"]
    np.testing.assert_allclose(diag[[0, 1, 5]], ref[[0, 1, 5]], rtol=1e-5, atol=1e-5)
    # boundary outflow: the CUDA path counts the unlimited outflow of drying cells
    assert diag[4] >= ref[4] - 1e-5 * max(1.0, ref[4])
    assert diag[3] == 0.0


@pytest.mark.parametrize("name", CASES)
def test_li_timestep_matches_reference_exactly(name):
    d = LI
    p = f"{name}/"
    st = F.surface_topology(d, p)
    assert O.li_stable_dt(st.characteristic_length_m, d[p + "h"]) == float(d[p + "dt_li"])


@pytest.mark.parametrize("prefix", ["coupled/", "grid/"])
def test_li_run_matches_reference(prefix):
    d = LI
    sc = F.scenario(d, prefix)
    assert sc.overrides["solver.surface_step_mode"] == "local_inertial"
    r = O.run(sc, max_steps=int(d[prefix + "step_count"]))
    assert r.step_count == int(d[prefix + "step_count"])
    assert r.t_end == float(d[prefix + "t_end"])
    np.testing.assert_array_equal(r.snapshot_times_s, d[prefix + "snap_t"])
    act = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(len(r.snapshot_times_s)):
        diff = (r.depth[k].astype(np.float64) - d[prefix + "snap_h"][k])[act]
        assert np.abs(diff).max() <= 2e-3, k
        assert np.sqrt(np.mean(diff ** 2)) <= 1e-4, k
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3", "unreturned_overflow_m3"]
    np.testing.assert_allclose([r.ledger[n] for n in names], d[prefix + "ledger"], rtol=1e-3, atol=0.05)


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def gpu():
    from floodgb import backend as B
    from floodgb import native
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    yield
    B.clear_cache()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_li_step_matches_oracle(gpu, name):
    from floodgb.backend import stable_local_inertial_triangular_timestep_s, step_triangular_surface_local_inertial
    from floodgb.topology import TriangularSurfaceForcing, TriangularSurfaceState

    d = LI
    p = f"{name}/"
    st = F.surface_topology(d, p)
    state = TriangularSurfaceState(d[p + "h"], d[p + "hu"], d[p + "hv"])
    forcing = TriangularSurfaceForcing(rainfall_rate_mps=d[p + "rain"], infiltration_capacity_mps=d[p + "infil"])
    new, diag = step_triangular_surface_local_inertial(state, st, forcing, float(d[p + "dt"]))
    h, hu, hv, odiag = O.li_step(st, d[p + "h"], d[p + "hu"], d[p + "hv"], float(d[p + "dt"]), d[p + "rain"],
                                 d[p + "infil"])
    within(new.h_m, h)
    within(new.hu_m2ps, hu)
    within(new.hv_m2ps, hv)
    np.testing.assert_allclose([diag.rainfall_input_m3, diag.infiltration_loss_m3, diag.boundary_outflow_m3],
                               odiag[[0, 1, 4]], rtol=1e-5, atol=1e-5)
    dt = stable_local_inertial_triangular_timestep_s(st, state, cfl=0.85)
    assert dt == float(d[p + "dt_li"])


@pytest.mark.gpu
@pytest.mark.parametrize("prefix", ["coupled/", "grid/"])
def test_gpu_li_run_matches_reference(gpu, prefix):
    from floodgb.config import load_config
    from floodgb.solver import solver_for_city

    d = LI
    sc = F.scenario(d, prefix)
    cfg = load_config(None, sc.overrides)
    s = solver_for_city(sc.city, sc.rainfall, cfg)
    try:
        s.run()
        prog = s.progress()
        t, h, hu, hv, v = s.snapshots()
        led = s.ledger()
    finally:
        s.close()
    assert prog.error == 0
    assert abs(prog.step_count - int(d[prefix + "step_count"])) <= 2
    ref = d[prefix + "snap_h"]
    assert h.shape == ref.shape
    act = np.asarray(sc.city.mesh.active_mask, bool)
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    for k in range(ref.shape[0]):
        diff = (h[k].astype(np.float64) - ref[k])[act]
        assert np.sqrt(np.mean(diff ** 2)) <= 2e-4, k
        vc, vr = float(np.sum(h[k] * area)), float(np.sum(ref[k] * area))
        assert abs(vc - vr) <= 5e-4 * max(abs(vr), 1.0), k
    np.testing.assert_allclose([led["rainfall_input_m3"], led["infiltration_loss_m3"]], d[prefix + "ledger"][:2],
                               rtol=1e-4, atol=1e-2)


@pytest.mark.gpu
def test_gpu_li_coupled_run_against_oracle_and_ledger_closes(gpu):
    from floodgb.config import load_config
    from floodgb.solver import solver_for_city
    from floodgb.synthetic import coupled_test_city

    sc = coupled_test_city(scale=1, seed=8, duration_min=15.0)
    sc.overrides["solver.surface_step_mode"] = "local_inertial"
    cfg = load_config(None, sc.overrides)
    ref = O.run(sc, cfg)
    topo = sc.city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    v0 = float(np.sum(np.asarray(topo.surface_state.h_m, np.float64) * area)) + float(
        np.sum(topo.pipe_state.node_volume_m3))
    s = solver_for_city(sc.city, sc.rainfall, cfg)
    try:
        s.run()
        prog = s.progress()
        t, h, hu, hv, v = s.snapshots()
        led = s.ledger()
    finally:
        s.close()
    assert prog.error == 0 and ref.error == 0
    assert abs(prog.step_count - ref.step_count) <= max(5, ref.step_count // 200)
    act = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(min(h.shape[0], ref.depth.shape[0])):
        diff = (h[k].astype(np.float64) - ref.depth[k])[act]
        assert np.sqrt(np.mean(diff ** 2)) <= 1e-3, k
    lhs = v0 + led["rainfall_input_m3"]
    rhs = (led["surface_volume_m3"] + led["node_volume_m3"] + led["infiltration_loss_m3"]
           + led["outfall_discharge_m3"] + led["unreturned_overflow_m3"] - led["boundary_net_flux_m3"])
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)
