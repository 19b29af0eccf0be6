"""GPU parity: libfloodgb (through its C ABI) against the reference's golden
vectors and the C oracle.

Tolerances are the ones the build targets: single-step h/hu/hv within 1e-6 m
absolute or 1e-5 relative; multi-step runs by the run-level gates (depth
RMSE <= 1e-3 m, flood-extent CSI >= 0.995 at 0.05 m, surface-volume error <=
0.05 %).
"""

import numpy as np
import pytest

import fixtures as F
import oracle as O
from floodgb import backend as B
from floodgb import native
from floodgb.config import load_config
from floodgb.exceptions import SimulationError
from floodgb.solver import solver_for_city
from floodgb.synthetic import coupled_test_city, make_grid_city
from floodgb.topology import TriangularPipeNetworkState, TriangularSurfaceForcing, TriangularSurfaceState

pytestmark = pytest.mark.gpu

SURFACE = F.load("surface_cases.npz")
PIPE = F.load("pipe_cases.npz")
RUNS = F.load("run_cases.npz")


def within_step_tolerance(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    bad = np.abs(a - b) > np.maximum(1e-6, 1e-5 * np.abs(b))
    assert not bad.any(), f"{bad.sum()} values outside 1e-6 abs / 1e-5 rel; worst {np.abs(a - b).max():.3e}"


def gates(depth, ref_depth, area, valid, threshold=0.05):
    d = depth.astype(np.float64)[valid]
    r = ref_depth.astype(np.float64)[valid]
    rmse = float(np.sqrt(np.mean((d - r) ** 2)))
    wet_c, wet_r = d >= threshold, r >= threshold
    union = int((wet_c | wet_r).sum())
    # nothing wet in either field yet: the extents agree
    csi = float((wet_c & wet_r).sum() / union) if union else 1.0
    vc = float(np.sum(depth.astype(np.float64) * area))
    vr = float(np.sum(ref_depth.astype(np.float64) * area))
    return rmse, csi, (vc - vr) / max(abs(vr), 1.0)


@pytest.fixture(scope="module", autouse=True)
def library():
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    yield
    B.clear_cache()


@pytest.mark.parametrize("name", [str(n) for n in SURFACE["cases"]])
def test_surface_step_matches_reference(name):
    d = SURFACE
    p = f"{name}/"
    st = F.surface_topology(d, p)
    stage = float(d[p + "stage"])
    stage = None if np.isnan(stage) else stage
    forcing = TriangularSurfaceForcing(rainfall_rate_mps=d[p + "rain"], infiltration_capacity_mps=d[p + "infil"],
                                       boundary_stage_m=stage)
    new, diag = B.step_triangular_surface(TriangularSurfaceState(d[p + "h"], d[p + "hu"], d[p + "hv"]), st, forcing,
                                          float(d[p + "dt"]))
    within_step_tolerance(new.h_m, d[p + "h_out"])
    within_step_tolerance(new.hu_m2ps, d[p + "hu_out"])
    within_step_tolerance(new.hv_m2ps, d[p + "hv_out"])
    ref = d[p + "diag"]
    got = [diag.rainfall_input_m3, diag.infiltration_loss_m3, diag.boundary_net_flux_m3, diag.boundary_inflow_m3,
           diag.boundary_outflow_m3, diag.final_surface_volume_m3]
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("name", [str(n) for n in SURFACE["cases"]])
def test_clamp_and_timestep_match_reference(name):
    d = SURFACE
    p = f"{name}/"
    st = F.surface_topology(d, p)
    out = B.clamp_velocity(TriangularSurfaceState(d[p + "h_out"], d[p + "hu_out"], d[p + "hv_out"]), 5.0,
                           topology=st)
    np.testing.assert_array_equal(out.hu_m2ps, d[p + "hu_clamped"])
    np.testing.assert_array_equal(out.hv_m2ps, d[p + "hv_clamped"])
    dt = B.stable_triangular_timestep_s(st, TriangularSurfaceState(d[p + "h"], d[p + "hu"], d[p + "hv"]), cfl=0.85)
    assert dt == float(d[p + "dt_cfl"])


@pytest.mark.parametrize("name", [str(n) for n in PIPE["cases"]])
def test_pipe_step_matches_reference(name):
    d = PIPE
    p = f"{name}/"
    st = F.surface_topology(d, "mesh/")
    cp, pp = F.coupling_pipe(d, p)
    h, state, diag = B.step_triangular_dynamic_pipe_network(
        d[p + "h"], st, cp, pp, TriangularPipeNetworkState(d[p + "V"], d[p + "Q"]), float(d[p + "dt"]),
        inlet_capture_rule=str(d[p + "rule"]))
    within_step_tolerance(h, d[p + "h_out"])
    # node volumes and flows are float32 / float-float here (float64 in the reference)
    np.testing.assert_allclose(state.node_volume_m3, d[p + "V_out"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(state.link_flow_m3ps, d[p + "Q_out"], rtol=1e-4, atol=1e-5)
    ref = d[p + "diag"]
    got = [diag.surface_capture_m3, diag.surface_surcharge_m3, diag.link_abs_flow_m3, diag.outfall_discharge_m3,
           diag.overflow_surcharge_m3, diag.unreturned_overflow_m3, diag.final_node_volume_m3]
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-4)


def run_device(sc, cfg=None, max_snapshots=None):
    cfg = cfg or load_config(None, sc.overrides)
    s = solver_for_city(sc.city, sc.rainfall, cfg, max_snapshots=max_snapshots)
    try:
        s.run()
        prog = s.progress()
        snaps = s.snapshots()
        state = s.get_state()
        led = s.ledger()
    finally:
        s.close()
    return prog, snaps, state, led


@pytest.mark.parametrize("prefix", ["coupled/", "grid/"])
def test_run_matches_reference_loop(prefix):
    d = RUNS
    sc = F.scenario(d, prefix)
    cfg = load_config(None, sc.overrides)
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.error == 0
    assert abs(prog.step_count - int(d[prefix + "step_count"])) <= 2
    ref_h = d[prefix + "snap_h"]
    assert h.shape == ref_h.shape
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(h.shape[0]):
        rmse, csi, verr = gates(h[k], ref_h[k], area, valid)
        assert rmse <= 1e-4 and csi >= 0.995 and abs(verr) <= 5e-4, (k, rmse, csi, verr)
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3"]
    np.testing.assert_allclose([led[n] for n in names], d[prefix + "ledger"][:5], rtol=1e-4, atol=1e-2)


def test_small_workload_hour_gates_against_oracle():
    sc = make_grid_city(n=100, seed=0)
    cfg = load_config(None, sc.overrides)
    ref = O.run(sc, cfg)
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.error == 0 and ref.error == 0
    assert abs(prog.step_count - ref.step_count) <= max(5, ref.step_count // 500)
    assert h.shape == ref.depth.shape
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.ones(h.shape[1], bool)
    for k in range(h.shape[0]):
        rmse, csi, verr = gates(h[k], ref.depth[k], area, valid)
        assert rmse <= 1e-3 and csi >= 0.995 and abs(verr) <= 5e-4, (k, rmse, csi, verr)
    np.testing.assert_allclose(led["rainfall_input_m3"], ref.ledger["rainfall_input_m3"], rtol=1e-4)


@pytest.mark.parametrize("n", [1, 16, 17, 23])
def test_tiny_and_ragged_meshes_against_oracle(n):
    """Meshes of 2 triangles (far below one 256-cell tile), exactly two
    tiles (512), and ragged last tiles (578, 1058 cells), each over 10
    simulated minutes, against the oracle."""

    sc = make_grid_city(n=n, size_m=10.0 * n, seed=n)
    cfg = load_config(None, dict(sc.overrides, **{"solver.duration_min": 10.0, "solver.snapshot_interval_min": 5.0}))
    ref = O.run(sc, cfg)
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.error == 0 and ref.error == 0
    assert abs(prog.step_count - ref.step_count) <= max(2, ref.step_count // 500)
    assert h.shape == ref.depth.shape == (3, 2 * n * n)
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.ones(h.shape[1], bool)
    for k in range(h.shape[0]):
        rmse, csi, verr = gates(h[k], ref.depth[k], area, valid)
        assert rmse <= 1e-3 and csi >= 0.995 and abs(verr) <= 5e-4, (k, rmse, csi, verr)
    np.testing.assert_allclose(led["rainfall_input_m3"], ref.ledger["rainfall_input_m3"], rtol=1e-4)


def test_coupled_city_hour_gates_against_oracle():
    sc = coupled_test_city(scale=2, seed=3, duration_min=60.0)
    cfg = load_config(None, sc.overrides)
    ref = O.run(sc, cfg)
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.error == 0 and ref.error == 0
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(min(h.shape[0], ref.depth.shape[0])):
        rmse, csi, verr = gates(h[k], ref.depth[k], area, valid)
        assert rmse <= 1e-3 and csi >= 0.995 and abs(verr) <= 5e-4, (k, rmse, csi, verr)


def test_surcharge_table_run_gates_against_oracle():
    """Weighted surcharge-return table (reference triangular_backend.py:1424-1474)
    through the device loop against the oracle's float64 restatement."""

    from floodgb.synthetic import add_surcharge_table

    sc = coupled_test_city(scale=1, seed=5, duration_min=20.0)
    add_surcharge_table(sc, seed=2)
    cfg = load_config(None, sc.overrides)
    ref = O.run(sc, cfg)
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.error == 0 and ref.error == 0
    assert ref.ledger["overflow_surcharge_m3"] > 100.0
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(min(h.shape[0], ref.depth.shape[0])):
        rmse, csi, verr = gates(h[k], ref.depth[k], area, valid)
        assert rmse <= 1e-3 and csi >= 0.995 and abs(verr) <= 5e-4, (k, rmse, csi, verr)
    for n in ("overflow_surcharge_m3", "outfall_discharge_m3", "unreturned_overflow_m3"):
        np.testing.assert_allclose(led[n], ref.ledger[n], rtol=2e-3, atol=0.5)


def test_mass_ledger_closes():
    sc = coupled_test_city(scale=1, seed=7, duration_min=20.0)
    cfg = load_config(None, sc.overrides)
    topo = sc.city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    v0 = float(np.sum(np.asarray(topo.surface_state.h_m, np.float64) * area)) + float(
        np.sum(topo.pipe_state.node_volume_m3))
    prog, snaps, (h, hu, hv, V, Q), led = run_device(sc, cfg)
    lhs = v0 + led["rainfall_input_m3"]
    rhs = (led["surface_volume_m3"] + led["node_volume_m3"] + led["infiltration_loss_m3"]
           + led["outfall_discharge_m3"] + led["unreturned_overflow_m3"] - led["boundary_net_flux_m3"])
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)


def test_closed_basin_conserves_volume_and_lake_at_rest():
    sc = make_grid_city(n=30, size_m=300.0, seed=5, boundary_mode="reflective", rain_mmhr=0.0, duration_min=5.0)
    st = sc.city.topologies.surface_topology
    area = np.asarray(st.cell_area_m2, np.float64)
    stage = float(np.max(st.bed_elevation_m)) + 0.2
    h0 = np.maximum(stage - np.asarray(st.bed_elevation_m, np.float64), 0).astype(np.float32)
    topo = sc.city.topologies
    topo.surface_state = TriangularSurfaceState(h0, np.zeros_like(h0), np.zeros_like(h0))
    prog, snaps, (h, hu, hv, V, Q), led = run_device(sc)
    assert prog.error == 0
    v0, v1 = float(np.sum(h0 * area)), float(np.sum(h.astype(np.float64) * area))
    assert abs(v1 - v0) <= 1e-6 * v0
    # hydrostatic reconstruction keeps a lake at rest over an uneven bed
    assert np.abs(hu).max() < 1e-4 and np.abs(hv).max() < 1e-4
    assert np.abs(h - h0).max() < 1e-4


def test_runs_are_bitwise_reproducible():
    sc = coupled_test_city(scale=1, seed=11, duration_min=10.0)
    a = run_device(sc)
    b = run_device(sc)
    for x, y in zip(a[1][1:], b[1][1:]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(a[2], b[2]):
        np.testing.assert_array_equal(x, y)


def test_nonfinite_depth_raises_simulation_error():
    # Fault injected on the host: an isolated storage node holding an infinite
    # volume overflows into its surface cell, whose depth becomes +inf at the
    # end of step 1; the finite check (every step here) must stop the run.
    # (A non-finite initial depth cannot be used: like the reference's CUDA
    # kernels, the depth update clips max(h, 0), which maps NaN to 0.)
    from floodgb.topology import TriangularNodeCouplingTopology, TriangularPipeNetworkTopology

    sc = make_grid_city(n=20, size_m=200.0, seed=1, duration_min=30.0)
    topo = sc.city.topologies
    zi, zf = np.zeros(0, np.int32), np.zeros(0, np.float32)
    topo.coupling_topology = TriangularNodeCouplingTopology(
        inlet_cell_index=zi, inlet_node_index=zi, node_surface_cell_index=np.array([57], np.int32),
        node_invert_elevation_m=np.array([-2.0], np.float32), node_storage_area_m2=np.array([1.0], np.float32),
        node_max_depth_m=np.array([1.0], np.float32))
    topo.pipe_topology = TriangularPipeNetworkTopology(
        link_from_node_index=zi, link_to_node_index=zi, link_length_m=zf, link_area_m2=zf,
        link_hydraulic_radius_m=zf, link_manning_n=zf)
    topo.pipe_state = TriangularPipeNetworkState(np.array([np.inf]), np.zeros(0))
    cfg = load_config(None, {**sc.overrides, "solver.finite_check_interval_steps": 1})
    s = solver_for_city(sc.city, sc.rainfall, cfg)
    try:
        with pytest.raises(SimulationError, match="Non-finite depth"):
            s.run()
        assert s.progress().step_count <= 3
    finally:
        s.close()


def test_step_cap_and_resume():
    sc = make_grid_city(n=20, size_m=200.0, seed=2, duration_min=5.0)
    cfg = load_config(None, sc.overrides)
    s = solver_for_city(sc.city, sc.rainfall, cfg)
    try:
        with pytest.raises(SimulationError, match="step cap"):
            s.run(max_steps=50)
        assert s.progress().step_count == 50
        s.run(120.0)
        assert s.progress().t_s >= 120.0
        s.run()
        p = s.progress()
        assert p.t_s == pytest.approx(300.0) and p.error == 0
        paused = s.snapshots()[1]
    finally:
        s.close()
    prog, (t, h, hu, hv, v), state, led = run_device(sc, cfg)
    assert prog.step_count == p.step_count
    np.testing.assert_array_equal(paused, h)


def test_bounded_device_wait_gives_up_and_reports():
    """A wait on an mbarrier that nothing arrives on ends after its limit with
    FL_E_TIMEOUT, and the device keeps working afterwards."""

    import ctypes as C

    st, el = C.c_int32(0), C.c_double(0.0)
    native.check(native.load().fl_wait_selftest(0.2, C.byref(st), C.byref(el)), "fl_wait_selftest")
    assert st.value == native.FL_E_TIMEOUT
    assert 0.19 <= el.value < 2.0
    native.check(native.load().fl_wait_selftest(0.05, C.byref(st), C.byref(el)), "fl_wait_selftest")
    assert st.value == native.FL_E_TIMEOUT


def test_engine_outputs_have_reference_names_and_dtypes(tmp_path):
    """run_simulation's result through floodgb.outputs: the NPZ array names,
    dtypes and ranks and the report keys of the reference writer
    (postprocessing/outputs.py:25-99, fixture written by it)."""

    import json

    from floodgb import outputs as fout
    from floodgb.engine import run_simulation

    ref = F.load("output_cases.npz")
    sc = coupled_test_city(scale=1, seed=21, duration_min=3.0)
    cfg = load_config(None, dict(sc.overrides, **{"solver.snapshot_interval_min": 1.0}))
    res = run_simulation(sc.city, sc.rainfall, cfg)
    path = fout.save_run_npz(res, tmp_path)
    with np.load(path, allow_pickle=False) as z:
        assert sorted(z.files) == [str(n) for n in ref["npz_names"]]
        for name in z.files:
            want = ref[f"npz/{name}"]
            assert z[name].dtype == want.dtype and z[name].ndim == want.ndim, (name, z[name].dtype, want.dtype)
        assert z["depth_snapshots_m"].shape == (len(z["snapshot_times_s"]), sc.cell_count)
    rep = fout.build_report(res, {"npz": path.name})
    assert set(rep) == set(json.loads(str(ref["report_json"])))
    assert abs(rep["mass_residual_ratio"]) <= 1e-5
