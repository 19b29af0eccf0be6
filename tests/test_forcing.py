"""External boundary inflow and surface recharge.

The oracle is pinned against the reference's own functions
(``production_event_support.apply_external_boundary_inflow_depth``,
``june5_production_drainage.apply_june5_surface_recharge``) through the
committed ``forcing_cases.npz`` fixtures: bit-for-bit on depths and stored
volumes, and on a coupled run with both.  The GPU path (``fl_step`` phases
and the device loop, through the C ABI) is then checked against the oracle.
"""

import numpy as np
import pytest

import fixtures as F
import oracle as O

FORCING = F.load("forcing_cases.npz")


def test_inflow_hydrograph_matches_reference():
    d = FORCING
    ext = F.inflow(d, "unit/")
    for k, t in enumerate(d["unit/ext_time"]):
        np.testing.assert_array_equal(O.inflow_q(ext, float(t)), d["unit/ext_q_at"][k])


def test_inflow_depth_matches_reference_bitwise():
    d = FORCING
    ext = F.inflow(d, "unit/")
    # two receivers share a cell: the per-cell sum is formed before it meets h
    cells = np.asarray(ext.receiver_cell_index)
    assert np.unique(cells).size < cells.size
    for k, (t, dt) in enumerate(zip(d["unit/ext_time"], d["unit/ext_dt"])):
        h, added = O.external_inflow(d["unit/area"], ext, d["unit/h"], float(t), float(dt))
        np.testing.assert_array_equal(h, d["unit/ext_h_out"][k])
        assert added == pytest.approx(float(d["unit/ext_added"][k]), rel=1e-6, abs=1e-9)


def test_recharge_matches_reference_bitwise():
    d = FORCING
    topo = F.recharge(d, "unit/")
    cells = np.asarray(topo.source_cell_index)
    assert np.unique(cells).size < cells.size  # a repeated cell: the last row sets the depth
    h, store = d["unit/rch_h"], d["unit/rch_storage0"]
    for k, dt in enumerate(d["unit/rch_dt"]):
        h, store, cap, loss = O.recharge(d["unit/area"], topo, h, store, float(dt))
        np.testing.assert_array_equal(h, d["unit/rch_h_out"][k])
        np.testing.assert_array_equal(store, d["unit/rch_storage_out"][k])
        assert cap == pytest.approx(float(d["unit/rch_capture"][k]), rel=1e-6)
        assert loss == pytest.approx(float(d["unit/rch_loss"][k]), rel=1e-6)


def test_run_with_inflow_and_recharge_matches_reference():
    d = FORCING
    p = "run/"
    sc = F.forcing_scenario(d, p)
    r = O.run(sc, max_steps=int(d[p + "step_count"]))
    assert r.step_count == int(d[p + "step_count"])
    assert r.t_end == float(d[p + "t_end"])
    np.testing.assert_array_equal(r.snapshot_times_s, d[p + "snap_t"])
    for k in range(len(r.snapshot_times_s)):
        diff = r.depth[k].astype(np.float64) - d[p + "snap_h"][k]
        assert np.abs(diff).max() <= 2e-5
        assert np.sqrt(np.mean(diff ** 2)) <= 2e-6
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3", "unreturned_overflow_m3", "external_boundary_inflow_m3",
             "surface_recharge_capture_m3", "surface_recharge_loss_m3"]
    got = np.array([r.ledger[n] for n in names])
    np.testing.assert_allclose(got, d[p + "ledger"], rtol=1e-6, atol=2e-3)
    assert d[p + "ledger"][6] > 1.0 and d[p + "ledger"][7] > 1.0 and d[p + "ledger"][8] > 0.1
    np.testing.assert_allclose(r.recharge_storage, d[p + "recharge_storage"], rtol=1e-5, atol=1e-4)


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def gpu():
    from floodgb import native
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")


def _solver(sc):
    from floodgb.config import load_config
    from floodgb.solver import solver_for_city

    return solver_for_city(sc.city, sc.rainfall, load_config(None, sc.overrides))


@pytest.mark.gpu
def test_gpu_inflow_step_matches_oracle_bitwise(gpu):
    from floodgb import native as N

    d = FORCING
    sc = F.forcing_scenario(d, "run/")
    sc.city.recharge_topology = None
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float32)
    ext = sc.city.external_boundary
    s = _solver(sc)
    try:
        h_ref = np.array(sc.city.topologies.surface_state.h_m, np.float32)
        t, total = 0.0, 0.0
        # steps before, inside and past the hydrograph table, landing on table times too
        for dt in (0.37, 1.0, 28.63, 30.0, 0.85, 45.0, 120.0, 60.0):
            s.step(dt, phases=N.FL_PHASE_INFLOW)
            h_ref, added = O.external_inflow(area, ext, h_ref, t + 0.5 * dt, dt)
            t += dt
            total += added
            np.testing.assert_array_equal(s.get_state()[0], h_ref)
        assert s.ledger()["external_boundary_inflow_m3"] == pytest.approx(total, rel=1e-6)
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_recharge_step_matches_oracle_bitwise(gpu):
    from floodgb import native as N

    d = FORCING
    sc = F.forcing_scenario(d, "run/")
    sc.city.external_boundary = None
    st = sc.city.topologies.surface_topology
    area = np.asarray(st.cell_area_m2, np.float32)
    topo = sc.city.recharge_topology
    rng = np.random.default_rng(4)
    h_ref = np.array(sc.city.topologies.surface_state.h_m, np.float32)
    h_ref[topo.source_cell_index] = rng.uniform(0.0, 0.6, topo.source_cell_index.size).astype(np.float32)
    store0 = np.zeros(topo.source_cell_index.size, np.float32)
    store0[::4] = np.asarray(topo.storage_capacity_m3, np.float32)[::4] * np.float32(0.95)
    s = _solver(sc)
    try:
        s.set_state(h=h_ref)
        s.set_recharge_storage(store0)
        store = store0.copy()
        cap_total = loss_total = 0.0
        for dt in (0.9, 30.0, 5.0, 120.0, 0.25):
            s.step(dt, phases=N.FL_PHASE_RECHARGE)
            h_ref, store, cap, loss = O.recharge(area, topo, h_ref, store, dt)
            cap_total += cap
            loss_total += loss
            np.testing.assert_array_equal(s.get_state()[0], h_ref)
            np.testing.assert_array_equal(s.recharge_storage(), store)
        led = s.ledger()
        assert led["surface_recharge_capture_m3"] == pytest.approx(cap_total, rel=1e-6)
        assert led["surface_recharge_loss_m3"] == pytest.approx(loss_total, rel=1e-6)
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_run_with_inflow_and_recharge_matches_reference(gpu):
    from floodgb.config import load_config
    from floodgb.engine import run_simulation

    d = FORCING
    p = "run/"
    sc = F.forcing_scenario(d, p)
    cfg = load_config(None, sc.overrides)
    res = run_simulation(sc.city, sc.rainfall, cfg)
    assert abs(res.step_count - int(d[p + "step_count"])) <= 2
    ref_h = d[p + "snap_h"]
    assert res.depth_snapshots_m.shape == ref_h.shape
    area = np.asarray(sc.city.topologies.surface_topology.cell_area_m2, np.float64)
    valid = np.asarray(sc.city.mesh.active_mask, bool)
    for k in range(ref_h.shape[0]):
        diff = (res.depth_snapshots_m[k].astype(np.float64) - ref_h[k])[valid]
        assert np.sqrt(np.mean(diff ** 2)) <= 1e-4, k
        vc, vr = float(np.sum(res.depth_snapshots_m[k] * area)), float(np.sum(ref_h[k] * area))
        assert abs(vc - vr) <= 5e-4 * max(abs(vr), 1.0), k
    mb = res.mass_balance
    names = ["rainfall_input_m3", "infiltration_loss_m3", "boundary_net_flux_m3", "outfall_discharge_m3",
             "overflow_surcharge_m3", "unreturned_overflow_m3", "external_boundary_inflow_m3",
             "surface_recharge_capture_m3", "surface_recharge_loss_m3"]
    np.testing.assert_allclose([mb[n] for n in names], d[p + "ledger"], rtol=1e-4, atol=1e-2)


@pytest.mark.gpu
def test_gpu_ledger_closes_with_inflow_and_recharge(gpu):
    from floodgb.domain import June5RechargeTopology

    d = FORCING
    sc = F.forcing_scenario(d, "run/")
    # rows sharing a cell each capture from the same depth while only the last
    # one lowers it (the reference's NumPy assignment), which creates volume:
    # keep one row per cell for the balance
    r = sc.city.recharge_topology
    _, first = np.unique(r.source_cell_index, return_index=True)
    keep = np.sort(first)
    assert keep.size < r.source_cell_index.size
    sc.city.recharge_topology = June5RechargeTopology(
        **{k: np.asarray(getattr(r, k))[keep] for k in ("source_cell_index", "overflow_cell_index", "storage_capacity_m3",
                                                         "capture_capacity_m3ps", "recharge_capacity_m3ps",
                                                         "activation_depth_m", "stop_depth_m")})
    topo = sc.city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    v0 = float(np.sum(np.asarray(topo.surface_state.h_m, np.float64) * area)) + float(
        np.sum(topo.pipe_state.node_volume_m3))
    s = _solver(sc)
    try:
        s.run()
        led = s.ledger()
        stored = float(np.sum(s.recharge_storage(), dtype=np.float64))
    finally:
        s.close()
    assert led["external_boundary_inflow_m3"] > 1.0 and led["surface_recharge_capture_m3"] > 1.0
    lhs = v0 + led["rainfall_input_m3"] + led["external_boundary_inflow_m3"]
    rhs = (led["surface_volume_m3"] + led["node_volume_m3"] + led["infiltration_loss_m3"]
           + led["outfall_discharge_m3"] + led["unreturned_overflow_m3"] - led["boundary_net_flux_m3"]
           + led["surface_recharge_loss_m3"] + stored)
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)
    assert led["surface_recharge_capture_m3"] == pytest.approx(stored + led["surface_recharge_loss_m3"], rel=1e-5)
