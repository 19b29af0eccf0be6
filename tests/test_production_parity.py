"""Parity at production size: the 981,880-triangle coupled 60-minute run
(1,490,015 edges, 817,573 active cells, 118,768 nodes, 139,798 links, 61,317
inlets, 46 outfalls, Horton infiltration, hour 1 of the 160 mm / 24 h
front-loaded hyetograph) through the device loop against the oracle's
restated engine loop on the same seeded inputs.

Gates, at every 10-minute snapshot (a finer schedule than the hourly one the
reference writes, so the trajectory is checked, not only its end): depth RMSE
<= 1e-3 m over the valid cells, flood-extent CSI >= 0.995 at 0.05 m and
surface-volume error <= 0.05 %, computed as the reference's
validate_v1_parity_run does (hybrid_flood/operational/parity_validation.py:
99-124) together with its own looser gates (:179-192).  Step counts agree
within 0.5 %, and both float64 mass ledgers close.

The oracle needs about two minutes of all host cores for the hour.
"""

import numpy as np
import pytest

import oracle as O
from floodgb import native
from floodgb.config import load_config
from floodgb.parity import compare_runs
from floodgb.solver import solver_for_city
from floodgb.synthetic import production_workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def production_runs():
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    sc = production_workload()
    cfg = load_config(None, dict(sc.overrides, **{"solver.snapshot_interval_min": 10.0}))
    s = solver_for_city(sc.city, sc.rainfall, cfg)
    try:
        s.run()
        prog = s.progress()
        snaps = s.snapshots()
        state = s.get_state()
        led = s.ledger()
    finally:
        s.close()
    ref = O.run(sc, cfg)
    return sc, prog, snaps, state, led, ref


def test_production_hour_meets_drop_in_gates(production_runs):
    sc, prog, (t, h, hu, hv, v), (fh, fhu, fhv, fV, fQ), led, ref = production_runs
    topo = sc.city.topologies
    assert topo.surface_topology.cell_count == 981_880
    assert topo.surface_topology.edge_count == 1_490_015
    assert topo.coupling_topology.node_count == 118_768 and topo.pipe_topology.link_count == 139_798
    assert prog.error == 0 and ref.error == 0
    assert abs(prog.step_count - ref.step_count) <= max(5, ref.step_count // 200), (prog.step_count, ref.step_count)
    assert h.shape == ref.depth.shape and h.shape[0] >= 7
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    mesh = sc.city.mesh
    valid = np.asarray(mesh.active_mask, bool) & ~np.asarray(mesh.building_mask, bool)
    r = compare_runs(ref.snapshot_times_s, ref.depth, t, h, valid, area,
                     ref_node_volume=ref.final_node_volume, cand_node_volume=fV,
                     ref_link_flow=ref.final_link_flow, cand_link_flow=fQ)
    rows = [(row["snapshot_index"], row["candidate_time_s"], row["valid_depth_rmse_m"], row["flood_extent_csi"],
             row["surface_volume_error_fraction"]) for row in r["snapshots"]]
    assert all(r["drop_in_gates"].values()), (r["summary"], rows)
    assert r["passed"], r["reference_gates"]
    # wherever anything is wet, the reference's own CSI figure is the gated one
    for row in r["snapshots"]:
        if row["reference_wet_triangle_count"] or row["candidate_wet_triangle_count"]:
            assert row["flood_extent_csi"] == row["extent_agreement_csi"] >= 0.995, row
    # the flood has developed: the final snapshot has a real wet extent
    assert r["snapshots"][-1]["reference_wet_triangle_count"] > 10_000


def test_production_hour_ledgers_close_and_agree(production_runs):
    sc, prog, snaps, state, led, ref = production_runs
    topo = sc.city.topologies
    area = np.asarray(topo.surface_topology.cell_area_m2, np.float64)
    v0 = float(np.sum(np.asarray(topo.surface_state.h_m, np.float64) * area)) + float(
        np.sum(topo.pipe_state.node_volume_m3))
    lhs = v0 + led["rainfall_input_m3"]
    rhs = (led["surface_volume_m3"] + led["node_volume_m3"] + led["infiltration_loss_m3"]
           + led["outfall_discharge_m3"] + led["unreturned_overflow_m3"] - led["boundary_net_flux_m3"])
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (lhs, rhs)
    rv = float(np.sum(ref.final_h.astype(np.float64) * area)) + float(np.sum(ref.final_node_volume))
    rl = ref.ledger
    rrhs = (rv + rl["infiltration_loss_m3"] + rl["outfall_discharge_m3"] + rl["unreturned_overflow_m3"]
            - rl["boundary_net_flux_m3"])
    assert abs((v0 + rl["rainfall_input_m3"]) - rrhs) <= 1e-5 * max(abs(lhs), 1.0)
    # source / sink terms against the oracle's (the rain total depends on the dt sequence only through the last step)
    for name, rtol in (("rainfall_input_m3", 1e-4), ("infiltration_loss_m3", 5e-4), ("surface_capture_m3", 5e-3),
                       ("outfall_discharge_m3", 5e-3), ("overflow_surcharge_m3", 2e-2)):
        assert abs(led[name] - rl[name]) <= rtol * max(abs(rl[name]), 1.0), (name, led[name], rl[name])
