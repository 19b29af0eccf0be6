"""Exact production topology export (NPZ with the reference export's array
names, ``gurugram_flood/domain/production_topology_loader.py:45-137``) and the
per-cell infiltration fields built from it."""

import numpy as np
import pytest

from floodgb.domain import (
    load_exact_production_topologies,
    prepare_production_infiltration_fields,
    production_city,
    save_exact_production_topologies,
)
from floodgb.synthetic import add_surcharge_table, coupled_test_city


def _city():
    sc = coupled_test_city(scale=1, seed=4, duration_min=5.0)
    add_surcharge_table(sc, seed=1)
    return sc


def test_npz_round_trip_keeps_every_array(tmp_path):
    sc = _city()
    topo = sc.city.topologies
    cp = topo.coupling_topology
    fill = np.linspace(0.0, 0.5, cp.node_count).astype(np.float32)
    from floodgb.topology import TriangularNodeCouplingTopology

    topo.coupling_topology = TriangularNodeCouplingTopology(**{**cp.__dict__, "node_initial_fill_depth_m": fill})
    p = tmp_path / "topology.npz"
    save_exact_production_topologies(p, topo)
    back = load_exact_production_topologies(p)
    st, bt = topo.surface_topology, back.surface_topology
    for name in ("bed_elevation_m", "manning_n", "cell_area_m2", "characteristic_length_m", "edge_left_cell",
                 "edge_right_cell", "edge_normal_x", "edge_normal_y", "edge_length_m", "boundary_code"):
        np.testing.assert_array_equal(np.asarray(getattr(bt, name)), np.asarray(getattr(st, name)), err_msg=name)
    np.testing.assert_array_equal(np.asarray(bt.active_mask) > 0.5, np.asarray(st.active_mask) > 0.5)
    for name in ("inlet_cell_index", "inlet_node_index", "node_surface_cell_index", "node_invert_elevation_m",
                 "node_storage_area_m2", "node_max_depth_m", "surcharge_cell_index", "surcharge_node_index",
                 "surcharge_return_weight"):
        np.testing.assert_array_equal(np.asarray(getattr(back.coupling_topology, name)),
                                      np.asarray(getattr(topo.coupling_topology, name)), err_msg=name)
    for name in ("link_from_node_index", "link_to_node_index", "link_length_m", "link_area_m2", "link_manning_n",
                 "link_hydraulic_radius_m", "outfall_area_m2", "link_diameter_m"):
        if getattr(topo.pipe_topology, name) is not None:
            np.testing.assert_array_equal(np.asarray(getattr(back.pipe_topology, name)),
                                          np.asarray(getattr(topo.pipe_topology, name)), err_msg=name)
    np.testing.assert_allclose(back.pipe_state.node_volume_m3,
                               np.asarray(cp.node_storage_area_m2, np.float64) * fill.astype(np.float64))
    assert back.mesh.triangle_count == topo.mesh.triangle_count
    assert back.surface_state.h_m.shape == (st.cell_count,)


def test_infiltration_fields_from_export_arrays():
    n = 5
    act = np.array([1, 1, 0, 1, 1], bool)
    f = prepare_production_infiltration_fields(active_mask=act)
    np.testing.assert_array_equal(f.rainfall_multiplier, np.ones(n, np.float32))
    assert f.horton_f0_mps[0] == np.float32(6.5 / 3.6e6) and f.horton_fc_mps[0] == np.float32(1.0 / 3.6e6)
    assert f.horton_k_per_s[0] == np.float32(2.0 / 3600.0)
    g = prepare_production_infiltration_fields(
        active_mask=act, rainfall_multiplier=np.full(n, 1.2), horton_f0_mmhr=np.full(n, 75.0),
        horton_fc_mmhr=np.full(n, 10.0), horton_decay_per_hr=np.full(n, 4.0), building_fraction=np.full(n, 0.99))
    assert g.horton_f0_mps[0] == np.float32(75.0 / 3.6e6) and g.horton_k_per_s[0] == np.float32(4.0 / 3600.0)
    np.testing.assert_allclose(g.open_fraction, 0.05)  # clipped at the minimum open fraction
    np.testing.assert_allclose(g.rainfall_multiplier, 1.2)


@pytest.mark.gpu
def test_gpu_run_from_exported_city_matches_original(tmp_path):
    from floodgb import native
    from floodgb.config import load_config
    from floodgb.solver import solver_for_city

    native.load(build_if_missing=True)
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    sc = _city()
    p = tmp_path / "topology.npz"
    save_exact_production_topologies(p, sc.city.topologies)
    city2 = production_city(p)
    city2.infiltration_fields = sc.city.infiltration_fields  # same forcing as the original run
    city2.topologies.surface_state = sc.city.topologies.surface_state
    city2.topologies.pipe_state = sc.city.topologies.pipe_state
    cfg = load_config(None, sc.overrides)
    out = []
    for city in (sc.city, city2):
        s = solver_for_city(city, sc.rainfall, cfg)
        try:
            s.run()
            out.append((s.snapshots()[1], s.get_state()))
        finally:
            s.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        np.testing.assert_array_equal(a, b)
