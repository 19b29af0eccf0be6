"""Host-side rows against the reference's own code (CPU only).

* The topology builder against the reference's
  ``build_triangular_surface_topology`` (triangular_backend.py:244-326,
  1815-1869) on the fixtures ``make_golden.py`` wrote from it: every array
  bit-for-bit on irregular meshes (Delaunay, jittered grids, clockwise input
  triangles, every boundary mode and alias), and the same ValueError text for
  every invalid input.
* The run outputs against the reference's writer (postprocessing/outputs.py:
  25-99): the NPZ's array names, dtypes, shapes and values, and the report's
  keys, for the same run.
* ``floodgb.parity`` against the reference's ``validate_v1_parity_run``
  (hybrid_flood/operational/parity_validation.py:43-253), which accepted a
  candidate directory written by ``floodgb.outputs`` when the fixture was made.
"""

import json
import re
from types import SimpleNamespace

import numpy as np
import pytest

import fixtures as F
from floodgb import outputs as fout
from floodgb.config import load_config
from floodgb.parity import compare_runs
from floodgb.topology import build_triangular_surface_topology

TOPO = F.load("topology_cases.npz")
OUT = F.load("output_cases.npz")
SURFACE = F.load("surface_cases.npz")

TOPO_FIELDS = {"bed": "bed_elevation_m", "manning": "manning_n", "area": "cell_area_m2",
               "char_len": "characteristic_length_m", "left": "edge_left_cell", "right": "edge_right_cell",
               "nx": "edge_normal_x", "ny": "edge_normal_y", "len": "edge_length_m", "bcode": "boundary_code"}


def assert_topology_equal(st, d, p):
    for key, attr in TOPO_FIELDS.items():
        got, want = np.asarray(getattr(st, attr)), d[p + key]
        assert got.dtype == want.dtype, (attr, got.dtype, want.dtype)
        np.testing.assert_array_equal(got, want, err_msg=attr)
    if int(d[p + "has_active"]):
        assert st.active_mask is not None
        np.testing.assert_array_equal(np.asarray(st.active_mask), d[p + "active"])
        assert np.asarray(st.active_mask).dtype == np.float32
    else:
        assert st.active_mask is None
    assert bool(st.has_stage_boundary) == bool(int(d[p + "has_stage"]))


@pytest.mark.parametrize("name", [str(n) for n in TOPO["cases"]])
def test_topology_builder_matches_reference(name):
    d = TOPO
    p = f"{name}/"
    kind = str(d[p + "manning_kind"])
    manning = {"cell": lambda: d[p + "in_manning"], "none": lambda: None,
               "scalar": lambda: float(d[p + "in_manning"])}[kind]()
    active = d[p + "in_active"] if d[p + "in_active"].size else None
    st = build_triangular_surface_topology(d[p + "nodes"], d[p + "triangles"], d[p + "in_bed"], manning, active,
                                           str(d[p + "mode"]))
    assert_topology_equal(st, d, p + "out/")


def test_topology_builder_matches_reference_on_surface_fixture():
    """The grid the surface-step fixtures were built on (outflow boundary, per-cell n, active mask)."""

    d = SURFACE
    st = build_triangular_surface_topology(d["topo_nodes"], d["topo_triangles"], d["topo_bed"], d["topo_manning"],
                                           d["topo_active"], "outflow")
    assert_topology_equal(st, d, "outflow_percell/")


@pytest.mark.parametrize("name", [str(n) for n in TOPO["errors"]])
def test_topology_builder_rejects_what_the_reference_rejects(name):
    d = TOPO
    p = f"err/{name}/"
    manning = d[p + "manning"] if d[p + "manning"].size else None
    active = d[p + "active"] if d[p + "active"].size else None
    with pytest.raises(ValueError, match="^" + re.escape(str(d[p + "message"])) + "$"):
        build_triangular_surface_topology(d[p + "nodes"], d[p + "triangles"], d[p + "bed"], manning, active,
                                          str(d[p + "mode"]))


def _result(which: str):
    d = OUT
    meta = json.loads(str(d["meta"]))
    static = {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith("static/")}
    mesh = SimpleNamespace(**{k.split("/", 1)[1]: v for k, v in static.items() if k.startswith("mesh/")})
    cp = SimpleNamespace(node_x_m=static["cp/node_x_m"], node_y_m=static["cp/node_y_m"],
                         node_count=int(static["cp/node_count"]), inlet_count=int(static["cp/inlet_count"]))
    pp = SimpleNamespace(link_from_node_index=static["pp/link_from_node_index"],
                         link_to_node_index=static["pp/link_to_node_index"], link_count=int(static["pp/link_count"]))
    city = SimpleNamespace(mesh=mesh, topologies=SimpleNamespace(coupling_topology=cp, pipe_topology=pp),
                           topology_mode=meta["topology_mode"])
    arrays = {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith(which + "/") and not k.endswith("mass_balance")}
    keys = ("step_count", "runtime_s", "cfl_eval_count", "cfl_reused_count", "backend_name", "is_gpu", "duration_min")
    return SimpleNamespace(**arrays, mass_balance=json.loads(str(d[which + "/mass_balance"])),
                           **{k: meta[k] for k in keys}, city=city,
                           rainfall=SimpleNamespace(source_csv=meta["source_csv"], total_depth_mm=meta["total_depth_mm"]),
                           config=load_config(None, {"solver.duration_min": 2.0})), static


def test_run_npz_matches_reference_writer(tmp_path):
    res, _ = _result("ref")
    path = fout.save_run_npz(res, tmp_path)
    assert path.name == "flood_simulation_outputs.npz"
    want = [str(n) for n in OUT["npz_names"]]
    with np.load(path, allow_pickle=False) as z:
        assert sorted(z.files) == want
        for name in want:
            ref = OUT[f"npz/{name}"]
            assert z[name].dtype == ref.dtype and z[name].shape == ref.shape, (name, z[name].dtype, ref.dtype)
            np.testing.assert_array_equal(z[name], ref, err_msg=name)


def _key_tree(d):
    return {k: _key_tree(v) if isinstance(v, dict) else None for k, v in d.items()}


def test_report_keys_match_reference_writer(tmp_path):
    res, _ = _result("ref")
    ref = json.loads(str(OUT["report_json"]))
    got = fout.build_report(res, {"npz": "flood_simulation_outputs.npz"})
    assert set(got) == set(ref)
    for k, v in ref.items():
        if k in ("implementation", "artifacts", "config"):
            continue
        assert got[k] == pytest.approx(v) if isinstance(v, float) else got[k] == v, k
    # config: every reference section and key; the extra keys are the inlet-exchange knobs
    rc, gc = _key_tree(ref["config"]), _key_tree(got["config"])
    assert set(rc) == set(gc)
    for section in rc:
        assert set(rc[section]) <= set(gc[section]), section
        extra = set(gc[section]) - set(rc[section])
        assert extra == (set() if section != "physics" else {
            "inlet_capture_rule", "inlet_orifice_area_m2", "inlet_orifice_coefficient", "inlet_weir_perimeter_m",
            "inlet_weir_coefficient"}), (section, extra)
    for section in ("topology", "solver", "physics"):
        for k in rc[section]:
            assert got["config"][section][k] == ref["config"][section][k], (section, k)
    # a report written with the topology path carries what the reference validator reads
    p = fout.write_report(res, tmp_path, topology_path=tmp_path / "topology.npz")
    written = json.loads(p.read_text())
    assert written["input_report"]["assets"]["assets"]["topology"]["path"].endswith("topology.npz")
    assert written["v1_compatible_mass_residual_ratio"] == res.mass_balance["mass_residual_ratio"]


def test_parity_figures_match_reference_validator():
    ref, static = _result("ref")
    cand, _ = _result("cand")
    val = json.loads(str(OUT["validation_json"]))
    valid = static["mesh/active_mask"].astype(bool) & ~static["mesh/building_mask"].astype(bool)
    r = compare_runs(ref.snapshot_times_min * 60.0, ref.depth_snapshots_m, cand.snapshot_times_min * 60.0,
                     cand.depth_snapshots_m, valid, static["cell_area_m2"],
                     ref_node_volume=ref.final_node_volume_m3, cand_node_volume=cand.final_node_volume_m3,
                     ref_link_flow=ref.final_link_flow_m3ps, cand_link_flow=cand.final_link_flow_m3ps)
    assert len(r["snapshots"]) == len(val["hourly"]) >= 3
    for mine, theirs in zip(r["snapshots"], val["hourly"]):
        for k, v in theirs.items():
            assert mine[k] == pytest.approx(v, rel=1e-12, abs=1e-15), (mine["snapshot_index"], k)
    for k, v in val["drainage_state"].items():
        assert r["drainage_state"][k] == pytest.approx(v, rel=1e-12), k
    s, vs = r["summary"], val["summary"]
    assert s["maximum_snapshot_valid_depth_rmse_m"] == pytest.approx(vs["maximum_hourly_valid_depth_rmse_m"], rel=1e-12)
    assert s["minimum_snapshot_flood_extent_csi"] == pytest.approx(vs["minimum_hourly_flood_extent_csi"], rel=1e-12)
    assert s["maximum_snapshot_surface_volume_error_fraction"] == pytest.approx(
        vs["maximum_hourly_surface_volume_error_fraction"], rel=1e-12)
    assert s["maximum_snapshot_time_delta_s"] == pytest.approx(vs["maximum_snapshot_time_delta_s"], abs=1e-9)
    # the perturbation was chosen to move the extent: the CSI gate has something to see
    assert 0.5 < s["minimum_snapshot_flood_extent_csi"] < 1.0
    assert r["reference_gates"]["finite_non_negative_depth"] == val["gates"]["finite_non_negative_depth"]
    assert r["reference_gates"]["snapshot_alignment_le_1s"] == val["gates"]["snapshot_alignment_le_1s"]
