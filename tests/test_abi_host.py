"""CPU-only checks of the C ABI library and the host-side logic (no GPU calls)."""

import re
from pathlib import Path

import numpy as np
import pytest

import fixtures as F
from floodgb import native
from floodgb.config import load_config
from floodgb.exceptions import BackendUnavailableError, ConfigError, RainfallInputError
from floodgb.rainfall import hourly_rainfall, make_rate_fn, rainfall_event
from floodgb.synthetic import make_grid_city
from floodgb.topology import TriangularSurfaceTopology

HEADER = Path(__file__).resolve().parents[1] / "include" / "floodgb.h"


@pytest.fixture(scope="module")
def lib():
    from floodgb.build import build_library

    build_library()
    return native.load()


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"FL_API\s+[\w\s\*]+?\b(fl_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    declared = declared_symbols()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(native.exported_symbols()) == declared
    assert lib.fl_abi_version() == 1


def test_no_device_is_reported_not_faked(lib):
    # No GPU in this container: creation must fail loudly, never fall back to the CPU.
    if native.device_count() > 0:
        pytest.skip("a GPU is visible")
    sc = make_grid_city(n=4, size_m=40.0)
    from floodgb.solver import solver_for_city

    with pytest.raises(BackendUnavailableError):
        solver_for_city(sc.city, sc.rainfall, load_config(None, sc.overrides))


def test_plan_layout_on_coupled_fixture(lib):
    d = F.load("run_cases.npz")
    sc = F.scenario(d, "coupled/")
    topo = sc.city.topologies
    st = topo.surface_topology
    stats, perm = native.plan_check(st, topo.coupling_topology, topo.pipe_topology, sc.city.mesh.centroids_xy)
    assert stats["cells"] == st.cell_count and stats["edges"] == st.edge_count
    interior = int((np.asarray(st.edge_right_cell) >= 0).sum())
    assert stats["slots"] == 2 * interior + (st.edge_count - interior)
    assert np.array_equal(np.sort(perm), np.arange(st.cell_count))
    cells_with_inlets = np.unique(topo.coupling_topology.inlet_cell_index).size
    assert stats["inlet_cells"] == cells_with_inlets
    coupled = set(np.unique(topo.coupling_topology.inlet_cell_index).tolist())
    coupled |= set(int(c) for c in topo.coupling_topology.node_surface_cell_index if c >= 0)
    orphans = int((np.asarray(topo.coupling_topology.node_surface_cell_index) < 0).sum())
    assert stats["groups"] == len(coupled) + orphans
    assert stats["nodes"] == topo.coupling_topology.node_count
    assert stats["links"] == topo.pipe_topology.link_count


def test_hilbert_renumbering_improves_locality(lib):
    sc = make_grid_city(n=64, size_m=640.0)
    st = sc.city.topologies.surface_topology
    _, perm = native.plan_check(st, centroids=sc.city.mesh.centroids_xy)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    left = np.asarray(st.edge_left_cell)
    right = np.asarray(st.edge_right_cell)
    m = right >= 0
    before = np.abs(left[m] - right[m])
    after = np.abs(inv[left[m]] - inv[right[m]])
    # far neighbours (other grid rows) become rare along the curve
    assert np.percentile(after, 90) < np.percentile(before, 90)


def _with(st, **kw):
    return TriangularSurfaceTopology(**{**st.__dict__, **kw})


def test_plan_rejects_bad_inputs(lib):
    sc = make_grid_city(n=6, size_m=60.0)
    st = sc.city.topologies.surface_topology
    bad_left = np.array(st.edge_left_cell, copy=True)
    bad_left[3] = st.cell_count + 5
    with pytest.raises(ValueError, match="out of range"):
        native.plan_check(_with(st, edge_left_cell=bad_left))
    bad_code = np.array(st.boundary_code, copy=True)
    bad_code[np.flatnonzero(np.asarray(st.edge_right_cell) < 0)[0]] = 9
    with pytest.raises(ValueError, match="boundary code"):
        native.plan_check(_with(st, boundary_code=bad_code))
    frac = np.full(st.cell_count, 0.7, np.float32)
    with pytest.raises(NotImplementedError, match="0/1"):
        native.plan_check(_with(st, active_mask=frac))
    # a fourth edge on one cell
    left = np.append(np.asarray(st.edge_left_cell), 0).astype(np.int32)
    right = np.append(np.asarray(st.edge_right_cell), -1).astype(np.int32)
    grow = lambda a: np.append(np.asarray(a), np.asarray(a)[:1])  # noqa: E731
    four = _with(st, edge_left_cell=left, edge_right_cell=right, edge_normal_x=grow(st.edge_normal_x),
                 edge_normal_y=grow(st.edge_normal_y), edge_length_m=grow(st.edge_length_m),
                 boundary_code=np.append(np.asarray(st.boundary_code), 4).astype(np.int32))
    with pytest.raises(ValueError, match="more than three edges"):
        native.plan_check(four)


def test_config_keys_and_validation():
    cfg = load_config({"solver": {"cfl": 0.5}}, {"solver.max_dt_s": 0.5})
    assert cfg.solver.cfl == 0.5 and cfg.solver.max_dt_s == 0.5
    assert cfg.solver.cfl_update_interval_steps == 32 and cfg.solver.cfl_reuse_safety_factor == 0.8
    with pytest.raises(ConfigError, match="Unknown config key"):
        load_config({"solver": {"nope": 1}})
    with pytest.raises(ConfigError, match="Unknown config section"):
        load_config(None, {"bogus.key": 1})
    with pytest.raises(ConfigError, match="cfl"):
        load_config(None, {"solver.cfl": 1.5})
    with pytest.raises(ConfigError, match="backend"):
        load_config(None, {"solver.backend": "numpy"})


def test_rainfall_rate_lookup_semantics():
    rate = make_rate_fn([0, 60, 180], [60, 120, 240], [36.0, 72.0, 3.6])
    mps = lambda mmhr: mmhr / 1000.0 / 3600.0  # noqa: E731
    assert rate(0.0) == mps(36.0)
    assert rate(3599.9) == mps(36.0)
    assert rate(3600.0) == mps(72.0)        # end is exclusive
    assert rate(7300.0) == 0.0              # gap between rows
    assert rate(10800.0) == mps(3.6)
    assert rate(14400.0) == 0.0             # after the last row
    ev = hourly_rainfall([10.0, 20.0])
    assert ev.total_depth_mm == pytest.approx(30.0) and ev.duration_min == 120.0
    with pytest.raises(RainfallInputError):
        rainfall_event([0], [0], [1.0])


def test_small_workload_shape():
    sc = make_grid_city(n=100)
    st = sc.city.topologies.surface_topology
    assert st.cell_count == 20_000 and st.edge_count == 30_200
    assert int((np.asarray(st.boundary_code) == 4).sum()) == 400


def test_plan_accepts_surcharge_table_and_rejects_bad_entries(lib):
    from floodgb.topology import TriangularNodeCouplingTopology

    d = F.load("pipe_cases.npz")
    st = F.surface_topology(d, "mesh/")
    cp, pp = F.coupling_pipe(d, "table_orifice/")
    assert cp.surcharge_cell_index is not None
    stats, _ = native.plan_check(st, cp, pp)
    assert stats["nodes"] == cp.node_count
    bad = np.array(cp.surcharge_node_index, copy=True)
    bad[0] = cp.node_count + 3
    with pytest.raises(ValueError, match="surcharge entry"):
        native.plan_check(st, TriangularNodeCouplingTopology(**{**cp.__dict__, "surcharge_node_index": bad}), pp)
    short = np.asarray(cp.surcharge_return_weight)[:-1]
    with pytest.raises(ValueError, match="differ in length"):
        native.plan_check(st, TriangularNodeCouplingTopology(**{**cp.__dict__, "surcharge_return_weight": short}), pp)


def _gemm_desc(**kw):
    """A well-formed GEMM descriptor with placeholder device addresses (the
    checks below run before anything is dereferenced)."""

    import ctypes as C

    d = native.FlGemmDesc()
    d.a[0] = native.FlGemmSegment(C.c_void_p(0x10000), None, 128, 128)
    d.n_seg, d.m, d.n = 1, 256, 128
    d.b, d.ldb = C.c_void_p(0x20000), 128
    d.out_bf16, d.ldo = C.c_void_p(0x30000), 128
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("field,value", [("out_bf16", 0x30008), ("bias", 0x40004), ("residual", 0x50008),
                                         ("ldo", 100), ("n", 60)])
def test_gemm_rejects_misaligned_or_ragged_arguments(lib, field, value):
    import ctypes as C

    kw = {field: C.c_void_p(value) if field in ("out_bf16", "bias", "residual") else value}
    if field == "residual":
        kw["ldr"] = 128
    d = _gemm_desc(**kw)
    rc = native.load().fl_gemm_bf16(C.byref(d), None)
    assert rc == native.FL_E_INVALID
    assert b"fl_gemm_bf16" in native.load().fl_last_error()
