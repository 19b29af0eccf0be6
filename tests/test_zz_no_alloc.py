"""The allocation-free CFL entry point against the solver's own one.

``fl_stable_timestep_noalloc`` serves callers that cannot allocate device
memory when they need a timestep (a plugin tied to its host application's
memory pool, code running under someone else's stream capture, a service that
forbids allocation after start-up): its scratch is a static device array
inside the library, shared by every call.  The cases here run it at 4 blocks,
at 1,956 blocks and at its limit of 4,096 blocks (8,388,608 cells), several
calls back to back on one stream before a single synchronisation (each call
must find the shared done counter back at zero), and on NaN depths and on
inputs where no cell gives a finite dt.  This file is collected last so that
a failure here leaves every other test already run.
"""

import ctypes as C

import numpy as np
import pytest

from floodgb import native
from floodgb.config import load_config
from floodgb.solver import FloodSolver
from floodgb.synthetic import make_grid_city

pytestmark = pytest.mark.gpu

LIMIT = 8_388_608


@pytest.fixture(scope="module")
def lib():
    from floodgb.build import build_library

    build_library()
    lib = native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    return lib


def wet_state(n, seed):
    rng = np.random.default_rng(seed)
    h = rng.uniform(0.0, 0.8, n).astype(np.float32)
    h[rng.random(n) < 0.3] = 0.0
    hu = (h * rng.uniform(-2, 2, n)).astype(np.float32)
    hv = (h * rng.uniform(-2, 2, n)).astype(np.float32)
    return h, hu, hv


def reference_dt(cl, h, hu, hv, cfl=0.85, g=9.80665, md=1.0e-5):
    """The reference's stable_timestep_s (equations.py:155-178) as it runs
    with NumPy on float32 arrays (every operation correctly rounded in
    float32), with -1.0 for "no finite cell" where the reference raises."""

    h_safe = np.maximum(h, np.float32(md))
    speed = np.sqrt((hu / h_safe) ** 2 + (hv / h_safe) ** 2) + np.sqrt(np.float32(g) * h_safe)
    local = np.float32(cfl) * cl / np.maximum(speed, np.float32(1.0e-12))
    m = np.where(np.isfinite(local), local, np.float32(np.inf)).min()
    return float(m) if np.isfinite(m) else -1.0


def noalloc_calls(lib, cl, states, cfl=0.85, dev=0):
    """One call per state, back to back on one stream, one sync at the end."""

    import torch

    device = torch.device("cuda", dev)
    stream = torch.cuda.current_stream(device)
    tcl = torch.tensor(cl, device=device)
    dev_states = [tuple(torch.tensor(a, device=device) for a in s) for s in states]
    out = torch.zeros(len(states), dtype=torch.float64, device=device)
    for k, (th, thu, thv) in enumerate(dev_states):
        rc = lib.fl_stable_timestep_noalloc(
            C.c_void_p(tcl.data_ptr()), C.c_void_p(th.data_ptr()), C.c_void_p(thu.data_ptr()),
            C.c_void_p(thv.data_ptr()), len(cl), cfl, 9.80665, 1.0e-5, C.c_void_p(out.data_ptr() + 8 * k),
            C.c_void_p(stream.cuda_stream))
        native.check(rc, "fl_stable_timestep_noalloc")
    torch.cuda.synchronize(device)
    return out.cpu().numpy().tolist()


def solver_dts(sc, states):
    st = sc.city.topologies.surface_topology
    cfg = load_config(None, sc.overrides)
    solver = FloodSolver(st, cfg=cfg, duration_s=60.0, centroids=sc.city.mesh.centroids_xy)
    try:
        out = []
        for h, hu, hv in states:
            solver.set_state(h, hu, hv)
            out.append(solver.stable_timestep())  # the existing entry point
        return out, cfg.solver.cfl
    finally:
        solver.close()


def test_noalloc_timestep_matches_solver_on_calls_in_a_row(lib):
    sc = make_grid_city(n=60, size_m=600.0, seed=3)  # 7,200 cells: 4 blocks
    st = sc.city.topologies.surface_topology
    states = [wet_state(st.cell_count, seed) for seed in (10, 11, 12)]
    expected, cfl = solver_dts(sc, states)
    got = noalloc_calls(lib, np.asarray(st.characteristic_length_m, np.float32), states, cfl)
    # both evaluate the same float32 expression, correctly rounded: the same bits
    assert got == expected


def test_noalloc_timestep_matches_solver_on_four_million_cells(lib):
    sc = make_grid_city(n=1415, size_m=14150.0, seed=4)  # 4,004,450 cells: 1,956 blocks
    st = sc.city.topologies.surface_topology
    assert st.cell_count == 4_004_450
    states = [wet_state(st.cell_count, seed) for seed in (20, 21)]
    expected, cfl = solver_dts(sc, states)
    cl = np.asarray(st.characteristic_length_m, np.float32)
    got = noalloc_calls(lib, cl, states, cfl)
    assert got == expected
    assert got == [reference_dt(cl, *s, cfl=cfl) for s in states]


def test_noalloc_timestep_at_its_limit(lib):
    """Exactly 8,388,608 cells (4,096 blocks, the last block reducing 4,096
    block minima), the global minimum placed in the last block, two calls in
    a row, against the reference's expression."""

    rng = np.random.default_rng(30)
    cl = rng.uniform(2.0, 12.0, LIMIT).astype(np.float32)
    states = [wet_state(LIMIT, seed) for seed in (31, 32)]
    states[1][1][LIMIT - 5] = np.float32(40.0)  # a fast wet cell in the last block
    states[1][0][LIMIT - 5] = np.float32(0.9)
    got = noalloc_calls(lib, cl, states)
    assert got == [reference_dt(cl, *s) for s in states]


def test_noalloc_skips_nan_depth_and_reports_no_finite_cell(lib):
    rng = np.random.default_rng(40)
    n = 20_000
    cl = rng.uniform(2.0, 12.0, n).astype(np.float32)
    h, hu, hv = wet_state(n, 41)
    # a NaN depth with large momentum next to a fast wet cell: the reference's
    # maximum passes the NaN through, so that cell is skipped, not clamped
    h[1234], hu[1234], hv[1234] = np.float32(np.nan), np.float32(50.0), np.float32(0.0)
    h[1235], hu[1235], hv[1235] = np.float32(0.2), np.float32(3.0), np.float32(0.0)
    nan_all = (np.full(n, np.nan, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32))
    got = noalloc_calls(lib, cl, [(h, hu, hv), nan_all, (h, hu, hv)])
    assert got[0] == reference_dt(cl, h, hu, hv) and got[0] > 0
    assert got[1] == -1.0
    assert got[2] == got[0]


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    import torch

    dev = torch.device("cuda", 0)
    x = torch.zeros(1, dtype=torch.float32, device=dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    rc = lib.fl_stable_timestep_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                        C.c_void_p(x.data_ptr()), LIMIT + 1, 0.85, 9.80665, 1.0e-5,
                                        C.c_void_p(out.data_ptr()), None)
    assert rc == native.FL_E_INVALID
    assert "allocation-free limit" in native.last_error()
