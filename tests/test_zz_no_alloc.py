"""The allocation-free CFL entry point against the solver's own one.

``fl_stable_timestep_noalloc`` serves callers that cannot allocate device
memory when they need a timestep (a plugin tied to its host application's
memory pool, code running under someone else's stream capture, a service that
forbids allocation after start-up): its scratch is a static device array
inside the library.  This file is collected last so that a failure here
leaves every other test already run.
"""

import ctypes as C

import numpy as np
import pytest

from floodgb import native
from floodgb.config import load_config
from floodgb.solver import FloodSolver
from floodgb.synthetic import make_grid_city

pytestmark = pytest.mark.gpu


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


def test_noalloc_timestep_matches_solver_on_two_calls(lib):
    import torch

    sc = make_grid_city(n=60, size_m=600.0, seed=3)
    st = sc.city.topologies.surface_topology
    cfg = load_config(None, sc.overrides)
    solver = FloodSolver(st, cfg=cfg, duration_s=60.0, centroids=sc.city.mesh.centroids_xy)
    dev = torch.device("cuda", 0)
    cl = torch.tensor(np.asarray(st.characteristic_length_m, np.float32), device=dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    try:
        for call, seed in enumerate((10, 11)):
            h, hu, hv = wet_state(st.cell_count, seed)
            solver.set_state(h, hu, hv)
            expected = solver.stable_timestep()          # the existing entry point
            th, thu, thv = (torch.tensor(a, device=dev) for a in (h, hu, hv))
            out.fill_(0.0)
            rc = lib.fl_stable_timestep_noalloc(
                C.c_void_p(cl.data_ptr()), C.c_void_p(th.data_ptr()), C.c_void_p(thu.data_ptr()),
                C.c_void_p(thv.data_ptr()), st.cell_count, cfg.solver.cfl, 9.80665, 1.0e-5,
                C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
            native.check(rc, "fl_stable_timestep_noalloc")
            torch.cuda.synchronize(dev)
            # both are the reference's float32 expression, correctly rounded: the same bits
            assert out.item() == expected, (call, out.item(), expected)
    finally:
        solver.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    import torch

    dev = torch.device("cuda", 0)
    x = torch.zeros(1, dtype=torch.float32, device=dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    rc = lib.fl_stable_timestep_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                        C.c_void_p(x.data_ptr()), 8_388_609, 0.85, 9.80665, 1.0e-5,
                                        C.c_void_p(out.data_ptr()), None)
    assert rc == native.FL_E_INVALID
    assert "allocation-free limit" in native.last_error()
