"""floodgb: the explicit finite-volume flood step on GB300 (sm_103a).

A from-scratch GPU implementation of the hot path of the coupled urban flood
model in arsanjeevk/gpu-urban-flood-cupy-jax, usable as a drop-in for that
model's CuPy backend:

* ``floodgb.engine.run_simulation`` -- the whole adaptive run on the device;
* ``floodgb.backend`` -- the per-step functions of the reference backend;
* ``floodgb.solver.FloodSolver`` -- the device solver over the C ABI
  (``include/floodgb.h``, ``libfloodgb.so``).
"""

from .config import RunConfig, load_config
from .exceptions import BackendUnavailableError, ConfigError, GurugramFloodError, SimulationError
from .topology import (
    TriangularNodeCouplingTopology,
    TriangularPipeNetworkState,
    TriangularPipeNetworkTopology,
    TriangularSurfaceForcing,
    TriangularSurfaceState,
    TriangularSurfaceTopology,
    build_triangular_surface_topology,
)

__all__ = [
    "RunConfig", "load_config", "BackendUnavailableError", "ConfigError", "GurugramFloodError", "SimulationError",
    "TriangularNodeCouplingTopology", "TriangularPipeNetworkState", "TriangularPipeNetworkTopology",
    "TriangularSurfaceForcing", "TriangularSurfaceState", "TriangularSurfaceTopology",
    "build_triangular_surface_topology",
]
