"""Error types with the reference's names and hierarchy.

``gurugram_flood/exceptions.py:11-41`` defines this hierarchy; callers that
catch ``SimulationError`` or ``BackendUnavailableError`` there catch the same
classes here.
"""

from __future__ import annotations


class GurugramFloodError(Exception):
    """Base class for errors raised deliberately by this package."""


class ConfigError(GurugramFloodError):
    """Invalid or inconsistent run configuration."""


class RainfallInputError(GurugramFloodError):
    """Malformed or implausible rainfall forcing."""


class BackendUnavailableError(GurugramFloodError):
    """The CUDA backend (libfloodgb + a visible GPU) could not be initialised."""


class SimulationError(GurugramFloodError):
    """The solver failed mid-run (non-finite depth, step cap, device error)."""


class NativeError(GurugramFloodError):
    """A libfloodgb call returned an error code not mapped to another type."""
