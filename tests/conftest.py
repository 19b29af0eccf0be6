"""Test configuration: import paths and the ``gpu`` marker.

Tests marked ``gpu`` need a CUDA device and the built ``libfloodgb.so``; the
rest run on CPU only.
"""

import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "gpu-urban-flood-cupy-jax_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfloodgb")
