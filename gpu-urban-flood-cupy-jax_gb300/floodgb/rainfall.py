"""Rainfall hyetograph forcing.

A hyetograph is a table of ``(start_min, end_min, intensity_mmhr)`` rows.  The
rate at simulation time ``t`` follows the reference's ``hyetograph_rate_fn``
(``gurugram_flood/domain/real_gurugram_domain.py:374-388``): find the first row
whose end is strictly after ``t``; if there is none, or ``t`` is before that
row's start, the rate is zero; otherwise it is ``intensity / 1000 / 3600`` m/s.
The same lookup runs on the device (one thread per step) from the table
uploaded by :func:`hyetograph_arrays`.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable

import numpy as np


@dataclass
class RainfallEvent:
    """Rainfall forcing ready for the solver (reference ``rainfall.py:54-69``)."""

    start_min: np.ndarray
    end_min: np.ndarray
    intensity_mmhr: np.ndarray
    rate_fn: Callable[[float], float]
    total_depth_mm: float
    duration_min: float
    source_csv: str = "synthetic"
    intensity_by_hour: dict[int, float] = field(default_factory=dict)

    @property
    def n_steps(self) -> int:
        return int(self.start_min.shape[0])


def hyetograph_arrays(event: RainfallEvent) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(start_s, end_s, rate_mps) float64 arrays, as the rate lookup uses them."""

    start_s = np.asarray(event.start_min, dtype=float) * 60.0
    end_s = np.asarray(event.end_min, dtype=float) * 60.0
    rate = np.asarray(event.intensity_mmhr, dtype=float) / 1000.0 / 3600.0
    return start_s, end_s, rate


class HyetographRate:
    """Callable ``t_s -> rainfall rate (m/s)`` of a hyetograph table."""

    def __init__(self, start_min, end_min, intensity_mmhr):
        self.start_s = np.asarray(start_min, dtype=float) * 60.0
        self.end_s = np.asarray(end_min, dtype=float) * 60.0
        self.rate_mps = np.asarray(intensity_mmhr, dtype=float) / 1000.0 / 3600.0

    def __call__(self, t_s: float) -> float:
        idx = int(np.searchsorted(self.end_s, t_s, side="right"))
        if idx >= len(self.rate_mps) or t_s < self.start_s[idx]:
            return 0.0
        return float(self.rate_mps[idx])


def make_rate_fn(start_min, end_min, intensity_mmhr) -> Callable[[float], float]:
    return HyetographRate(start_min, end_min, intensity_mmhr)


def rainfall_event(start_min, end_min, intensity_mmhr, source: str = "synthetic") -> RainfallEvent:
    start = np.asarray(start_min, dtype=float)
    end = np.asarray(end_min, dtype=float)
    inten = np.asarray(intensity_mmhr, dtype=float)
    if start.shape != end.shape or start.shape != inten.shape or start.ndim != 1 or start.size == 0:
        from .exceptions import RainfallInputError

        raise RainfallInputError("hyetograph needs equal-length non-empty start/end/intensity columns")
    if np.any(end <= start) or np.any(inten < 0) or np.any(np.diff(end) < 0):
        from .exceptions import RainfallInputError

        raise RainfallInputError("hyetograph rows must have end > start, sorted ends and intensity >= 0")
    total = float(np.sum(inten * (end - start) / 60.0))
    by_hour = {int(s // 60): float(i) for s, i in zip(start, inten)}
    return RainfallEvent(
        start_min=start,
        end_min=end,
        intensity_mmhr=inten,
        rate_fn=make_rate_fn(start, end, inten),
        total_depth_mm=total,
        duration_min=float(end.max()),
        source_csv=source,
        intensity_by_hour=by_hour,
    )


def uniform_rainfall(intensity_mmhr: float, duration_min: float) -> RainfallEvent:
    return rainfall_event([0.0], [duration_min], [intensity_mmhr])


def hourly_rainfall(intensities_mmhr) -> RainfallEvent:
    inten = np.asarray(intensities_mmhr, dtype=float)
    start = np.arange(inten.size) * 60.0
    return rainfall_event(start, start + 60.0, inten)
