"""Precision of the eliminations and the checked reduced-precision contract.

Mirrors ``crates/caroli-green/src/precision.rs``: ``Precision`` (``:22-32``), ``PrecisionOptions``
(``:34-61``), ``PrecisionReport`` (``:63-78``) and ``checked`` (``:80-134``): run a batch in the
chosen precision, recompute one point in ``every`` (and every failed point) in double precision,
and recompute the whole batch in double precision when a sampled difference exceeds the tolerance.
``MIXED`` is new: complex-f32 fronts precondition an FP64 iterative refinement of the whole solve.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np


class Precision(IntEnum):
    DOUBLE = 0
    SINGLE = 1
    MIXED = 2


@dataclass
class PrecisionOptions:
    precision: Precision = Precision.DOUBLE
    tolerance: float = 0.0
    every: int = 0

    @staticmethod
    def double():
        return PrecisionOptions(Precision.DOUBLE, 0.0, 0)

    @staticmethod
    def single():
        return PrecisionOptions(Precision.SINGLE, 1e-2, 50)

    @staticmethod
    def mixed():
        return PrecisionOptions(Precision.MIXED, 1e-8, 50)


@dataclass
class PrecisionReport:
    precision: Precision = Precision.DOUBLE
    checked: int = 0
    median: float = 0.0
    max: float = 0.0
    failed: int = 0
    fallback: str | None = None


def checked(points, options: PrecisionOptions, run, distance=lambda a, b: abs(a - b)):
    """``run(points, precision) -> list of results (value or exception)`` over the whole batch."""
    report = PrecisionReport(precision=options.precision)
    out = list(run(points, options.precision))
    if options.precision == Precision.DOUBLE or len(points) == 0:
        return out, report
    every = max(options.every, 1)
    redo = [i for i in range(len(points)) if isinstance(out[i], Exception) or i % every == 0]
    exact = run([points[i] for i in redo], Precision.DOUBLE)
    diffs = []
    for i, d in zip(redo, exact):
        if isinstance(out[i], Exception):
            report.failed += 1
        elif isinstance(d, Exception):
            diffs.append(float("nan"))
        else:
            diffs.append(distance(out[i], d))
        out[i] = d
    report.checked = len(diffs)
    diffs.sort(key=lambda x: (np.isnan(x), x))
    if diffs:
        report.median = diffs[len(diffs) // 2]
        report.max = float("nan") if any(np.isnan(d) for d in diffs) else diffs[-1]
    if np.isnan(report.max) or report.max > options.tolerance:
        report.fallback = (f"largest difference {report.max:.1e} above the tolerance {options.tolerance:.1e}: "
                           f"all {len(points)} points recomputed in double precision")
        report.precision = Precision.DOUBLE
        out = list(run(points, Precision.DOUBLE))
    return out, report
