"""The checked reduced-precision contract (crates/caroli-green/src/precision.rs:80-134).

``checked`` runs a batch in the reduced precision, recomputes one point in ``every`` and every
failed point in double precision, and recomputes the whole batch in double precision when a
sampled difference exceeds the tolerance. The CPU test is the reference's own unit test
(precision.rs:140-171) on a synthetic run; the GPU tests run the contract on the transmission
path: the sample, the failed count (a point made to fail on the host with a non-finite
self-energy) and the whole-batch fallback.
"""
import numpy as np
import pytest

from caroli_gb300 import GreenError, Precision, PrecisionOptions, checked
from caroli_gb300.nested import LeadSelfEnergies


def _synthetic(points, precision):
    """precision.rs:144-151: index 7 is off by 1e-4 in single precision, index 3 fails."""
    out = []
    for i in points:
        if precision == Precision.SINGLE and i == 7:
            out.append(7.0 + 1e-4)
        elif precision == Precision.SINGLE and i == 3:
            out.append(GreenError("Singular", "synthetic"))
        else:
            out.append(float(i))
    return out


def test_checked_sample_failures_and_fallback():
    points = list(range(10))
    opts = PrecisionOptions(Precision.SINGLE, 1e-6, 5)
    out, rep = checked(points, opts, _synthetic)
    assert (rep.checked, rep.failed, rep.fallback) == (2, 1, None)
    assert out[3] == 3.0 and out[7] == 7.0 + 1e-4
    out, rep = checked(points, PrecisionOptions(Precision.SINGLE, 1e-6, 7), _synthetic)
    assert rep.fallback is not None and rep.precision == Precision.DOUBLE
    assert out == [float(i) for i in points]
    out, rep = checked(points, PrecisionOptions.double(), _synthetic)
    assert (rep.checked, rep.failed, rep.fallback, rep.precision) == (0, 0, None, Precision.DOUBLE)


def test_checked_nan_difference_falls_back():
    """A point that fails only in double precision gives a NaN difference, which fails the check."""
    def run(points, precision):
        return [GreenError("Singular", "x") if (precision == Precision.DOUBLE and i == 5) else float(i)
                for i in points]

    _, rep = checked(list(range(10)), PrecisionOptions(Precision.SINGLE, 1.0, 5), run)
    assert np.isnan(rep.max) and rep.fallback is not None


@pytest.mark.gpu
def test_transmissions_checked_mixed_on_gpu():
    from systems import clean_bhz_ribbon, oracle_T

    sys_ = clean_bhz_ribbon()
    energies = list(np.linspace(-0.16, 0.16, 12))
    out, rep = sys_.transmissions_checked(energies, PrecisionOptions(Precision.MIXED, 1e-8, 5))
    assert rep.precision == Precision.MIXED and rep.fallback is None
    assert (rep.checked, rep.failed) == (3, 0)  # the sample: indices 0, 5 and 10
    assert rep.max <= 1e-8
    for e, t in zip(energies, out):
        assert abs(t - oracle_T(sys_, sys_.self_energies(e))) <= 1e-8


@pytest.mark.gpu
def test_checked_counts_a_failed_point_and_falls_back_on_gpu():
    from systems import clean_bhz_ribbon, oracle_T

    sys_ = clean_bhz_ribbon()
    energies = list(np.linspace(-0.12, 0.12, 8))
    sigmas = [sys_.self_energies(e) for e in energies]
    bad = LeadSelfEnergies(sigmas[4].energy, [(np.full_like(sl, np.nan), sr) for sl, sr in sigmas[4].blocks])

    def run(idx, precision):
        return sys_.transmissions_with([bad if i == 4 else sigmas[i] for i in idx], [0] * len(idx), precision)

    out, rep = checked(list(range(8)), PrecisionOptions(Precision.MIXED, 1e-8, 3), run)
    assert rep.failed == 1 and rep.checked == 3 and rep.fallback is None, rep  # sample 0, 3, 6
    assert isinstance(out[4], GreenError)
    for i in (0, 1, 2, 3, 5, 6, 7):
        assert abs(out[i] - oracle_T(sys_, sigmas[i])) <= 1e-8
    # Single precision against a tolerance it cannot meet: the whole batch in double precision.
    out, rep = checked(list(range(8)), PrecisionOptions(Precision.SINGLE, 1e-14, 2), run)
    assert rep.fallback is not None and rep.precision == Precision.DOUBLE
    assert isinstance(out[4], GreenError)
    for i in (0, 1, 2, 3, 5, 6, 7):
        assert abs(out[i] - oracle_T(sys_, sigmas[i])) <= 1e-10 * (1 + abs(out[i]))
