"""Failures made on the host and determinism (the failure-detection plan of the path: statuses
instead of traps). Non-finite self-energies in one energy slot of a batch give that point a
GreenError and leave the other points untouched; a batch run twice gives the same bits; devices of
length 1 to 3 (no interior, or one slice that is both lead slices) solve correctly, as the
reference's tests/nested.rs checks them against its RGF."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import GreenError, LeadSelfEnergies, NestedTwoTerminal, Precision, Region, bhz, square


def _hash(w, norb):
    mask = (1 << 64) - 1

    def term(site):
        k = (site.cell[0] * 7919 + site.cell[1] * 104_729 + site.sub * 31) & mask
        u = (((k * 6_364_136_223_846_793_005 + 1_442_695_040_888_963_407) & mask) >> 11) / float(1 << 53)
        return np.eye(norb) * (w * (u - 0.5))

    return term


def _short(model, length, width, w):
    norb = model.lattice.sublattices[0].orbitals
    return NestedTwoTerminal.from_model(model.with_onsite_term(_hash(w, norb)), model,
                                        Region.cuboid(model.lattice, [length, width, 0]), 0)


SHORT = [(square(), 5, 1.5, (-1.1, 0.4)), (bhz(), 4, 0.6, (-0.15, 0.3))]


@pytest.mark.parametrize("length", [1, 2, 3])
@pytest.mark.parametrize("model,width,w,energies", SHORT)
def test_oracle_short_devices(length, model, width, w, energies):
    from oracle import rgf
    from systems import oracle_T

    sys_ = _short(model, length, width, w)
    for e in energies:
        s = sys_.self_energies(e)
        ref = rgf.transmission(sys_.system, e, s.blocks)
        assert abs(oracle_T(sys_, s) - ref) <= 1e-9 * (1 + abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("length", [1, 2, 3])
@pytest.mark.parametrize("model,width,w,energies", SHORT)
def test_gpu_short_devices(length, model, width, w, energies):
    from oracle import rgf

    sys_ = _short(model, length, width, w)
    sig = [sys_.self_energies(e) for e in energies]
    for prec, tol in ((Precision.DOUBLE, 1e-9), (Precision.MIXED, 1e-8)):
        for s, t in zip(sig, sys_.transmissions_with(sig, precision=prec)):
            ref = rgf.transmission(sys_.system, s.energy, s.blocks)
            assert abs(t - ref) <= tol * (1 + abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("prec", [Precision.DOUBLE, Precision.MIXED])
def test_gpu_nonfinite_sigma_fails_alone(bad, prec):
    m = bhz()
    sys_ = NestedTwoTerminal.from_model(m.with_onsite_term(_hash(0.6, 4)), m, Region.cuboid(m.lattice, [12, 8, 0]), 0)
    energies = [-0.12, 0.03, 0.2, 0.35]
    good = [sys_.self_energies(e) for e in energies]
    clean = sys_.transmissions_with(good, precision=prec)
    poisoned = []
    for k, s in enumerate(good):
        if k == 1:
            (sl, sr), rest = s.blocks[0], s.blocks[1:]
            sl = sl.copy()
            sl[0, 0] = bad
            s = LeadSelfEnergies(s.energy, [(sl, sr)] + list(rest))
        poisoned.append(s)
    got = sys_.transmissions_with(poisoned, precision=prec)
    assert isinstance(got[1], GreenError)
    for k in (0, 2, 3):
        assert not isinstance(got[k], GreenError)
        assert abs(got[k] - clean[k]) <= 1e-12 * (1 + abs(clean[k]))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [Precision.DOUBLE, Precision.MIXED])
def test_gpu_batch_is_deterministic(prec):
    from systems import magnetic_bhz

    sys_ = magnetic_bhz(24, 12, configs=2)
    sig = [sys_.self_energies(e) for e in (-0.1, 0.02, 0.13)]
    pairs = [(s, c) for s in sig for c in range(2)]
    a = sys_.transmissions_with([p[0] for p in pairs], [p[1] for p in pairs], precision=prec)
    b = sys_.transmissions_with([p[0] for p in pairs], [p[1] for p in pairs], precision=prec)
    assert np.array_equal(np.array(a), np.array(b))
