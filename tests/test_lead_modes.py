"""Self-energies formed on the GPU from the lead modes (`caroli_lead_modes`,
`caroli_sigma_from_modes`): leads with a scalar coupling h01 = s c 1 (square and cubic leads, the
definite fast path of crates/caroli-green/src/modes.rs:540-710). The host classifies the roots per
transverse mode; the device forms Σ_L, Σ_R, Γ and W_R. The transmissions must equal those with the
host's self-energies."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Precision, Region, bhz, cubic, square


def _hash_disorder(w, norb):
    mask = (1 << 64) - 1

    def term(site):
        k = (site.cell[0] * 7919 + site.cell[1] * 104_729 + site.cell[2] * 15_485_863 + site.sub * 31) & mask
        u = (((k * 6_364_136_223_846_793_005 + 1_442_695_040_888_963_407) & mask) >> 11) / float(1 << 53)
        return np.eye(norb) * (w * (u - 0.5))

    return term


def _square(length=10, width=7, w=1.5):
    m = square()
    return NestedTwoTerminal.from_model(m.with_onsite_term(_hash_disorder(w, 1)), m,
                                        Region.cuboid(m.lattice, [length, width, 0]), 0)


def _cubic(length=8, width=5, depth=5, w=4.0):
    m = cubic()
    return NestedTwoTerminal.from_model(m.with_onsite_term(_hash_disorder(w, 1)), m,
                                        Region.cuboid(m.lattice, [length, width, depth]), 0)


def test_channel_weights_factor_gamma():
    """The open channels and weights the host hands to the device: W_R W_R^† = Γ_R of the host's
    Σ_R, and the roots rebuild the host's Σ_L and Σ_R."""
    sys_ = _square()
    for e in (-2.6, -0.3, 1.4):
        ms = sys_.self_energies_on_device(e)
        hs = sys_.self_energies(e)
        (left, right), = sys_._solvers
        dl, lam_r, cols, w = ms.blocks[0]
        s, c, _, y = right.cell
        sig_r = (s * c) * (y * lam_r) @ y.conj().T
        sig_l = (s * c) * (y * dl) @ y.conj().T
        sl, sr = hs.blocks[0]
        assert np.max(np.abs(sig_l - sl)) < 1e-13 and np.max(np.abs(sig_r - sr)) < 1e-13
        wr = y[:, cols] * w[None, :]
        gam = 1j * (sr - sr.conj().T)
        assert np.max(np.abs(wr @ wr.conj().T - gam)) < 1e-12


def test_general_leads_are_refused():
    m = bhz()
    sys_ = NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [6, 4, 0]), 0)
    assert not sys_.leads_on_device()
    with pytest.raises(ValueError):
        sys_.self_energies_on_device(0.1)


@pytest.mark.gpu
@pytest.mark.parametrize("make,energies", [(_square, [-2.6, -0.3, 0.0, 1.4, 2.0]),
                                           (_cubic, [-2.5, -0.7, 0.4, 1.9])])
def test_device_sigma_transmissions(make, energies):
    sys_ = make()
    host = [sys_.self_energies(e) for e in energies]
    dev = [sys_.self_energies_on_device(e) for e in energies]
    for prec, tol in ((Precision.DOUBLE, 1e-12), (Precision.MIXED, 1e-9)):
        th = np.array(sys_.transmissions_with(host, precision=prec))
        td = np.array(sys_.transmissions_with(dev, precision=prec))
        assert np.max(np.abs(td - th)) <= tol * max(1.0, np.abs(th).max())


@pytest.mark.gpu
def test_device_sigma_at_subband_edge():
    """A clean square ribbon at a subband edge: both paths shift the energy the same way."""
    m = square()
    sys_ = NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [6, 5, 0]), 0)
    theta = sys_._solvers[0][1].cell[2]
    e = float(theta[0] + 2.0)  # μ = 2 for the lowest transverse mode
    th = sys_.transmissions_with([sys_.self_energies(e)])[0]
    td = sys_.transmissions_with([sys_.self_energies_on_device(e)])[0]
    assert abs(td - th) < 1e-10
