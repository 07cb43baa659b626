"""Known answers of the reference's own tests: quantum Hall plateaus of a disordered ribbon in a
field and gauge invariance (crates/caroli-green/tests/magnetic.rs:33-70), and the analytic
transmissions of a chain (crates/caroli-green/src/two_terminal.rs:436-466): T = 1 for a clean chain,
1 / (1 + (u / (2 sin k))^2) through one impurity u at E = -2 cos k. The CPU suite checks the
oracle against them; the GPU tests check the CUDA path against them and against the oracle."""
from __future__ import annotations

import math

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Region, square
from caroli_gb300.model import landau_x


def _hash2(w):
    """On-site disorder of magnetic.rs:22-30 (cell hash, no sublattice term)."""
    mask = (1 << 64) - 1

    def term(site):
        k = (site.cell[0] * 7919 + site.cell[1] * 104_729) & mask
        u = (((k * 6_364_136_223_846_793_005 + 1_442_695_040_888_963_407) & mask) >> 11) / float(1 << 53)
        return np.eye(1) * (w * (u - 0.5))

    return term


def _qh(b=0.1, w=0.2, length=40, width=60, y0=0.0):
    phase = (lambda ri, rj: -b * 0.5 * (ri[1] + rj[1] - 2 * y0) * (ri[0] - rj[0])) if y0 else landau_x(b)
    clean = square().with_peierls(phase)
    dev = square().with_onsite_term(_hash2(w)).with_peierls(phase)
    return NestedTwoTerminal.from_model(dev, clean, Region.cuboid(clean.lattice, [length, width, 0]), 0)


PLATEAUS = [(-3.8, 1.0), (-3.6, 2.0), (-3.4, 3.0)]


def _chain(u=None, length=9):
    m = square()
    dev = m if u is None else m.with_onsite_term(lambda s: np.eye(1) * u if s.cell[0] == length // 2 else None)
    return NestedTwoTerminal.from_model(dev, m, Region.cuboid(m.lattice, [length, 1, 0]), 0)


def _chain_answer(e, u):
    k = math.acos(-e / 2.0)
    return 1.0 / (1.0 + (u / (2.0 * math.sin(k))) ** 2)


# -- CPU: the oracle ------------------------------------------------------------------------------
def test_oracle_quantum_hall_plateaus():
    from systems import oracle_T

    sys_ = _qh()
    for e, plateau in PLATEAUS:
        assert abs(oracle_T(sys_, sys_.self_energies(e)) - plateau) < 1e-6


def test_oracle_chain():
    from systems import oracle_T

    clean, dirty = _chain(), _chain(0.7)
    for e in (-1.5, -0.4, 0.3, 1.2):
        assert abs(oracle_T(clean, clean.self_energies(e)) - 1.0) < 1e-12
        assert abs(oracle_T(dirty, dirty.self_energies(e)) - _chain_answer(e, 0.7)) < 1e-12


# -- GPU ------------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_quantum_hall_plateaus_and_gauge():
    from systems import oracle_T

    sys_ = _qh()
    shifted = _qh(y0=3.7)
    sig = [sys_.self_energies(e) for e, _ in PLATEAUS]
    t = sys_.transmissions_with(sig)
    tm = sys_.transmissions_with(sig, precision=2)
    ts = shifted.transmissions([e for e, _ in PLATEAUS])
    for (e, plateau), a, m, b, s in zip(PLATEAUS, t, tm, ts, sig):
        assert abs(a - plateau) < 1e-6
        assert abs(a - oracle_T(sys_, s)) < 1e-9
        assert abs(m - a) < 1e-8
        assert abs(b - a) < 1e-9  # gauge invariance


@pytest.mark.gpu
def test_gpu_chain():
    clean, dirty = _chain(), _chain(0.7)
    energies = [-1.5, -0.4, 0.3, 1.2]
    for prec in (0, 2):
        tc = clean.transmissions(energies, precision=prec)
        td = dirty.transmissions(energies, precision=prec)
        for e, a, b in zip(energies, tc, td):
            assert abs(a - 1.0) < 1e-10
            assert abs(b - _chain_answer(e, 0.7)) < 1e-10


# -- the thesis' magnetic-impurity conductances (ti_conductance_disorder.rs) ------------------------
def _thesis_golden():
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ti_cond2t_disorder.json")) as f:
        return json.load(f)["cases"]


CASES = ["ti-cond2t-same-g", "ti-cond2t-isotropic", "ti-cond2t-opposite-g"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_thesis_conductance(case):
    """RGF oracle, Σ at E + 1e-5 i and the Re Γ trace: the thesis' values to 1e-9."""
    from oracle import rgf
    from systems import thesis_ribbon

    g = _thesis_golden()[case]
    for iu, u in enumerate(g["couplings"]):
        sys_ = thesis_ribbon(case, u)
        for ie, e in enumerate(g["energies"]):
            sig = sys_.self_energies_broadened(e, 1e-5)
            t = rgf.transmission(sys_.system, e, sig.blocks, gamma=lambda m: np.real(m).astype(complex))
            assert abs(t - g["cond"][iu + 3 * ie]) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_thesis_conductance(case):
    from systems import thesis_ribbon

    g = _thesis_golden()[case]
    for iu, u in enumerate(g["couplings"]):
        sys_ = thesis_ribbon(case, u)
        for ie, e in enumerate(g["energies"]):
            t = sys_.transmission_thesis(sys_.self_energies_broadened(e, 1e-5))
            assert abs(t - g["cond"][iu + 3 * ie]) < 1e-9
