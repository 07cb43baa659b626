"""Host lead algebra (CPU): the unit-current propagating modes the scattering matrix uses, the two
eigen paths of the general lead problem (standard eigenproblem of B^-1 A and QZ of the pencil)
agreeing, and the Landauer-Büttiker voltages of a four-terminal device."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Region, bhz, graphene, lead_voltages, square
from caroli_gb300.leads import LeadSolver


def _lead(model, width):
    s = NestedTwoTerminal.from_model(model, model, Region.cuboid(model.lattice, [3, width, 0]), 0)
    b = s.system.blocks[0]
    return LeadSolver(b.right_h00, b.right_h01)


def _current(h01, phi, lam):
    return (1j * (lam * np.vdot(phi, h01 @ phi) - np.conj(lam) * np.vdot(phi, h01.conj().T @ phi))).real


@pytest.mark.parametrize("model,width,energies", [(square(), 7, (-2.5, -0.3, 1.1)), (bhz(), 12, (0.3, 0.6)),
                                                  (graphene(), 6, (-1.2, 0.4))])
def test_modes_carry_unit_current(model, width, energies):
    ls = _lead(model, width)
    for e in energies:
        rm, rl, lm, ll, rest, _ = ls.modes(e)
        assert rm.shape[1] == lm.shape[1] and rm.shape[1] > 0
        for k in range(rm.shape[1]):
            assert abs(_current(ls.h01, rm[:, k], rl[k]) - 1.0) < 1e-9
            assert abs(_current(ls.h01, lm[:, k], ll[k]) + 1.0) < 1e-9
            assert abs(abs(rl[k]) - 1.0) < 1e-6 and abs(abs(ll[k]) - 1.0) < 1e-6
        # The channel count is the rank of Γ_R = i (Σ - Σ^†).
        g = 1j * (rest - rest.conj().T)
        assert np.sum(np.linalg.eigvalsh(0.5 * (g + g.conj().T)) > 1e-9) == rm.shape[1]


def test_standard_and_qz_paths_agree():
    ls = _lead(bhz(), 16)
    assert ls.h01_inv is not None
    for e in (-0.13, 0.02, 0.3, complex(0.05, 1e-5)):
        fast = ls.self_energies(e)
        inv, ls.h01_inv = ls.h01_inv, None
        try:
            slow = ls.self_energies(e)
        finally:
            ls.h01_inv = inv
        for a, b in zip(fast[:2], slow[:2]):
            assert np.max(np.abs(a - b)) < 1e-11 * max(1.0, np.abs(b).max())


def test_graphene_coupling_takes_qz():
    assert _lead(graphene(), 6).h01_inv is None


def test_lead_voltages_four_terminal():
    """A symmetric four-terminal cross, T_pq = t between neighbouring leads and d across: a unit
    current from lead 0 to lead 1 (opposite) with 2 and 3 floating puts the floating leads halfway,
    and the voltages reproduce the imposed currents."""
    t, d = 0.7, 0.2
    # Leads 0, 1 opposite; 2, 3 opposite.
    T = np.array([[0, d, t, t], [d, 0, t, t], [t, t, 0, d], [t, t, d, 0]], float)
    v = lead_voltages(T, [1.0, -1.0, 0.0, 0.0], 1)
    assert abs(v[2] - v[3]) < 1e-12 and abs(v[2] - 0.5 * v[0]) < 1e-12
    # I_p = Σ_q (T_qp V_p - T_pq V_q) reproduces the imposed currents.
    cur = [sum(T[q][p] * v[p] - T[p][q] * v[q] for q in range(4)) for p in range(4)]
    assert np.allclose(cur, [1.0, -1.0, 0.0, 0.0], atol=1e-12)


@pytest.mark.parametrize("width", [4, 10, 16])
def test_reduced_pencil_equals_full_pencil(width):
    """Graphene's rank-deficient coupling: the reduced 2r pencil gives the self-energies of the 2n
    QZ path (narrow ribbons, where the QZ path's eigenvectors are well conditioned)."""
    ls = _lead(graphene(), width)
    assert ls.uv is not None and ls.uv[0].shape[1] < ls.n
    for e in (-2.1, -0.4, 0.1, 0.45, 1.3):
        sl1, sr1 = ls._general(e)
        sl2, sr2 = ls._reduced(e)
        assert np.abs(sl1 - sl2).max() < 1e-11 and np.abs(sr1 - sr2).max() < 1e-11, e


@pytest.mark.parametrize("width", [24, 40, 100])
def test_reduced_pencil_solves_the_dyson_equation(width):
    """Σ_R = h01 (E - h00 - Σ_R)^-1 h01^† and Σ_L = h01^† (E - h00 - Σ_L)^-1 h01 to 1e-11, where the
    edge states make the evanescent eigenvectors nearly parallel (Schur bases)."""
    ls = _lead(graphene(), width)
    eye = np.eye(ls.n)
    for e in (-0.4, 0.1, 0.45):
        sl, sr = ls._reduced(e)
        rr = sr - ls.h01 @ np.linalg.solve(e * eye - ls.h00 - sr, ls.h01.conj().T)
        rl = sl - ls.h01.conj().T @ np.linalg.solve(e * eye - ls.h00 - sl, ls.h01)
        assert max(np.abs(rr).max(), np.abs(rl).max()) < 1e-11, e


def test_self_energies_many_matches_serial_and_keeps_failures_in_place(monkeypatch):
    """Σ of many energies on host threads (as the reference's parallel map over energies,
    nested.rs:622-626) equals the serial Σ bit for bit; with errors=True a failing energy (made to
    fail on the host) is a GreenError in its place, the others unaffected; without it, it raises."""
    from caroli_gb300 import GreenError

    m = bhz()
    s = NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [6, 12, 0]), 0)
    es = list(np.linspace(-0.3, 0.3, 9))
    serial = [s.self_energies(e) for e in es]
    par = s.self_energies_many(es, threads=4)
    for a, b in zip(serial, par):
        assert a.energy == b.energy
        for (al, ar), (bl, br) in zip(a.blocks, b.blocks):
            assert np.array_equal(al, bl) and np.array_equal(ar, br)
    orig = s.self_energies

    def flaky(e):
        if e == es[3]:
            raise GreenError("Eigen", "made to fail")
        return orig(e)

    monkeypatch.setattr(s, "self_energies", flaky)
    out = s.self_energies_many(es, threads=4, errors=True)
    assert isinstance(out[3], GreenError)
    for i, o in enumerate(out):
        if i != 3:
            assert not isinstance(o, GreenError)
            assert np.array_equal(o.blocks[0][0], serial[i].blocks[0][0])
    with pytest.raises(GreenError):
        s.self_energies_many(es, threads=4)


def test_lead_modes_are_per_thread():
    """The modes of the reduced pencil (graphene's zigzag lead) computed on several threads at
    once equal those computed one after another: each thread keeps its own last modes."""
    from concurrent.futures import ThreadPoolExecutor

    ls = _lead(graphene(), 24)
    assert ls.uv is not None
    es = [-1.2, -0.7, -0.2, 0.4, 0.9, 1.3]
    serial = [ls.modes(e) for e in es]
    with ThreadPoolExecutor(max_workers=4) as pool:
        par = list(pool.map(ls.modes, es))
    for a, b in zip(serial, par):
        assert a[0].shape == b[0].shape and a[2].shape == b[2].shape
        for x, y in zip(a[:5], b[:5]):
            assert np.array_equal(x, y)


def test_transmissions_places_failed_energies(monkeypatch):
    """NestedTwoTerminal.transmissions (nested.rs:622-626): an energy whose self-energies fail is a
    GreenError in its place and the others are solved in one batch, in order (the batch call is
    replaced by a stand-in that returns each energy, so no GPU is needed)."""
    from caroli_gb300 import GreenError

    m = bhz()
    s = NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [6, 12, 0]), 0)
    es = [-0.2, -0.1, 0.0, 0.1, 0.2]
    orig = s.self_energies

    def flaky(e):
        if e == 0.0:
            raise GreenError("Eigen", "made to fail")
        return orig(e)

    seen = {}

    def batch(sigmas, configs, precision):
        seen["configs"] = list(configs)
        return [sg.energy for sg in sigmas]

    monkeypatch.setattr(s, "self_energies", flaky)
    monkeypatch.setattr(s, "transmissions_with", batch)
    out = s.transmissions(es, config=3)
    assert isinstance(out[2], GreenError)
    assert [out[i] for i in (0, 1, 3, 4)] == [es[i] for i in (0, 1, 3, 4)]
    assert seen["configs"] == [3, 3, 3, 3]
