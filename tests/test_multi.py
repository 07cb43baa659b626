"""Multi-terminal transmissions (NestedMultiTerminal): the four-terminal square cross of the
reference's benchmark against its published T_pq, crosses of BHZ (two spin blocks) and graphene
against a dense inverse of the whole device (MultiTerminal), and two leads against the
two-terminal solver (crates/caroli-green/src/multi.rs:244-276)."""
from __future__ import annotations

import numpy as np
import pytest

from systems import bench_golden, cross_problem, cross_system


def _off_diagonal(t):
    n = len(t)
    return np.array([t[p][q] for p in range(n) for q in range(n) if q != p])


def _full_leads(dev, clean, region, interfaces):
    from caroli_gb300 import attach_leads

    return attach_leads(clean, region, interfaces)


# -- CPU: the oracle and the host logic ------------------------------------------------------------
def test_dense_oracle_reproduces_published_cross():
    """The dense oracle on the W = 32 square cross (2 048 sites) at three of the eight published
    energies: the reference's T_pq to 1e-10."""
    from oracle import multi as om

    g = bench_golden()["caroli/square-cross/32"]
    runs = np.array(g["runs"])
    dev, clean, region, interfaces = cross_problem(32)
    s = cross_system(32)
    leads = _full_leads(dev, clean, region, interfaces)
    for k in (0, 4, 7):
        t = om.transmissions(s.system, leads, g["energies"][k])
        assert np.max(np.abs(_off_diagonal(t) - runs[0][12 * k:12 * k + 12])) < 1e-10


def test_blocks_and_restricted_leads():
    """BHZ cross: two spin blocks, each with the part of every lead it reaches; the dense oracle
    on the blocks' restricted leads adds up to the oracle on the full leads."""
    from oracle import multi as om

    s = cross_system(8, model="bhz", seed=3, anderson=0.5)
    assert s.block_count() == 2 and s.lead_count() == 4
    dev, clean, region, interfaces = cross_problem(8, model="bhz", seed=3, anderson=0.5)
    full = om.transmissions(s.system, _full_leads(dev, clean, region, interfaces), 0.05)
    parts = np.zeros((4, 4))
    for b, leads in enumerate(s.block_leads):
        assert all(l is not None for l in leads)
        rows = s.system.block_rows(b)
        for l in leads:
            assert np.all(np.isin(l.orbitals, rows))
        parts += om.transmissions(s.system, leads, 0.05)
    assert np.max(np.abs(parts - full)) < 1e-10


def test_lead_voltages_two_terminal():
    from caroli_gb300 import lead_voltages

    v = lead_voltages([[0.0, 2.5], [2.5, 0.0]], [1.0, -1.0], 1)
    assert abs(v[0] - 1.0 / 2.5) < 1e-14 and v[1] == 0.0
    with pytest.raises(ValueError):
        lead_voltages([[0.0, 1.0], [1.0, 0.0]], [1.0, 0.0], 1)


# -- GPU ------------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("width", [32, 64])
def test_gpu_square_cross_matches_published(width):
    """Every T_pq of the benchmark's square cross at its eight energies, FP64, against the
    reference's published values (its runs agree among themselves to ~1e-11)."""
    g = bench_golden()[f"caroli/square-cross/{width}"]
    runs = np.array(g["runs"])
    s = cross_system(width)
    got = s.transmissions_batch(g["energies"])
    for k, t in enumerate(got):
        assert np.max(np.abs(_off_diagonal(t) - runs[0][12 * k:12 * k + 12])) < 1e-8


@pytest.mark.gpu
def test_gpu_square_cross_single_precision():
    from caroli_gb300 import Precision

    g = bench_golden()["caroli/square-cross/32"]
    runs = np.array(g["runs"])
    s = cross_system(32)
    got = s.transmissions_batch(g["energies"], precision=Precision.SINGLE)
    for k, t in enumerate(got):
        assert np.max(np.abs(_off_diagonal(t) - runs[0][12 * k:12 * k + 12])) < 1e-2


@pytest.mark.gpu
@pytest.mark.parametrize("model,seed,w", [("bhz", 3, 0.5), ("graphene", 4, 1.0)])
def test_gpu_cross_against_dense_oracle(model, seed, w):
    from oracle import multi as om

    s = cross_system(12, model=model, seed=seed, anderson=w)
    dev, clean, region, interfaces = cross_problem(12, model=model, seed=seed, anderson=w)
    leads = _full_leads(dev, clean, region, interfaces)
    energies = [-0.2, 0.05, 0.3] if model == "bhz" else [-1.1, 0.4, 1.3]
    got = s.transmissions_batch(energies)
    for e, t in zip(energies, got):
        ref = om.transmissions(s.system, leads, e)
        assert np.max(np.abs(t - ref)) < 1e-9 * (1.0 + np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_two_leads_equal_two_terminal():
    """A disordered square ribbon with leads on its first and last slices: T_01 = T_10 = the
    two-terminal T (multi.rs:244-276)."""
    from caroli_gb300 import Interface, NestedMultiTerminal, NestedTwoTerminal, Region, square

    clean = square()
    pot = {(2, 1): 0.7, (3, 2): -0.4}
    dev = clean.with_onsite_term(lambda s: np.eye(1) * pot[s.cell[:2]] if s.cell[:2] in pot else None)
    region = Region.cuboid(clean.lattice, [6, 4, 0])
    sl = region.slices(0)
    multi = NestedMultiTerminal.from_model(dev, clean, region, [Interface(sl[0], (-1, 0, 0)),
                                                                Interface(sl[5], (1, 0, 0))])
    two = NestedTwoTerminal.from_model(dev, clean, region, 0)
    for e in (-1.3, 0.2, 0.9):
        t2 = two.transmission(e)
        tm = multi.transmissions(e)
        assert abs(tm[0][1] - t2) < 1e-10 and abs(tm[1][0] - t2) < 1e-10


@pytest.mark.gpu
def test_gpu_multi_configs_and_errors():
    from caroli_gb300 import NestedMultiTerminal, Precision, _native
    from caroli_gb300.disorder import ScalarPotential, bench_disorder

    dev, clean, region, interfaces = cross_problem(12)
    devs = []
    for c in range(3):
        pot = bench_disorder(5 + c, 12, 18, 18, 1, 1.0)
        devs.append(clean.with_onsite_term(ScalarPotential(pot, 18, 1, 1, origin=(-3, -3))))
    multi = NestedMultiTerminal.from_models(devs, clean, region, interfaces)
    energies = [-1.7, 0.1, 0.9]
    pairs = [(e, c) for e in energies for c in range(3)]
    got = multi.transmissions_batch([p[0] for p in pairs], [p[1] for p in pairs])
    for (e, c), t in zip(pairs, got):
        one = NestedMultiTerminal.from_model(devs[c], clean, region, interfaces)
        assert np.max(np.abs(t - one.transmissions(e))) < 1e-11
    sig = multi.self_energies(0.1)
    slot = multi._slot(sig)
    with pytest.raises(_native.NativeError):
        multi.plan().multi_solve([slot], [0], 7, 4)  # no such precision
    with pytest.raises(_native.NativeError):
        multi.plan().solve([slot], [0], int(Precision.DOUBLE))
    t, st = multi.plan().multi_solve([], [], int(Precision.DOUBLE), 4)
    assert t.shape == (0, 4, 4)


# -- multi-terminal scattering states ------------------------------------------------------------
def _arm_current(currents, lead):
    """Net bond current from the centre of a cross into the arm of `lead` (left, right, bottom,
    top): across x = 0 / x = w - 1 / y = 0 / y = w - 1."""
    tot = 0.0
    for b in currents:
        a, c = b.from_.cell, b.to.cell
        inside = {0: lambda s: s[0] < 0, 1: lambda s: s[0] >= W_ARM, 2: lambda s: s[1] < 0,
                  3: lambda s: s[1] >= W_ARM}[lead]
        if inside(c) and not inside(a):
            tot += b.current
        elif inside(a) and not inside(c):
            tot -= b.current
    return tot


W_ARM = 12


@pytest.mark.gpu
@pytest.mark.parametrize("model,seed,w,energy", [("square", 5, 1.0, 0.9), ("bhz", 3, 0.5, 0.05)])
def test_gpu_multi_states_spectral_and_currents(model, seed, w, energy):
    """ψ_p ψ_p^† = G Γ_p G^† of the dense oracle for every lead, and with lead p filled (f = e_p)
    the current into the arm of lead q equals T_qp."""
    from oracle import multi as om

    s = cross_system(W_ARM, model=model, seed=seed, anderson=w)
    dev, clean, region, interfaces = cross_problem(W_ARM, model=model, seed=seed, anderson=w)
    leads = _full_leads(dev, clean, region, interfaces)
    st = s.scattering_states(energy)
    ref = om.spectral(s.system, leads, energy)
    for psi, g in zip(st.leads, ref):
        assert np.max(np.abs(psi @ psi.conj().T - g)) <= 1e-9 * max(1.0, np.abs(g).max())
    t = s.transmissions(energy)
    for p in range(4):
        f = [1.0 if k == p else 0.0 for k in range(4)]
        cur = s.bond_currents(st, f)
        for q in range(4):
            if q != p:
                assert abs(_arm_current(cur, q) - t[q][p]) < 1e-9


# -- sector transmissions --------------------------------------------------------------------------
def _spin_labels(s):
    tags = [[[0, 0, 1, 1][k] for k in kinds] for kinds in s.orbital_kinds]
    labels = [(p, a) for p in range(4) for a in (0, 1)]
    return labels, tags


def test_sector_oracle_adds_up_to_leads():
    """Summed over the sectors of both leads, the oracle's sector transmissions are its T_pq."""
    from oracle import multi as om

    s = cross_system(8, model="bhz", seed=3, anderson=0.5)
    dev, clean, region, interfaces = cross_problem(8, model="bhz", seed=3, anderson=0.5)
    leads = _full_leads(dev, clean, region, interfaces)
    labels, tags = _spin_labels(s)
    ts = om.sector_transmissions(s.system, leads, 0.05, labels, tags)
    t = om.transmissions(s.system, leads, 0.05)
    folded = ts.reshape(4, 2, 4, 2).sum(axis=(1, 3))
    assert np.max(np.abs(folded - t)) < 1e-10


@pytest.mark.gpu
def test_gpu_spin_sector_transmissions():
    """BHZ cross with spin-conserving disorder, sectors [0, 0, 1, 1] (spin up, spin down) on every
    lead: against the dense oracle, no spin flips, and the sum over sectors equals T_pq."""
    from oracle import multi as om

    s = cross_system(W_ARM, model="bhz", seed=3, anderson=0.5)
    dev, clean, region, interfaces = cross_problem(W_ARM, model="bhz", seed=3, anderson=0.5)
    leads = _full_leads(dev, clean, region, interfaces)
    for e in (-0.2, 0.05):
        labels, t = s.sector_transmissions(e, [[0, 0, 1, 1]] * 4)
        ref_labels, tags = _spin_labels(s)
        assert labels == ref_labels
        ref = om.sector_transmissions(s.system, leads, e, labels, tags)
        assert np.max(np.abs(t - ref)) < 1e-9 * (1.0 + np.abs(ref).max())
        spin = np.array([a for _, a in labels])
        assert np.max(np.abs(t[spin[:, None] != spin[None, :]])) < 1e-10
        folded = t.reshape(4, 2, 4, 2).sum(axis=(1, 3))
        assert np.max(np.abs(folded - s.transmissions(e))) < 1e-9
    with pytest.raises(ValueError):
        s.sector_transmissions(0.05, [[0, 0, 1, 1]] * 3)


@pytest.mark.gpu
@pytest.mark.parametrize("model,seed,w,energies", [("square", 5, 1.0, (-2.5, 0.1, 1.7)),
                                                   ("bhz", 3, 0.5, (-0.2, 0.05, 0.3))])
def test_gpu_multi_mixed_matches_double(model, seed, w, energies):
    """CAROLI_MIXED T_pq (few channels per lead: refined in FP64) against FP64: ≤ 1e-8."""
    from caroli_gb300 import Precision

    s = cross_system(8, model=model, seed=seed, anderson=w)
    td = s.transmissions_batch(list(energies))
    tm = s.transmissions_batch(list(energies), precision=Precision.MIXED)
    for a, b in zip(td, tm):
        assert np.max(np.abs(a - b)) < 1e-8


@pytest.mark.gpu
def test_gpu_multi_mixed_routes_many_channels():
    """The W = 32 square cross has up to 128 sources per block solve: CAROLI_MIXED takes the FP64
    path for those and still gives the published values."""
    from caroli_gb300 import Precision

    g = bench_golden()["caroli/square-cross/32"]
    runs = np.array(g["runs"])
    s = cross_system(32)
    got = s.transmissions_batch(g["energies"], precision=Precision.MIXED)
    for k, t in enumerate(got):
        assert np.max(np.abs(_off_diagonal(t) - runs[0][12 * k:12 * k + 12])) < 1e-8
