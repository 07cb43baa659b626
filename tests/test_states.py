"""Scattering states, bond currents and densities: the GPU states against sparse direct solves, and
the observables against the lesser Green's function, on the samples of the reference's own test
(`crates/caroli-keldysh/tests/nested_states.rs`: disordered square, BHZ, graphene, a square sample
in a magnetic field; occupations and bond currents to 1e-10, the currents through every
cross-section equal to T (f_L - f_R) to 1e-9)."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Region, ScatteringStates, bhz, graphene, square
from caroli_gb300.states import bond_currents, site_densities


def _hash_disorder(w, norb):
    """Reproducible on-site disorder w (u - 0.5) per site, u from a 64-bit LCG step of a hash of
    the site (the fixture of nested_states.rs:33-41)."""
    mask = (1 << 64) - 1

    def term(site):
        k = (site.cell[0] * 7919 + site.cell[1] * 104_729 + site.sub * 31) & mask
        u = (((k * 6_364_136_223_846_793_005 + 1_442_695_040_888_963_407) & mask) >> 11) / float(1 << 53)
        return np.eye(norb) * (w * (u - 0.5))

    return term


def _field(b):
    """Peierls phase of a uniform field b in the gauge A = (-b y, 0): exp(-i b y dx) on a hop."""

    def term(frm, to, t):
        dx = to.cell[0] - frm.cell[0]
        return None if dx == 0 else t * np.exp(-1j * b * frm.cell[1] * dx)

    return term


def _sample(name):
    if name == "square":
        m = square()
        return m.with_onsite_term(_hash_disorder(1.5, 1)), m, Region.cuboid(m.lattice, [10, 7, 0]), [-2.6, -0.3, 0.0, 1.4]
    if name == "bhz":
        m = bhz()
        return m.with_onsite_term(_hash_disorder(0.6, 4)), m, Region.cuboid(m.lattice, [8, 6, 0]), [-0.15, 0.03, 0.35]
    if name == "graphene":
        m = graphene()
        return m.with_onsite_term(_hash_disorder(0.8, 1)), m, Region.cuboid(m.lattice, [7, 5, 0]), [-1.3, 0.45, 1.1]
    if name == "field":
        m = square()
        lead = m.with_hopping_term(_field(0.15))
        dev = m.with_onsite_term(_hash_disorder(1.0, 1)).with_hopping_term(_field(0.15))
        return dev, lead, Region.cuboid(m.lattice, [9, 8, 0]), [-3.3, -1.1, 0.6]
    raise KeyError(name)


SAMPLES = ["square", "bhz", "graphene", "field"]


def _system(name):
    dev, lead, region, energies = _sample(name)
    return NestedTwoTerminal.from_model(dev, lead, region, 0), energies


def _oracle_states(sys_, sigma, config=0):
    from oracle import states as ost

    psi = ost.scattering_states(sys_.system, sigma.energy, sigma.blocks, sigma.w_left(), sigma.w_right(), config)
    return ScatteringStates(sigma.energy, psi, config)


def _through(currents, x, axis=0):
    """Net current from the sites at cell[axis] <= x to those beyond."""
    tot = 0.0
    for b in currents:
        a, c = b.from_.cell[axis] <= x, b.to.cell[axis] <= x
        tot += b.current if (a and not c) else (-b.current if (c and not a) else 0.0)
    return tot


def _check_observables(sys_, sigma, states, t, tol=1e-10):
    """Occupations, bond currents and (BHZ) spin densities against the lesser Green's function;
    cross-section currents against T (f_L - f_R)."""
    from oracle import states as ost

    s = sys_.system
    for f in ([1.0, 0.0], [0.3, 0.8]):
        occ = states.occupation(f)
        ref = ost.lesser_occupation(s, sigma.energy, sigma.blocks, f, states.config)
        assert np.max(np.abs(occ - ref)) < tol
        cur = sys_.bond_currents(states, f)
        ref_c = ost.lesser_currents(s, sigma.energy, sigma.blocks, f, states.config)
        idx = {(sys_.sites.index(b.from_), sys_.sites.index(b.to)): b.current for b in cur}
        assert set(idx) == set(ref_c)
        assert max(abs(idx[k] - ref_c[k]) for k in ref_c) < tol
        xs = sorted({site.cell[0] for site in sys_.sites})
        for x in xs[:-1]:
            assert abs(_through(cur, x) - t * (f[0] - f[1])) < 1e-9
        norb = int(s.site_orbitals[0])
        if norb == 4:
            up = np.diag([1.0, 1.0, 0.0, 0.0]).astype(np.complex128)
            dens = sys_.site_densities(states, f, up)
            ref_d = ost.lesser_site_densities(s, sigma.energy, sigma.blocks, f, states.config, up)
            assert np.max(np.abs(dens - ref_d)) < tol
            sz = np.diag([1.0, 1.0, -1.0, -1.0]).astype(np.complex128)
            oc = {(sys_.sites.index(b.from_), sys_.sites.index(b.to)): b.current for b in sys_.operator_currents(states, f, sz)}
            ref_o = ost.lesser_currents(s, sigma.energy, sigma.blocks, f, states.config, sz)
            assert max(abs(oc[k] - ref_o[k]) for k in ref_o) < tol
        dens = sys_.site_densities(states, f)
        ref_d = ost.lesser_site_densities(s, sigma.energy, sigma.blocks, f, states.config)
        assert np.max(np.abs(dens - ref_d)) < tol


# -- CPU: the host observables on the oracle's states ---------------------------------------------
@pytest.mark.parametrize("name", SAMPLES)
def test_observables_of_oracle_states(name):
    from systems import oracle_T

    sys_, energies = _system(name)
    e = energies[1]
    sigma = sys_.self_energies(e)
    states = _oracle_states(sys_, sigma)
    _check_observables(sys_, sigma, states, oracle_T(sys_, sigma))


def test_states_without_region_name_sites_by_index():
    sys_, energies = _system("square")
    sigma = sys_.self_energies(energies[0])
    states = _oracle_states(sys_, sigma)
    cur = bond_currents(sys_.system, states, [1.0, 0.0])
    assert all(isinstance(b.from_, int) and b.from_ < b.to for b in cur)
    assert len(site_densities(sys_.system, states, [1.0, 1.0])) == len(sys_.sites)
    with pytest.raises(ValueError):
        states.occupation([1.0])


# -- GPU ------------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("name", SAMPLES)
def test_gpu_states_match_direct_solve(name):
    sys_, energies = _system(name)
    sigmas = [sys_.self_energies(e) for e in energies]
    got = sys_.scattering_states_batch(sigmas)
    t = sys_.transmissions_with(sigmas)
    for sigma, st, te in zip(sigmas, got, t):
        assert isinstance(st, ScatteringStates)
        ref = _oracle_states(sys_, sigma)
        for a, b in zip(st.leads, ref.leads):
            assert a.shape == b.shape
            scale = max(1.0, np.max(np.abs(b)))
            assert np.max(np.abs(a - b)) <= 1e-9 * scale
        _check_observables(sys_, sigma, st, te)


@pytest.mark.gpu
def test_gpu_states_magnetic_configs_batch():
    """Several disorder configurations and energies in one call (two spin blocks broken by the
    exchange), against the direct solve."""
    from systems import magnetic_bhz

    sys_ = magnetic_bhz(24, 12, configs=3)
    sigmas = [sys_.self_energies(e) for e in (-0.05, 0.12)]
    pairs = [(s, c) for s in sigmas for c in range(3)]
    got = sys_.scattering_states_batch([p[0] for p in pairs], [p[1] for p in pairs])
    for (sigma, c), st in zip(pairs, got):
        ref = _oracle_states(sys_, sigma, c)
        for a, b in zip(st.leads, ref.leads):
            assert np.max(np.abs(a - b)) <= 1e-9 * max(1.0, np.max(np.abs(b)))


@pytest.mark.gpu
def test_gpu_states_larger_ribbon_current_conservation():
    """A 96 x 48 magnetic BHZ ribbon (about 18k orbitals): states against the direct solve, and the
    cross-section currents against the transmission."""
    from systems import magnetic_bhz

    sys_ = magnetic_bhz(96, 48, configs=1)
    sigma = sys_.self_energies(0.08)
    st = sys_.scattering_states_with(sigma)
    ref = _oracle_states(sys_, sigma)
    for a, b in zip(st.leads, ref.leads):
        assert np.max(np.abs(a - b)) <= 1e-9 * max(1.0, np.max(np.abs(b)))
    t = sys_.transmissions_with([sigma])[0]
    cur = sys_.bond_currents(st, [1.0, 0.0])
    for x in (0, 30, 94):
        assert abs(_through(cur, x) - t) < 1e-9


@pytest.mark.gpu
def test_gpu_states_invalid_arguments():
    from caroli_gb300 import _native

    sys_, energies = _system("square")
    sigma = sys_.self_energies(energies[0])
    plan = sys_.plan()
    slot = sys_._slot(sigma)
    outs, st = plan.scattering_states([], [], [], [], sys_.system.n)
    assert outs == [] and len(st) == 0
    wl = [np.zeros((len(b.left), len(b.left) + 1), np.complex128) for b in sys_.system.blocks]
    with pytest.raises(_native.NativeError):
        plan.scattering_states([slot], [0], [wl], [sigma.w_right()], sys_.system.n)
    with pytest.raises(_native.NativeError):
        plan.scattering_states([slot], [5], [sigma.w_left()], [sigma.w_right()], sys_.system.n)


# -- transmission eigenvalues (nested.rs:753-780; the reference's test tests/nested.rs:131-156) ----
@pytest.mark.gpu
def test_gpu_transmission_eigenvalues_and_shot_noise():
    m = square()
    region = Region.cuboid(m.lattice, [12, 7, 0])
    dirty = NestedTwoTerminal.from_model(m.with_onsite_term(_hash_disorder(2.0, 1)), m, region, 0)
    clean = NestedTwoTerminal.from_model(m, m, region, 0)
    barrier = m.with_onsite_term(lambda s: np.eye(1) * 40.0 if s.cell[0] == 6 else None)
    tunnel = NestedTwoTerminal.from_model(barrier, m, region, 0)
    for e in (-2.3, -0.7, 0.9):
        taus = dirty.transmission_eigenvalues(e)
        t = dirty.transmission(e)
        assert abs(taus.sum() - t) < 1e-10
        assert np.all((taus >= -1e-10) & (taus <= 1.0 + 1e-10))
        perfect = clean.transmission_eigenvalues(e)
        assert np.all(np.abs(perfect - 1.0) < 1e-9) and abs(clean.fano_factor(e)) < 1e-8
        assert tunnel.fano_factor(e) > 0.99
    # Against the oracle's G_LR on a BHZ ribbon (two blocks): the same eigenvalues.
    from oracle import states as ost

    b = bhz()
    sys_ = NestedTwoTerminal.from_model(b.with_onsite_term(_hash_disorder(0.6, 4)), b,
                                        Region.cuboid(b.lattice, [8, 6, 0]), 0)
    sigma = sys_.self_energies(0.03)
    taus = sys_.transmission_eigenvalues(0.03)
    psi = ost.scattering_states(sys_.system, 0.03, sigma.blocks, sigma.w_left(), sigma.w_right())[1]
    ref = []
    c0 = 0
    for blk, wl, wr in zip(sys_.system.blocks, sigma.w_left(), sigma.w_right()):
        tm = wl.conj().T @ psi[blk.left, c0:c0 + wr.shape[1]]
        ref.extend(np.linalg.svd(tm, compute_uv=False) ** 2)
        c0 += wr.shape[1]
    assert np.max(np.abs(taus - np.sort(ref)[::-1])) < 1e-10
