"""dT/dV (every on-site potential) and dT/dJ (exchange coupling) of the adjoint path against
central finite differences of the oracle's FP64 transmission (step 1e-6), as the gradient workload
asks; the reference has no derivative code of its own."""
import numpy as np
import pytest

from systems import gradient_bhz, oracle_T

pytestmark = pytest.mark.gpu


def _diag_index(system, a):
    lo, hi = system.row_ptr[a], system.row_ptr[a + 1]
    q = lo + np.nonzero(system.cols[lo:hi] == a)[0]
    assert len(q) == 1
    return int(q[0])


def _oracle_T_with(sys_, sigma, vals):
    from oracle import Oracle

    if not hasattr(sys_, "_oracle"):
        sys_._oracle = Oracle(sys_.system)
    return sys_._oracle.transmission(sigma.energy, vals, sigma.blocks)


@pytest.mark.parametrize("energy", [-0.12, 0.05])
def test_gradient_matches_finite_differences(energy):
    sys_, derivs = gradient_bhz(20, 10, configs=2)
    sys_.set_parameter_derivatives(derivs)
    sigma = sys_.self_energies(energy)
    t, st, dv, dp = sys_.transmissions_with_grad([sigma, sigma], [0, 1])
    assert (st == 0).all(), st
    rng = np.random.default_rng(7)
    h = 1e-6
    for c in range(2):
        base = sys_.system.values[c]
        assert abs(t[c] - _oracle_T_with(sys_, sigma, base)) < 1e-8
        for a in rng.choice(sys_.system.n, size=12, replace=False):
            q = _diag_index(sys_.system, a)
            vp, vm = base.copy(), base.copy()
            vp[q] += h
            vm[q] -= h
            fd = (_oracle_T_with(sys_, sigma, vp) - _oracle_T_with(sys_, sigma, vm)) / (2 * h)
            assert abs(dv[c, a] - fd) <= 1e-4 * abs(fd) + 1e-5, (c, a, dv[c, a], fd)
        d = derivs[c][0]
        fdj = (_oracle_T_with(sys_, sigma, base + h * d) - _oracle_T_with(sys_, sigma, base - h * d)) / (2 * h)
        assert abs(dp[c, 0] - fdj) <= 1e-4 * abs(fdj) + 1e-5, (c, dp[c, 0], fdj)


def test_gradient_sums_to_the_uniform_shift():
    """A uniform potential V on every orbital is an energy shift: Σ_a dT/dV_a = -dT/dE at fixed
    self-energies (the leads do not move), checked against the oracle."""
    sys_, derivs = gradient_bhz(16, 8, configs=1)
    sigma = sys_.self_energies(-0.08)
    t, st, dv, dp = sys_.transmissions_with_grad([sigma], [0])
    assert st[0] == 0
    h = 1e-6
    base = sys_.system.values[0]
    vp, vm = base.copy(), base.copy()
    for a in range(sys_.system.n):
        q = _diag_index(sys_.system, a)
        vp[q] += h
        vm[q] -= h
    fd = (_oracle_T_with(sys_, sigma, vp) - _oracle_T_with(sys_, sigma, vm)) / (2 * h)
    assert abs(dv[0].sum() - fd) <= 1e-4 * abs(fd) + 1e-5


@pytest.mark.slow
def test_gradient_workload_64_sites():
    """The gradient workload (BHZ 100 x 40, Anderson W = 0.02 + magnetic c = 0.1, J = 0.3): dT/dV on
    64 random orbitals and dT/dJ against central differences (step 1e-6) of the FP64 oracle."""
    from oracle import Oracle

    sys_, derivs = gradient_bhz(100, 40, configs=1)
    sys_.set_parameter_derivatives(derivs)
    sigma = sys_.self_energies(0.03)
    t, st, dv, dp = sys_.transmissions_with_grad([sigma], [0])
    assert st[0] == 0
    orc = Oracle(sys_.system)
    base = sys_.system.values[0]
    h = 1e-6
    sites = np.random.default_rng(11).choice(sys_.system.n, size=64, replace=False)
    vals = []
    for a in sites:
        q = _diag_index(sys_.system, a)
        for sgn in (1, -1):
            v = base.copy()
            v[q] += sgn * h
            vals.append(v)
    d = derivs[0][0]
    vals += [base + h * d, base - h * d]
    nb = sys_.block_count()
    blocks = [b for _ in vals for b in range(nb)]
    ts, sts = orc.solve_batch(blocks, [sigma.energy] * len(blocks), [v for v in vals for _ in range(nb)],
                              [sigma.blocks[b][0] for _ in vals for b in range(nb)],
                              [sigma.blocks[b][1] for _ in vals for b in range(nb)], threads=0)
    assert (sts == 0).all()
    tt = ts.reshape(len(vals), nb).sum(axis=1)
    for i, a in enumerate(sites):
        fd = (tt[2 * i] - tt[2 * i + 1]) / (2 * h)
        assert abs(dv[0, a] - fd) <= 1e-4 * abs(fd) + 1e-5, (a, dv[0, a], fd)
    fdj = (tt[-2] - tt[-1]) / (2 * h)
    assert abs(dp[0, 0] - fdj) <= 1e-4 * abs(fdj) + 1e-5
