"""The batched workloads at their full sizes, on oracle samples.

- Many ribbons: 256 graphene zigzag ribbons of widths 40-160 and lengths 100-400 cells are drawn
  (xoshiro seed 1, Anderson W = 1); the largest, the smallest and two others, at two of the 64
  energies, run in one batch (caroli_solve_multi) in FP64 and mixed precision against the oracle.
- Cubic wire 64 x 32 x 32 (Anderson W = 16.5, 32 x 32-site leads with ~650 open channels): the
  mixed path with the channel cutoff lifted (one refinement right-hand side per channel) against
  the oracle, and its gradient dT/dV against central differences (step 1e-6) of the FP64 GPU
  transmission, which the same test pins to the oracle.
"""
import numpy as np
import pytest

from systems import cubic_wire, graphene_ribbons, oracle_T
from caroli_gb300 import Precision, solve_systems
from caroli_gb300.disorder import Xoshiro256

pytestmark = pytest.mark.gpu


def test_many_ribbons_at_size_sample():
    rng = Xoshiro256.seed_from_u64(1)
    shapes = [(rng.integer(40, 160), rng.integer(100, 400)) for _ in range(256)]
    area = [w * l for w, l in shapes]
    pick = sorted({int(np.argmax(area)), int(np.argmin(area)), 17, 200})
    ribbons = graphene_ribbons(256, seed=1, widths=(40, 160), lengths=(100, 400), pick=pick)
    energies = np.linspace(-0.5, 0.5, 64)[[5, 40]]
    items = [(rb, rb.self_energies(e), 0) for rb in ribbons for e in energies]
    ref = np.array([oracle_T(rb, s) for rb, s, _ in items])
    for precision, tol in ((Precision.DOUBLE, 1e-10), (Precision.MIXED, 1e-8)):
        t, st, _ = solve_systems(items, precision)
        assert (st == 0).all(), (precision, st)
        err = np.abs(t - ref) / (1 + np.abs(ref))
        assert err.max() <= tol, (precision, err.max(), t, ref)


def test_cubic_64x32x32_mixed_and_gradient():
    from caroli_gb300.nested import context

    sys_ = cubic_wire(64, 32, 32)
    e = np.linspace(-1.0, 1.0, 32)[8]
    sigma = sys_.self_energies(e)
    ctx = context(0)
    try:
        ctx.set_mixed_max_channels(100000)
        tm, st, _ = sys_.solve_batch([sigma], [0], Precision.MIXED)
        assert st[0] == 0 and sys_.plan().last_stats()[0] == 0  # refined, not recomputed in FP64
        t, st, dv, dp = sys_.transmissions_with_grad([sigma], [0])
        assert st[0] == 0
    finally:
        ctx.set_mixed_max_channels(96)
    ref = oracle_T(sys_, sigma)
    assert abs(tm[0] - ref) <= 1e-8 * (1 + abs(ref)), (tm[0], ref)
    assert abs(t[0] - tm[0]) <= 1e-12 * (1 + abs(ref))
    t64, st64, _ = sys_.solve_batch([sigma], [0], Precision.DOUBLE)
    assert st64[0] == 0 and abs(t64[0] - ref) <= 1e-10 * (1 + abs(ref))
    # dT/dV against central differences of the FP64 path (pinned above) on sites of the middle
    # slice and near the leads.
    base = sys_.system.values[0]
    plan = sys_.plan()
    sys_n = sys_.system.n
    sites = [5, sys_n // 2, sys_n // 2 + 517, sys_n - 900]
    h = 1e-6
    vals = []
    for a in sites:
        lo, hi = sys_.system.row_ptr[a], sys_.system.row_ptr[a + 1]
        q = lo + int(np.nonzero(sys_.system.cols[lo:hi] == a)[0][0])
        for sgn in (1, -1):
            v = base.copy()
            v[q] += sgn * h
            vals.append(v)
    plan.upload_values(np.stack(vals))
    try:
        tf, stf, _ = sys_.solve_batch([sigma] * len(vals), list(range(len(vals))), Precision.DOUBLE)
    finally:
        plan.upload_values(np.stack(sys_.system.values))
    assert (stf == 0).all()
    scale = np.abs(dv[0, sites]).max()
    for i, a in enumerate(sites):
        fd = (tf[2 * i] - tf[2 * i + 1]) / (2 * h)
        assert abs(dv[0, a] - fd) <= 1e-4 * scale + 1e-9, (a, dv[0, a], fd)


def test_tensor_core_sweeps_many_channels():
    """Solves with many lead channels sweep their large fronts and the root as tensor-core GEMMs
    (tcgemm.cuh; from 32 columns on). A 24 x 12 x 12 cubic wire (about 90 channels) in mixed
    precision, forward T and the adjoint gradient, against the oracle and the FP64 path."""
    from caroli_gb300.nested import context

    sys_ = cubic_wire(24, 12, 12, configs=2)
    sigmas = [sys_.self_energies(e) for e in (-0.7, 0.4)]
    S, C = [s for s in sigmas for _ in range(2)], [0, 1, 0, 1]
    assert min(s.w_right()[0].shape[1] for s in sigmas) >= 32
    ctx = context(0)
    try:
        ctx.set_mixed_max_channels(100000)
        tm, st, _ = sys_.solve_batch(S, C, Precision.MIXED)
        assert (st == 0).all() and sys_.plan().last_stats()[0] == 0
        tg, stg, dv, _ = sys_.transmissions_with_grad(S, C)
        assert (stg == 0).all()
    finally:
        ctx.set_mixed_max_channels(96)
    t64, st64, _ = sys_.solve_batch(S, C, Precision.DOUBLE)
    for k, (s, c) in enumerate(zip(S, C)):
        ref = oracle_T(sys_, s, config=c)
        assert abs(tm[k] - ref) <= 1e-8 * (1 + abs(ref)), (k, tm[k], ref)
        assert abs(tg[k] - tm[k]) <= 1e-12 * (1 + abs(ref))
        assert abs(t64[k] - ref) <= 1e-10 * (1 + abs(ref))
    # The uniform-shift sum rule of the gradient: Σ_a dT/dV_a = -dT/dE at fixed self-energies.
    h = 1e-6
    plan = sys_.plan()
    vals = []
    for c in (0, 1):
        base = sys_.system.values[c]
        for sgn in (1, -1):
            v = base.copy()
            for a in range(sys_.system.n):
                lo, hi = sys_.system.row_ptr[a], sys_.system.row_ptr[a + 1]
                v[lo + int(np.nonzero(sys_.system.cols[lo:hi] == a)[0][0])] += sgn * h
            vals.append(v)
    plan.upload_values(np.stack(vals))
    try:
        tf, stf, _ = sys_.solve_batch([sigmas[0]] * 4, [0, 1, 2, 3], Precision.DOUBLE)
    finally:
        plan.upload_values(np.stack(sys_.system.values))
    for c in (0, 1):
        fd = (tf[2 * c] - tf[2 * c + 1]) / (2 * h)
        assert abs(dv[c].sum() - fd) <= 1e-4 * abs(fd) + 1e-8, (c, dv[c].sum(), fd)
