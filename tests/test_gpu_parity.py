"""GPU path against the oracle on the same inputs (all through the C ABI)."""
import numpy as np
import pytest

from systems import bench_golden, bench_system, clean_bhz_ribbon, cubic_wire, magnetic_bhz, oracle_T
from caroli_gb300 import GreenError, Precision

pytestmark = pytest.mark.gpu


def test_clean_bhz_33_energies_double():
    """Plain FP64: clean BHZ 16 x 10, 33 energies in [-0.16, 0.16]; T(0) = 2 to 1e-8."""
    sys_ = clean_bhz_ribbon()
    energies = np.linspace(-0.16, 0.16, 33)
    sigmas = [sys_.self_energies(e) for e in energies]
    ts = sys_.transmissions_with(sigmas)
    for s, t in zip(sigmas, ts):
        ref = oracle_T(sys_, s)
        assert abs(t - ref) <= 1e-10 * (1 + abs(ref)), (s.energy, t, ref)
    assert abs(ts[16] - 2.0) < 1e-8


@pytest.mark.parametrize("problem", ["square-anderson", "bhz-anderson", "graphene-anderson", "square-clean"])
def test_bench_w32_double_matches_oracle_and_published(problem):
    gold = bench_golden()[f"caroli/{problem}/32"]
    sys_ = bench_system(problem, 32)
    sigmas = [sys_.self_energies(e) for e in gold["energies"]]
    ts = sys_.transmissions_with(sigmas)
    runs = np.array(gold["runs"])
    for k, (s, t) in enumerate(zip(sigmas, ts)):
        ref = oracle_T(sys_, s)
        assert abs(t - ref) <= 1e-10 * (1 + abs(ref)), (problem, s.energy, t, ref)
        assert abs(t - np.median(runs[:, k])) <= 1e-8 * (1 + abs(t))


def test_clean_square_delayed_pivots():
    """Clean square lattice at E = 0: interior blocks are exactly singular and get delayed
    (tests/nested.rs covers E = 0); the GPU re-plans those solves."""
    sys_ = bench_system("square-clean", 32)
    s = sys_.self_energies(0.0)
    t = sys_.transmission_with(s)
    assert abs(t - oracle_T(sys_, s)) < 1e-9
    assert abs(t - round(t)) < 1e-8


def test_magnetic_configurations_batch():
    sys_ = magnetic_bhz(24, 12, configs=3)
    sigmas = [sys_.self_energies(e) for e in (-0.12, 0.0, 0.07)]
    pairs = [(s, c) for s in sigmas for c in range(3)]
    ts = sys_.transmissions_with([p[0] for p in pairs], [p[1] for p in pairs])
    for (s, c), t in zip(pairs, ts):
        ref = oracle_T(sys_, s, config=c)
        assert abs(t - ref) <= 1e-10 * (1 + abs(ref))


def test_cubic_wire():
    sys_ = cubic_wire(12, 6, 6, configs=2)
    for e in (-0.5, 0.3):
        s = sys_.self_energies(e)
        for c in range(2):
            t = sys_.transmission_with(s, config=c)
            assert abs(t - oracle_T(sys_, s, config=c)) <= 1e-10 * (1 + t)


def test_single_precision_follows_double():
    sys_ = bench_system("bhz-anderson", 32)
    s = sys_.self_energies(0.3)
    t32 = sys_.transmission_with_precision(s, Precision.SINGLE)
    assert abs(t32 - oracle_T(sys_, s)) < 1e-2


def test_mixed_refined_matches_double():
    """Mixed precision: f32 factors + FP64 refinement reach |ΔT| <= 1e-8 of the oracle."""
    sys_ = magnetic_bhz(40, 16, configs=2)
    sigmas = [sys_.self_energies(e) for e in np.linspace(-0.16, 0.16, 5)]
    pairs = [(s, c) for s in sigmas for c in range(2)]
    t, st, err = sys_.solve_batch([p[0] for p in pairs], [p[1] for p in pairs], Precision.MIXED)
    assert (st == 0).all(), st
    for (s, c), tm in zip(pairs, t):
        ref = oracle_T(sys_, s, config=c)
        assert abs(tm - ref) <= 1e-8, (s.energy, c, tm, ref)


@pytest.mark.parametrize("problem", ["bhz-anderson", "graphene-anderson", "square-anderson"])
def test_mixed_bench_w32(problem):
    gold = bench_golden()[f"caroli/{problem}/32"]
    sys_ = bench_system(problem, 32)
    sigmas = [sys_.self_energies(e) for e in gold["energies"]]
    t, st, err = sys_.solve_batch(sigmas, [0] * len(sigmas), Precision.MIXED)
    assert (st == 0).all(), st
    fallbacks, iters = sys_.plan().last_stats()
    assert fallbacks == 0 and iters <= 4, (fallbacks, iters)
    for s, tm in zip(sigmas, t):
        ref = oracle_T(sys_, s)
        assert abs(tm - ref) <= 1e-8, (problem, s.energy, tm, ref)


def test_magnetic_200x64_double_and_mixed_match_oracle():
    """The full-size magnetic workload (BHZ 200 x 64, c = 0.2, J = 0.4, eight configurations) at the
    band edge E = -0.16, where ill-conditioned pivot blocks occur: FP64 and mixed both within 1e-8
    of the oracle."""
    from oracle import Oracle

    sys_ = magnetic_bhz(200, 64, configs=8)
    s = sys_.self_energies(-0.16)
    cfg = list(range(8))
    t64, st64, _ = sys_.solve_batch([s] * 8, cfg, Precision.DOUBLE)
    tm, stm, _ = sys_.solve_batch([s] * 8, cfg, Precision.MIXED)
    assert (st64 == 0).all() and (stm == 0).all()
    orc = Oracle(sys_.system)
    nb = sys_.block_count()
    blocks = [b for _ in cfg for b in range(nb)]
    ref, st = orc.solve_batch(blocks, [s.energy] * len(blocks), [sys_.system.values[c] for c in cfg for _ in range(nb)],
                              [s.blocks[b][0] for _ in cfg for b in range(nb)],
                              [s.blocks[b][1] for _ in cfg for b in range(nb)], threads=0)
    assert (st == 0).all()
    ref = ref.reshape(8, nb).sum(axis=1)
    assert np.abs(t64 - ref).max() <= 1e-8, np.abs(t64 - ref)
    assert np.abs(tm - ref).max() <= 1e-8, np.abs(tm - ref)


def test_magnetic_200x64_mixed_across_the_band():
    """The headline workload's mixed path against the oracle over the band: eight energies of the
    bench's 33-point grid in [-0.16, 0.16] (both ends, the gap edges and mid-gap) x the eight
    configurations (128 block solves), every point within 1e-8 and none recomputed in FP64."""
    from oracle import Oracle

    sys_ = magnetic_bhz(200, 64, configs=8)
    energies = [-0.16, -0.13, -0.08, -0.03, 0.0, 0.06, 0.12, 0.16]
    sigmas = [sys_.self_energies(e) for e in energies]
    pairs = [(s, c) for s in sigmas for c in range(8)]
    tm, stm, _ = sys_.solve_batch([p[0] for p in pairs], [p[1] for p in pairs], Precision.MIXED)
    assert (stm == 0).all(), stm
    fallbacks, _ = sys_.plan().last_stats()
    assert fallbacks == 0
    orc = Oracle(sys_.system)
    nb = sys_.block_count()
    ref, st = orc.solve_batch([b for _ in pairs for b in range(nb)], [s.energy for s, _ in pairs for _ in range(nb)],
                              [sys_.system.values[c] for _, c in pairs for _ in range(nb)],
                              [s.blocks[b][0] for s, _ in pairs for b in range(nb)],
                              [s.blocks[b][1] for s, _ in pairs for b in range(nb)], threads=0)
    assert (st == 0).all()
    ref = ref.reshape(len(pairs), nb).sum(axis=1)
    dT = np.abs(tm - ref)
    assert dT.max() <= 1e-8, (dT.max(), pairs[int(dT.argmax())][0].energy)


def test_tensor_core_updates_match_cuda_cores():
    """The f32 rank-32 updates on tcgen05 (3xTF32) against the same updates on the CUDA cores:
    unrefined single-precision T is as close to the oracle either way (f32 rounding differs, and
    near a band edge it moves T by up to ~1e-3), and both mixed-precision results reach the oracle
    within 1e-8 with about the same refinement effort (GMRES steps over the batch)."""
    from caroli_gb300.nested import context

    sys_ = magnetic_bhz(60, 48, configs=2)
    sigmas = [sys_.self_energies(e) for e in (-0.14, 0.02, 0.11)]
    pairs = [(s, c) for s in sigmas for c in range(2)]
    S, C = [p[0] for p in pairs], [p[1] for p in pairs]
    ctx = context(0)
    out = {}
    ctx.set_autotune(False)  # the schedule as set here, not the tuner's choice
    try:
        for tc in (True, False):
            ctx.set_tensor_cores(tc)
            t32, st32, _ = sys_.solve_batch(S, C, Precision.SINGLE)
            tm, stm, _ = sys_.solve_batch(S, C, Precision.MIXED)
            assert (st32 == 0).all() and (stm == 0).all()
            out[tc] = (t32, tm, sys_.plan().last_refine_steps()[0])
    finally:
        ctx.set_tensor_cores(True)
        ctx.set_autotune(True)
    for k, (s, c) in enumerate(pairs):
        ref = oracle_T(sys_, s, config=c)
        e_tc, e_cc = abs(out[True][0][k] - ref), abs(out[False][0][k] - ref)
        # Unrefined f32 either way (3xTF32 products carry about 4x the rounding of an f32 FMA).
        assert e_tc <= 1e-2 and e_cc <= 1e-2, (s.energy, c, e_tc, e_cc)
        a, b = out[True][1][k], out[False][1][k]
        assert abs(a - ref) <= 1e-8 and abs(b - ref) <= 1e-8, (s.energy, c, a, b, ref)
    assert out[True][2] <= out[False][2] + 4, (out[True][2], out[False][2])


def test_uneven_ribbons_in_one_batch():
    """Ribbons of different widths and lengths (different trees, roots and leads) in one batch:
    each T equals the oracle's, in FP64 and mixed precision."""
    from caroli_gb300 import solve_systems
    from systems import graphene_ribbons

    ribbons = graphene_ribbons(6)
    items = []
    for k, sys_ in enumerate(ribbons):
        for e in (-0.4, 0.1 + 0.05 * k, 0.45):
            items.append((sys_, sys_.self_energies(e), 0))
    for precision, tol in ((Precision.DOUBLE, 1e-10), (Precision.MIXED, 1e-8)):
        t, st, _ = solve_systems(items, precision)
        assert (st == 0).all(), st
        for (sys_, s, c), tv in zip(items, t):
            ref = oracle_T(sys_, s, config=c)
            assert abs(tv - ref) <= tol * (1 + abs(ref)), (precision, s.energy, tv, ref)


def test_cubic_wire_wide_separators():
    """A cubic wire with a 20 x 20-site cross-section: separators of 400 variables, so the FP64 panel
    sweep runs in global memory (its candidate rows no longer fit in shared memory); mixed precision
    takes the FP64 path there (hundreds of lead channels). Both against the oracle."""
    sys_ = cubic_wire(16, 20, 20)
    s = sys_.self_energies(-0.3)
    ref = oracle_T(sys_, s)
    for precision in (Precision.DOUBLE, Precision.MIXED):
        t, st, _ = sys_.solve_batch([s], [0], precision)
        assert st[0] == 0
        assert abs(t[0] - ref) <= 1e-10 * (1 + abs(ref)), (precision, t[0], ref)


def test_invalid_arguments_and_empty_batch():
    """Bad plan, slot or configuration: an error from the C ABI (no launch); an empty batch: empty
    results."""
    from caroli_gb300 import _native

    sys_ = clean_bhz_ribbon(8, 6)
    s = sys_.self_energies(0.05)
    sys_.solve_batch([s], [0])
    plan = sys_.plan()
    with pytest.raises(_native.NativeError):
        plan.solve([57], [0])
    with pytest.raises(_native.NativeError):
        plan.solve([0], [3])
    with pytest.raises(_native.NativeError):
        plan.solve([0], [0], precision=7)
    t, st, err = plan.solve([], [])
    assert t.shape == (0,) and st.shape == (0,)
