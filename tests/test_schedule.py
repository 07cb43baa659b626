"""The autotuned factorization schedule and CUDA graph replay of repeated batches.

The autotuner times the f32 factorization of a plan set under each candidate schedule (fronts up
to 48, 64 or 96 variables in one CTA; larger fronts' Schur complements as one tensor-core GEMM,
as rank-32 tensor-core updates, or on the CUDA cores) and keeps the fastest; every schedule must
give the oracle's T in mixed precision. A batch solved
again with the same plans and buffers replays its factorization as one CUDA graph; the replay must
give the same bits as the direct launches.
"""
import numpy as np
import pytest

from systems import magnetic_bhz, oracle_T
from caroli_gb300 import Precision
from caroli_gb300.nested import context

pytestmark = pytest.mark.gpu


def test_autotuner_picks_the_fastest_trial_and_keeps_parity():
    sys_ = magnetic_bhz(60, 48, configs=2)
    sigmas = [sys_.self_energies(e) for e in (-0.14, 0.05)]
    S, C = [s for s in sigmas for _ in range(2)], [0, 1, 0, 1]
    ctx = context(0)
    ctx.set_autotune(True)
    t, st, _ = sys_.solve_batch(S, C, Precision.MIXED)
    assert (st == 0).all()
    sch = ctx.last_schedule()
    assert sch["tuned"]
    trials = [x for x in sch["trial_ms"] if x is not None]
    assert len(trials) == 9 and min(trials) > 0
    idx = [48, 64, 96].index(sch["small_max"]) * 3 + (2 - sch["update_mode"])
    assert sch["trial_ms"][idx] == min(trials)
    for (s, c), tv in zip(zip(S, C), t):
        assert abs(tv - oracle_T(sys_, s, config=c)) <= 1e-8
    # Every candidate schedule reaches the oracle too (the tuner may pick any of them).
    ctx.set_autotune(False)
    try:
        t0, st0, _ = sys_.solve_batch(S, C, Precision.MIXED)
        assert (st0 == 0).all() and np.abs(t0 - t).max() <= 2e-8
    finally:
        ctx.set_autotune(True)


def test_graph_replay_gives_the_same_bits():
    sys_ = magnetic_bhz(40, 24, configs=2)
    sigmas = [sys_.self_energies(e) for e in (-0.1, 0.03, 0.12)]
    S, C = [s for s in sigmas for _ in range(2)], [0, 1] * 3
    ctx = context(0)
    for precision in (Precision.MIXED, Precision.DOUBLE):
        ctx.set_graphs(False)
        ref, st, _ = sys_.solve_batch(S, C, precision)
        assert (st == 0).all()
        ctx.set_graphs(True)
        before = ctx.last_schedule()
        outs = [sys_.solve_batch(S, C, precision)[0] for _ in range(3)]
        after = ctx.last_schedule()
        assert after["graph_captures"] == before["graph_captures"] + 1
        assert after["graph_replays"] >= before["graph_replays"] + 1
        for o in outs:
            assert np.array_equal(o, ref), (precision, np.abs(o - ref).max())
