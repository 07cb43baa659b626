"""The oracle (C++ restatement of nested.rs) and the host inputs (models, disorder, lead
self-energies) against caroli's published transmissions and the thesis golden case."""
import json
import os

import numpy as np
import pytest

from systems import GOLDEN, bench_golden, bench_problem, clean_bhz_ribbon, oracle_T
from caroli_gb300 import NestedTwoTerminal


@pytest.mark.parametrize("problem", ["square-clean", "square-anderson", "bhz-anderson", "graphene-anderson"])
def test_bench_w32_matches_published(problem):
    gold = bench_golden()[f"caroli/{problem}/32"]
    dev, lead, region = bench_problem(problem, 32)
    sys_ = NestedTwoTerminal.from_model(dev, lead, region, 0)
    runs = np.array(gold["runs"])
    for k, e in enumerate(gold["energies"]):
        t = oracle_T(sys_, sys_.self_energies(e))
        # The published runs agree among themselves to ~1e-11 (faer vs Accelerate, thread count).
        assert abs(t - np.median(runs[:, k])) < 1e-9 * (1 + abs(t)), (problem, e, t, runs[:, k])


def test_thesis_clean_ribbon_integer_transmission():
    """ti_conductance.rs:26-47: integer T within 0.025 of the thesis, T = 2 on the QSH plateau."""
    with open(os.path.join(GOLDEN, "ti_cond2t_clean.json")) as f:
        g = json.load(f)
    sys_ = clean_bhz_ribbon()
    for e, gr in zip(g["energies"], g["conductance"]):
        t = oracle_T(sys_, sys_.self_energies(e))
        assert abs(t - round(t)) < 1e-8, (e, t)
        assert abs(t - gr) < 0.025, (e, t, gr)
    for e in (-0.05, 0.0, 0.02, 0.05):
        assert abs(oracle_T(sys_, sys_.self_energies(e)) - 2.0) < 1e-8


def test_blocks_of_bhz_are_spin_blocks():
    sys_ = clean_bhz_ribbon()
    assert sys_.block_count() == 2
    assert set(np.unique(sys_.system.labels[::4])) == {0} and set(np.unique(sys_.system.labels[2::4])) == {1}


@pytest.mark.slow
@pytest.mark.parametrize("problem", ["bhz-anderson", "square-anderson"])
def test_bench_w64_matches_published(problem):
    gold = bench_golden()[f"caroli/{problem}/64"]
    dev, lead, region = bench_problem(problem, 64)
    sys_ = NestedTwoTerminal.from_model(dev, lead, region, 0)
    runs = np.array(gold["runs"])
    for k in (1, 4, 6):
        e = gold["energies"][k]
        t = oracle_T(sys_, sys_.self_energies(e))
        assert abs(t - np.median(runs[:, k])) < 1e-8 * (1 + abs(t))


def test_graphene_w64_matches_published():
    """Graphene zigzag leads (rank-deficient coupling: the reduced 2r pencil with Schur bases of the
    edge states) at W = 64: the published transmissions to 1e-10."""
    gold = bench_golden()["caroli/graphene-anderson/64"]
    dev, lead, region = bench_problem("graphene-anderson", 64)
    sys_ = NestedTwoTerminal.from_model(dev, lead, region, 0)
    runs = np.array(gold["runs"])
    for k, e in enumerate(gold["energies"]):
        t = oracle_T(sys_, sys_.self_energies(e))
        assert abs(t - np.median(runs[:, k])) < 1e-10 * (1 + abs(t)), (e, t, runs[:, k])
