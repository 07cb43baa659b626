"""The library's symbolic phase (C++ planner behind caroli_plan_upload) builds the reference's
tree: the same fronts in the same post-order, with the same sizes as the oracle's restatement of
split/symbolic/front_vars (nested.rs:127-179, :1049-1122). No GPU work is involved."""
import numpy as np
import pytest

from systems import bench_problem, clean_bhz_ribbon, cubic_wire, magnetic_bhz
from caroli_gb300 import NestedTwoTerminal, _native
from oracle import Oracle


def _library_fronts(sys_, block):
    try:
        ctx = _native.Context(0)
    except _native.NativeError:
        pytest.skip("the planner is reached through a device context; no CUDA device here")
    plan = _native.Plan(ctx, sys_.system)
    return plan.fronts(block)


@pytest.mark.gpu
@pytest.mark.parametrize("make", [clean_bhz_ribbon, lambda: magnetic_bhz(30, 12, 2),
                                  lambda: cubic_wire(8, 4, 4),
                                  lambda: NestedTwoTerminal.from_model(*bench_problem("graphene-anderson", 16), 0)])
def test_planner_matches_oracle_tree(make):
    sys_ = make()
    orc = Oracle(sys_.system)
    for b in range(sys_.block_count()):
        n, ne, level = _library_fronts(sys_, b)
        on, one = orc.tree_fronts(b)
        assert np.array_equal(n, on) and np.array_equal(ne, one)
        # Children run before their parents: levels never decrease along the post-order of a path.
        assert level.min() == 0
