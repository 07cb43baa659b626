"""A bounded device wait that runs out: the tensor-core update's pipeline waits given no polls.

The failure is made without faulting or hanging the GPU: caroli_set_wait_limit(ctx, 0) makes
every pipeline wait of tc_update_kernel give up at once, on barriers that have not completed yet.
The kernel then drains the copies and products it issued (those waits keep their own bound),
frees its tensor memory and marks the solve CAROLI_TIMEOUT. The status must reach the caller, a
mixed-precision solve must be recomputed in FP64 (status 105 per block solve) with the oracle's T,
and after the limit is restored the same context must give the oracle's results again.
"""
import numpy as np
import pytest

from systems import bench_system, oracle_T
from caroli_gb300 import Precision, _native

pytestmark = pytest.mark.gpu


def test_wait_limit_timeout_reaches_caller_and_context_recovers():
    sys_ = bench_system("bhz-anderson", 32)  # fronts above 96 variables: the tensor-core update runs
    sigmas = [sys_.self_energies(e) for e in (-0.1, 0.3)]
    ref = [oracle_T(sys_, s) for s in sigmas]
    plan = sys_.plan()
    ctx = plan.ctx
    ctx.set_tensor_cores(True)
    ctx.set_autotune(False)  # the default schedule: fronts above 96 variables on the tensor cores
    try:
        ctx.set_wait_limit(0)
        t, st, _ = sys_.solve_batch(sigmas, [0, 0], Precision.SINGLE)
        assert (st == _native.TIMEOUT).all(), st
        t, st, _ = sys_.solve_batch(sigmas, [0, 0], Precision.MIXED)
        assert (st == _native.OK).all(), st
        _, _, jst = plan.last_job_info()
        assert (np.asarray(jst) == 100 + _native.TIMEOUT).all(), jst
        for tm, r in zip(t, ref):
            assert abs(tm - r) <= 1e-10 * (1 + abs(r)), (tm, r)
    finally:
        ctx.set_wait_limit(-1)
        ctx.set_autotune(True)
    ctx.set_autotune(False)
    t, st, _ = sys_.solve_batch(sigmas, [0, 0], Precision.SINGLE)
    ctx.set_autotune(True)
    assert (st == _native.OK).all(), st
    for ts, r in zip(t, ref):
        assert abs(ts - r) < 1e-2, (ts, r)
    t, st, _ = sys_.solve_batch(sigmas, [0, 0], Precision.MIXED)
    assert (st == _native.OK).all(), st
    _, _, jst = plan.last_job_info()
    assert (np.asarray(jst) == 0).all(), jst
    for tm, r in zip(t, ref):
        assert abs(tm - r) <= 1e-8, (tm, r)
