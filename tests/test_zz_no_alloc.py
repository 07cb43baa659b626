"""The transmission entry point that allocates no device memory (caroli_solve_batch_noalloc).

Callers whose device memory is already reserved by another allocator (for example a framework's
caching pool that has claimed the whole GPU), or that solve inside a loop where allocating is not
allowed, cannot let the library call cudaMalloc when they solve. This entry point runs the
double-precision path on a fixed static device array instead. It must give the same
transmissions as caroli_solve_batch, call after call (the array keeps the previous call's
contents), and refuse batches larger than the array with a clear error.
"""
import ctypes

import numpy as np
import pytest

from systems import clean_bhz_ribbon
from caroli_gb300 import _native

pytestmark = pytest.mark.gpu


def _noalloc(plan, slots, configs):
    lib = plan.ctx.lib
    slots = np.ascontiguousarray(slots, np.int32)
    configs = np.ascontiguousarray(configs, np.int32)
    t = np.zeros(len(slots))
    st = np.zeros(len(slots), np.int32)
    rc = lib.caroli_solve_batch_noalloc(plan.ctx.h, plan.id, len(slots), _native.ptr(slots), _native.ptr(configs),
                                        _native.ptr(t), _native.ptr(st))
    return rc, t, st


def test_noalloc_matches_solve_batch_twice():
    sys_ = clean_bhz_ribbon()
    sigmas = [sys_.self_energies(e) for e in (-0.16, -0.05, 0.0, 0.07, 0.13)]
    slots = [sys_._slot(s) for s in sigmas]
    plan = sys_.plan()
    t_ref, st_ref, _ = plan.solve(slots, [0] * len(slots), _native.DOUBLE)
    assert (st_ref == 0).all()
    for _ in range(2):
        rc, t, st = _noalloc(plan, slots, [0] * len(slots))
        assert rc == _native.OK, plan.ctx.lib.caroli_last_error(plan.ctx.h)
        assert (st == 0).all(), st
        assert np.all(np.abs(t - t_ref) <= 1e-10 * (1 + np.abs(t_ref))), (t, t_ref)


def test_noalloc_rejects_batches_beyond_its_scratch():
    sys_ = clean_bhz_ribbon()
    slot = sys_._slot(sys_.self_energies(0.0))
    plan = sys_.plan()
    rc, _, _ = _noalloc(plan, [slot] * 20000, [0] * 20000)
    assert rc == _native.EINVAL
    assert b"static scratch" in plan.ctx.lib.caroli_last_error(plan.ctx.h)
