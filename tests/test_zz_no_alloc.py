"""The transmission entry point that allocates no device memory (caroli_solve_batch_noalloc).

Callers whose device memory is already reserved by another allocator (for example a framework's
caching pool that has claimed the whole GPU), or that solve inside a loop where allocating is not
allowed, cannot let the library call cudaMalloc when they solve. This entry point runs the
double-precision path on a fixed static device array instead. It must give the same
transmissions as caroli_solve_batch, call after call (the array keeps the previous call's
contents), leave the device's free memory unchanged, report instances whose fronts refuse their
pivots as CAROLI_PIVOT_DELAYED (it does not re-plan), and refuse batches larger than the array
with a clear error.
"""
import numpy as np
import pytest

from systems import bench_system, clean_bhz_ribbon
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


def test_noalloc_reports_delayed_pivots_without_replanning():
    """Clean square lattice: at E = 0 interior blocks are exactly singular (their fronts refuse
    their pivots), at E = 0.3 they are not. The allocation-free call returns PIVOT_DELAYED for the
    first instance and the re-planned solve's T for the other; caroli_solve_batch resolves both."""
    sys_ = bench_system("square-clean", 32)
    slots = [sys_._slot(sys_.self_energies(e)) for e in (0.0, 0.3)]
    plan = sys_.plan()
    t_ref, st_ref, _ = plan.solve(slots, [0, 0], _native.DOUBLE)
    assert (st_ref == 0).all(), st_ref
    for _ in range(2):
        rc, t, st = _noalloc(plan, slots, [0, 0])
        assert rc == _native.OK, plan.ctx.lib.caroli_last_error(plan.ctx.h)
        assert st[0] == _native.PIVOT_DELAYED, st
        assert st[1] == _native.OK, st
        assert abs(t[1] - t_ref[1]) <= 1e-10 * (1 + abs(t_ref[1])), (t, t_ref)


def test_noalloc_leaves_device_memory_unchanged():
    torch = pytest.importorskip("torch")
    sys_ = clean_bhz_ribbon()
    slots = [sys_._slot(sys_.self_energies(e)) for e in (-0.1, 0.05)]
    plan = sys_.plan()
    rc, _, _ = _noalloc(plan, slots, [0, 0])  # warm: kernels loaded, host paths taken once
    assert rc == _native.OK
    free0, _ = torch.cuda.mem_get_info(sys_.device)
    for _ in range(3):
        rc, _, st = _noalloc(plan, slots, [0, 0])
        assert rc == _native.OK and (st == 0).all()
    free1, _ = torch.cuda.mem_get_info(sys_.device)
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_batches_beyond_its_scratch():
    sys_ = clean_bhz_ribbon()
    slot = sys_._slot(sys_.self_energies(0.0))
    plan = sys_.plan()
    rc, _, _ = _noalloc(plan, [slot] * 20000, [0] * 20000)
    assert rc == _native.EINVAL
    assert b"static scratch" in plan.ctx.lib.caroli_last_error(plan.ctx.h)
