"""Error paths of the newer C ABI entry points: bad arguments come back as CAROLI_EINVAL with a
message, and the context stays usable (a solve afterwards gives the right T)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Region, square
from caroli_gb300 import _native

pytestmark = pytest.mark.gpu


def _two():
    m = square()
    return NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [6, 4, 0]), 0)


def test_two_terminal_entry_points_refuse_bad_arguments():
    from systems import cross_system

    s = _two()
    plan = s.plan()
    lib, h = plan.ctx.lib, plan.ctx.h
    sig = s.self_energies(0.3)
    slot = s._slot(sig)
    # Lead modes for a side that does not exist, and self-energies from modes never uploaded.
    y = np.eye(4, dtype=np.complex128)
    with pytest.raises(_native.NativeError):
        plan.lead_modes(0, 2, y, -1.0)
    with pytest.raises(_native.NativeError):
        plan.sigma_from_modes(slot + 1, 0.3, [(np.ones(4, complex), np.ones(4, complex), [0], [1.0])])
    # Disorder of an unknown kind.
    bad = _native.Disorder(kind=7, seed=1)
    with pytest.raises(_native.NativeError):
        plan.generate_values(s.system.values[0], [bad], 1)
    # Multi-terminal calls on a two-terminal plan, and a left factor with too many columns.
    assert lib.caroli_multi_transmissions(h, plan.id, 0, None, None, 0, None, None) == _native.EINVAL
    wl = [[np.zeros((4, 5), np.complex128)]]
    with pytest.raises(_native.NativeError):
        plan.transmission_matrices([slot], [0], wl, [4])
    assert lib.caroli_root_green(h, plan.id, 1, None, None, None, None, None) == _native.EINVAL
    assert lib.caroli_gamma_override(h, plan.id, 99, None, None) == _native.EINVAL
    # The context still solves.
    assert abs(s.transmission_with(sig) - s.transmissions([0.3])[0]) < 1e-12
    # Two-terminal calls on a multi-terminal plan.
    multi = cross_system(8)
    mp = multi.plan()
    msig = multi.self_energies(0.4)
    mslot = multi._slot(msig)
    with pytest.raises(_native.NativeError):
        mp.solve([mslot], [0], int(_native.DOUBLE))
    bad_ptr = np.ones(4 * multi.block_count() + 1, np.int64)  # lead_ptr[0] != 0
    orbs = np.zeros(1, np.int64)
    assert lib.caroli_multi_leads(h, mp.id, 4, _native.ptr(bad_ptr), _native.ptr(orbs)) == _native.EINVAL
    labels, t = multi.sector_transmissions(0.4, [None] * 4)
    assert np.max(np.abs(t - multi.transmissions(0.4))) < 1e-11
