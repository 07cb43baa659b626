"""On-device disorder (`caroli_values_generate`): the values of CLI-style configurations generated
on the GPU against the host's (`disorder.disordered`, the restatement of caroli-disorder pinned by
tests/test_rng.py), bit for bit where no cos/sin enters, and the transmissions they give."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import NestedTwoTerminal, Region, bhz, cubic
from caroli_gb300.disorder import Moments, disordered
from caroli_gb300.model import bhz_spin


def _on_pattern(system, mat):
    """Values of the sparse matrix `mat` on the system's pattern (which must contain it)."""
    n = system.n
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(system.row_ptr))
    keys = rows * n + np.asarray(system.cols, np.int64)
    mr = np.repeat(np.arange(n, dtype=np.int64), np.diff(mat.row_ptr))
    mk = mr * n + np.asarray(mat.cols, np.int64)
    pos = np.searchsorted(keys, mk)
    assert np.all(keys[np.minimum(pos, len(keys) - 1)] == mk), "host entry outside the pattern"
    out = np.zeros(len(keys), np.complex128)
    out[pos] = mat.vals
    return out


def _magnetic(moments, exchange=0.4, concentration=0.2, anderson=None):
    entries = []
    if anderson is not None:
        entries.append({"kind": "anderson", "strength": anderson})
    entries.append({"kind": "magnetic", "concentration": concentration, "exchange": exchange, "moments": moments,
                    "spin": bhz_spin("opposite-g")})
    return entries


CASES = {
    # The workload's disorder: polarized moments (n = z): no cos/sin, bit-exact.
    "polarized": (lambda: _magnetic(Moments.polarized(1.0)), True),
    # Anderson first, then isotropic moments (the gradient workload's entries).
    "anderson+isotropic": (lambda: _magnetic(Moments.isotropic(), 0.3, 0.1, anderson=0.02), False),
    "cone": (lambda: _magnetic(Moments.cone(0.7)), False),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_generated_values_match_host(case):
    make, exact = CASES[case]
    entries = make()
    m = bhz()
    region = Region.cuboid(m.lattice, [20, 10, 0])
    first = 3
    sys_ = NestedTwoTerminal.from_disorder(m, m, region, 0, entries, 4, first_config=first)
    for c in range(4):
        host = _on_pattern(sys_.system, disordered(m, region, entries, first + c).sparse_hamiltonian(region))
        dev = sys_.generated_values(c)
        if exact:
            assert np.array_equal(dev, host)
        else:
            assert np.max(np.abs(dev - host)) <= 4e-16 * max(1.0, np.abs(host).max())
    # The transmissions of the generated configurations against host-built ones on one plan.
    host_sys = NestedTwoTerminal.from_models([disordered(m, region, entries, first + c) for c in range(4)], m,
                                             region, 0)
    sig_d = [sys_.self_energies(e) for e in (-0.1, 0.05)]
    sig_h = [host_sys.self_energies(e) for e in (-0.1, 0.05)]
    pairs = [(i, c) for i in range(2) for c in range(4)]
    td = sys_.transmissions_with([sig_d[i] for i, _ in pairs], [c for _, c in pairs])
    th = host_sys.transmissions_with([sig_h[i] for i, _ in pairs], [c for _, c in pairs])
    assert np.max(np.abs(np.array(td) - np.array(th))) < 1e-10


@pytest.mark.gpu
def test_generated_anderson_cubic():
    m = cubic()
    region = Region.cuboid(m.lattice, [8, 5, 5])
    entries = [{"kind": "anderson", "strength": 16.5, "seed": 1}]
    sys_ = NestedTwoTerminal.from_disorder(m, m, region, 0, entries, 3)
    for c in range(3):
        host = _on_pattern(sys_.system, disordered(m, region, entries, c).sparse_hamiltonian(region))
        assert np.array_equal(sys_.generated_values(c), host)


@pytest.mark.gpu
def test_generate_refuses_missing_pattern():
    """Spin matrices with entries outside the plan's pattern are refused, not dropped."""
    from caroli_gb300 import _native

    m = bhz()
    region = Region.cuboid(m.lattice, [8, 6, 0])
    sys_ = NestedTwoTerminal.from_model(m, m, region, 0)
    plan = sys_.plan()
    spin = np.ascontiguousarray(np.stack([np.asfortranarray(s, np.complex128).ravel(order="F")
                                          for s in bhz_spin("opposite-g")]))
    bad = _native.Disorder(kind=_native.MAGNETIC, moments=_native.MOMENTS_ISOTROPIC, seed=1, concentration=0.2,
                           exchange=0.4, orbitals=4, spin=spin.ctypes.data)
    with pytest.raises(_native.NativeError):
        plan.generate_values(sys_.system.values[0], [bad], 2)
