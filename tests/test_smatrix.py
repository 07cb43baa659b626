"""Scattering matrix in the basis of the lead modes (smatrix.rs; NestedTwoTerminal::smatrix,
nested.rs:717-752; NestedMultiTerminal::smatrix, nested_multi.rs:440-495), as the reference's tests
check it (tests/nested_multi.rs:321-395, tests/nested.rs:185-205): unitary, its blocks give the
transmissions, a clean ribbon sends each mode straight through, and the two-terminal and
multi-terminal matrices agree."""
from __future__ import annotations

import numpy as np
import pytest

from caroli_gb300 import Interface, NestedMultiTerminal, NestedTwoTerminal, Region, bhz, square
from systems import cross_system


def _hash_disorder(w, norb):
    mask = (1 << 64) - 1

    def term(site):
        k = (site.cell[0] * 7919 + site.cell[1] * 104_729 + site.sub * 31) & mask
        u = (((k * 6_364_136_223_846_793_005 + 1_442_695_040_888_963_407) & mask) >> 11) / float(1 << 53)
        return np.eye(norb) * (w * (u - 0.5))

    return term


def _unitary(s, tol=1e-9):
    full = s.full()
    assert full.shape[0] == full.shape[1]
    assert np.max(np.abs(full.conj().T @ full - np.eye(full.shape[1]))) < tol


def test_smatrix_from_dense_green():
    """The host mode algebra on the oracle's dense G of a disordered square ribbon: unitary, and
    Σ |S_RL|² = T."""
    from caroli_gb300.leads import LeadSolver
    from caroli_gb300.smatrix import ScatteringLead, assemble, scattering_blocks
    from oracle import multi as om
    from systems import oracle_T

    m = square()
    sys_ = NestedTwoTerminal.from_model(m.with_onsite_term(_hash_disorder(2.0, 1)), m,
                                        Region.cuboid(m.lattice, [10, 6, 0]), 0)
    blk = sys_.system.blocks[0]
    for e in (-2.6, -0.9, 0.4):
        sigma = sys_.self_energies(e)
        sl, sr = sigma.blocks[0]
        a = e * np.eye(sys_.system.n) - om.dense_h(sys_.system)
        a[np.ix_(blk.left, blk.left)] -= sl
        a[np.ix_(blk.right, blk.right)] -= sr
        kept = np.concatenate([blk.left, blk.right])
        g = np.linalg.inv(a)[np.ix_(kept, kept)]
        left_out = blk.left_h01.conj().T
        leads = [ScatteringLead(np.arange(len(blk.left)), left_out, left_out,
                                LeadSolver(blk.left_h00, left_out).modes(e), e),
                 ScatteringLead(len(blk.left) + np.arange(len(blk.right)), blk.right_h01, blk.right_h01,
                                LeadSolver(blk.right_h00, blk.right_h01).modes(e), e)]
        s = assemble(e, [scattering_blocks(g, leads, [blk.left_h00, blk.right_h00], e)])
        _unitary(s)
        assert abs(s.transmission(1, 0) - oracle_T(sys_, sigma)) < 1e-9


@pytest.mark.gpu
def test_gpu_smatrix_cross_and_bhz():
    s_sq = cross_system(8, model="square", seed=5, anderson=1.5)
    s_bhz = cross_system(8, model="bhz", seed=3, anderson=0.5)
    for sys_, energies in ((s_sq, (-2.7, -0.4, 1.3)), (s_bhz, (-0.2, 0.02, 0.3))):
        for e in energies:
            s = sys_.smatrix(e)
            _unitary(s)
            t = sys_.transmissions(e)
            for p in range(4):
                for q in range(4):
                    if p != q:
                        assert abs(s.transmission(p, q) - t[p][q]) < 1e-9


@pytest.mark.gpu
def test_gpu_smatrix_clean_ribbon_and_two_terminal():
    m = square()
    region = Region.cuboid(m.lattice, [8, 9, 0])
    sl = region.slices(0)
    multi = NestedMultiTerminal.from_model(m, m, region, [Interface(sl[0], (-1, 0, 0)), Interface(sl[7], (1, 0, 0))])
    for e in (-2.9, -1.1, 0.3, 1.7):
        s = multi.smatrix(e)
        t = s.blocks[1][0]
        mod = np.abs(t)
        assert np.all(np.sum(np.abs(mod - 1.0) < 1e-9, axis=0) == 1)
        assert np.all(np.sum(mod < 1e-9, axis=0) == t.shape[0] - 1)
        assert np.max(np.abs(s.blocks[0][0])) < 1e-9
    dev = m.with_onsite_term(_hash_disorder(2.0, 1))
    region = Region.cuboid(m.lattice, [10, 6, 0])
    sl = region.slices(0)
    two = NestedTwoTerminal.from_model(dev, m, region, 0)
    multi = NestedMultiTerminal.from_model(dev, m, region, [Interface(sl[0], (-1, 0, 0)), Interface(sl[9], (1, 0, 0))])
    for e in (-2.6, -0.9, 0.4, 1.8):
        s2, sm = two.smatrix(e), multi.smatrix(e)
        _unitary(s2)
        assert np.max(np.abs(s2.full() - sm.full())) < 1e-9
        assert abs(s2.transmission(1, 0) - two.transmission(e)) < 1e-9
    b = bhz()
    two = NestedTwoTerminal.from_model(b.with_onsite_term(_hash_disorder(0.6, 4)), b, Region.cuboid(b.lattice, [8, 6, 0]), 0)
    for e in (-0.15, 0.35):
        s = two.smatrix(e)
        _unitary(s)
        assert abs(s.transmission(1, 0) - two.transmission(e)) < 1e-9
