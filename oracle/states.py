"""ORACLE — test infrastructure only (tests). Scattering states and the lesser Green's function of
a two-terminal system by sparse direct solves in FP64 (scipy SuperLU), block by block.

- ``scattering_states`` restates ``NestedTwoTerminal::scattering_states``
  (``crates/caroli-green/src/nested.rs:851-899``): ψ_p = G W_p with the sources W_L on the left
  slice and W_R on the right slice of each block, columns concatenated over blocks, zero outside a
  block's orbitals. Any exact solve of A X = B gives the same X; this one factors
  A = E - H - Σ_L - Σ_R of the block with SuperLU instead of the nested elimination.
- ``lesser_currents`` and ``lesser_occupation`` compute G^< = i G (f_L Γ_L + f_R Γ_R) G^† from the
  dense G of each block, independent of the states: the reference checks its states against the
  recursive lesser Green's function the same way (``crates/caroli-keldysh/tests/nested_states.rs:44-100``:
  occupations and bond currents to 1e-10, cross-section currents equal to T (f_L - f_R) to 1e-9).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _block_matrix(system, values, b, energy, sl, sr):
    """A = E - H - Σ_L - Σ_R on block b's orbitals (sorted), and the positions of its lead slices."""
    rows = system.block_rows(b)
    pos = -np.ones(system.n, np.int64)
    pos[rows] = np.arange(len(rows))
    r = np.repeat(np.arange(system.n, dtype=np.int64), np.diff(system.row_ptr))
    c = np.asarray(system.cols, np.int64)
    keep = (pos[r] >= 0) & (pos[c] >= 0)
    m = len(rows)
    h = sp.coo_matrix((np.asarray(values)[keep], (pos[r[keep]], pos[c[keep]])), shape=(m, m)).tocsc()
    a = (energy * sp.identity(m, dtype=np.complex128, format="csc") - h).tolil()
    blk = system.blocks[b]
    li, ri = pos[np.asarray(blk.left)], pos[np.asarray(blk.right)]
    a[np.ix_(li, li)] = a[np.ix_(li, li)].toarray() - sl
    a[np.ix_(ri, ri)] = a[np.ix_(ri, ri)].toarray() - sr
    return rows, a.tocsc(), li, ri


def scattering_states(system, energy, sigmas, w_left, w_right, config=0):
    """[ψ_L, ψ_R] (n x channels each) with the caller's lead factors ``w_left[b]``, ``w_right[b]``."""
    values = system.values[config]
    cl = sum(w.shape[1] for w in w_left)
    cr = sum(w.shape[1] for w in w_right)
    psi_l = np.zeros((system.n, cl), np.complex128)
    psi_r = np.zeros((system.n, cr), np.complex128)
    c0l = c0r = 0
    for b, (sl, sr) in enumerate(sigmas):
        rows, a, li, ri = _block_matrix(system, values, b, energy, np.asarray(sl), np.asarray(sr))
        wl, wr = np.asarray(w_left[b]), np.asarray(w_right[b])
        rhs = np.zeros((len(rows), wl.shape[1] + wr.shape[1]), np.complex128)
        rhs[li, :wl.shape[1]] = wl
        rhs[ri, wl.shape[1]:] = wr
        x = spla.splu(a).solve(rhs) if rhs.shape[1] else rhs
        psi_l[rows, c0l:c0l + wl.shape[1]] = x[:, :wl.shape[1]]
        psi_r[rows, c0r:c0r + wr.shape[1]] = x[:, wl.shape[1]:]
        c0l += wl.shape[1]
        c0r += wr.shape[1]
    return [psi_l, psi_r]


def _lesser_blocks(system, energy, sigmas, f, config):
    """Per block: its orbitals and the dense G^< = i G (f_L Γ_L + f_R Γ_R) G^† on them."""
    values = system.values[config]
    out = []
    for b, (sl, sr) in enumerate(sigmas):
        sl, sr = np.asarray(sl), np.asarray(sr)
        rows, a, li, ri = _block_matrix(system, values, b, energy, sl, sr)
        g = np.linalg.inv(a.toarray())
        gam = np.zeros_like(g)
        gam[np.ix_(li, li)] += f[0] * 1j * (sl - sl.conj().T)
        gam[np.ix_(ri, ri)] += f[1] * 1j * (sr - sr.conj().T)
        out.append((rows, 1j * (g @ gam @ g.conj().T)))
    return out


def lesser_occupation(system, energy, sigmas, f, config=0):
    """Im G^<_aa / 2π of every orbital (0 outside the blocks)."""
    occ = np.zeros(system.n)
    for rows, gl in _lesser_blocks(system, energy, sigmas, f, config):
        occ[rows] = np.diag(gl).imag / (2.0 * np.pi)
    return occ


def lesser_currents(system, energy, sigmas, f, config=0, op=None):
    """{(i, j): current} over site pairs i < j coupled by H: 2 Re Σ_ab H_ab G^<_ba, or with an
    on-site operator O, Re Tr[(O H_ij + H_ij O) G^<_ji] (``bond_currents``, nested.rs:927-1000)."""
    values = np.asarray(system.values[config])
    owner = np.empty(system.n, np.int64)
    for i, (o, k) in enumerate(zip(system.site_offsets, system.site_orbitals)):
        owner[o:o + k] = i
    pos, lesser = {}, []
    for rows, gl in _lesser_blocks(system, energy, sigmas, f, config):
        for k, a in enumerate(rows):
            pos[int(a)] = (k, len(lesser))
        lesser.append(gl)

    def g_at(b, a):  # G^<_ba; zero between blocks and on dropped orbitals
        if b not in pos or a not in pos or pos[b][1] != pos[a][1]:
            return 0.0
        return lesser[pos[b][1]][pos[b][0], pos[a][0]]

    hblk = {}
    for a in range(system.n):
        for q in range(system.row_ptr[a], system.row_ptr[a + 1]):
            bcol = int(system.cols[q])
            i, j = owner[a], owner[bcol]
            if i >= j or values[q] == 0:
                continue
            hblk.setdefault((int(i), int(j)), []).append((a, bcol, values[q]))
    out = {}
    offs, norb = system.site_offsets, system.site_orbitals
    for (i, j), ent in hblk.items():
        if op is None:
            out[(i, j)] = float(sum((2.0 * h * g_at(bcol, a)).real for a, bcol, h in ent))
        else:
            hij = np.zeros((norb[i], norb[j]), np.complex128)
            for a, bcol, h in ent:
                hij[a - offs[i], bcol - offs[j]] += h
            g = np.zeros((norb[j], norb[i]), np.complex128)
            for bb in range(norb[j]):
                for aa in range(norb[i]):
                    g[bb, aa] = g_at(int(offs[j] + bb), int(offs[i] + aa))
            w = op @ hij + hij @ op
            out[(i, j)] = float(np.sum(w * g.T).real)
    return out


def lesser_site_densities(system, energy, sigmas, f, config=0, op=None):
    """Tr[O (-i G^<)_ii] / 2π of every site i (``site_densities``, nested.rs:1002-1026)."""
    pos, lesser = {}, []
    for rows, gl in _lesser_blocks(system, energy, sigmas, f, config):
        for k, a in enumerate(rows):
            pos[int(a)] = (k, len(lesser))
        lesser.append(gl)
    out = np.zeros(len(system.site_offsets))
    for i, (o, k) in enumerate(zip(system.site_offsets, system.site_orbitals)):
        g = np.zeros((k, k), np.complex128)
        for a in range(k):
            for b in range(k):
                pa, pb = pos.get(int(o + a)), pos.get(int(o + b))
                if pa is not None and pb is not None and pa[1] == pb[1]:
                    g[a, b] = -1j * lesser[pa[1]][pa[0], pb[0]]
        m = g if op is None else np.asarray(op) @ g
        out[i] = np.trace(m).real / (2.0 * np.pi)
    return out
