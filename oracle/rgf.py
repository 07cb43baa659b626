"""Second oracle: the recursive Green's function (RGF) transmission, slice by slice along the
transport axis, in FP64 numpy.

Test infrastructure only: the tests compare the nested-dissection oracle (and through it the GPU
path) with this independent method, as the reference checks nested dissection against its RGF
(`crates/caroli-green/tests/nested.rs:42-50`, cubic `:160-177`).

The recursion follows `TwoTerminal::solve` (`crates/caroli-green/src/two_terminal.rs:260-282`):
left-connected Green's functions g_n = [z - H_nn - V_{n-1}^† g_{n-1} V_{n-1} - Σ]^-1 and the first
row G_1n = G_1,n-1 V_{n-1} g_n, then T = Tr[Γ_L G_1N Γ_R G_1N^†] (`caroli-green/src/lib.rs:106-113`).
It runs per independent block of the system, on the block's slices in the order of the transport
axis, with the lead slices in the order of the self-energies (lead-cell order).
"""
from __future__ import annotations

import numpy as np


def _orbital_sites(system):
    site = np.empty(system.n, dtype=np.int64)
    for s, (off, cnt) in enumerate(zip(system.site_offsets, system.site_orbitals)):
        site[off:off + cnt] = s
    return site


def _slices(system, b):
    """Orbitals of block b grouped by slice along the transport axis, first and last slice in
    the order of the block's lead orbitals."""
    blk = system.blocks[b]
    rows = system.block_rows(b)
    x = system.cells[_orbital_sites(system)[rows], system.axis]
    out = []
    for v in np.unique(x):
        out.append(rows[x == v])
    left, right = np.asarray(blk.left, np.int64), np.asarray(blk.right, np.int64)
    if set(out[0].tolist()) != set(left.tolist()) or set(out[-1].tolist()) != set(right.tolist()):
        raise ValueError("the lead slices are not the first and last device slices")
    out[0] = left
    out[-1] = right
    return out


def _dense(system, values, rows, cols):
    """H restricted to rows x cols (global orbital indices), dense."""
    pos = -np.ones(system.n, np.int64)
    pos[cols] = np.arange(len(cols))
    out = np.zeros((len(rows), len(cols)), np.complex128)
    for a, r in enumerate(rows):
        lo, hi = system.row_ptr[r], system.row_ptr[r + 1]
        cs = system.cols[lo:hi].astype(np.int64)
        keep = pos[cs] >= 0
        np.add.at(out[a], pos[cs[keep]], values[lo:hi][keep])
    return out


def transmission(system, energy, sigmas, config=0, gamma=None):
    """T at real energy `energy` with `sigmas[b] = (Σ_L, Σ_R)` per block, summed over blocks.
    `gamma(Γ)` transforms the broadenings before the trace (the thesis codes take their real part,
    caroli-validation/src/thesis.rs:84-95); None keeps them."""
    values = system.values[config]
    total = 0.0
    for b, (sl, sr) in enumerate(sigmas):
        sl = np.asarray(sl, np.complex128)
        sr = np.asarray(sr, np.complex128)
        sl_ = _slices(system, b)
        n = len(sl_)
        z = complex(energy, 0.0)

        def resolvent(k):
            h = _dense(system, values, sl_[k], sl_[k])
            return z * np.eye(len(sl_[k])) - h

        a = resolvent(0) - sl
        if n == 1:
            a = a - sr
        g = np.linalg.inv(a)
        g1n = g.copy()
        for k in range(1, n):
            v = _dense(system, values, sl_[k - 1], sl_[k])  # V_{k-1} = H_{k-1,k}
            a = resolvent(k) - v.conj().T @ g @ v
            if k == n - 1:
                a = a - sr
            g = np.linalg.inv(a)
            g1n = g1n @ v @ g
        gl = 1j * (sl - sl.conj().T)
        gr = 1j * (sr - sr.conj().T)
        if gamma is not None:
            gl, gr = gamma(gl), gamma(gr)
        total += float(np.real(np.trace(gl @ g1n @ gr @ g1n.conj().T)))
    return total
