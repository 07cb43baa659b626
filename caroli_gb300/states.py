"""Scattering states and the observables built from them.

``ScatteringStates`` mirrors ``caroli_green::ScatteringStates`` (``crates/caroli-green/src/nested.rs:473-502``):
``leads[p]`` is ``ψ_p = G W_p`` on every device orbital (region order), one column per channel of
lead ``p`` (left, then right). The states come from the GPU (``caroli_scattering_states``); the
observables below are host reductions over them, as in the reference:

- ``occupation``      ``Σ_p f_p |ψ_p,a|² / 2π`` per orbital (nested.rs:488-500)
- ``bond_currents``   ``2 Re Tr[H_ij G^<_ji]``, ``G^< = i Σ_p f_p ψ_p ψ_p†`` (nested.rs:927-1000)
- ``site_densities``  ``Σ_p f_p ψ_p† O ψ_p / 2π`` per site (nested.rs:1002-1026)
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class ScatteringStates:
    energy: float
    leads: list  # [ψ_L (n x channels), ψ_R (n x channels)], complex128
    config: int = 0

    def occupation(self, f):
        """Occupied spectral density of every orbital for lead occupations ``f``."""
        _check_f(self, f)
        acc = np.zeros(self.leads[0].shape[0] if self.leads else 0)
        for m, fp in zip(self.leads, f):
            acc += fp * np.sum(np.abs(m) ** 2, axis=1)
        return acc / (2.0 * np.pi)


@dataclass(frozen=True)
class BondCurrent:
    """Spectral particle current from site ``from_`` to site ``to`` (region site indices, or the
    region's ``Site`` objects when the system was built from a region)."""

    from_: object
    to: object
    current: float


def _check_f(states, f):
    if len(f) != len(states.leads):
        raise ValueError("one occupation per lead")


def _owners(system):
    owner = np.empty(system.n, dtype=np.int64)
    for i, (o, k) in enumerate(zip(system.site_offsets, system.site_orbitals)):
        owner[o:o + k] = i
    return owner


def _lesser_rows(states, f, b, a):
    """``G^<_ba`` for index arrays ``b``, ``a`` (elementwise): ``i Σ_p f_p Σ_k ψ_bk conj(ψ_ak)``."""
    acc = np.zeros(len(b), np.complex128)
    for m, fp in zip(states.leads, f):
        if m.shape[1] == 0 or fp == 0.0:
            continue
        for lo in range(0, len(b), 1 << 16):
            hi = min(len(b), lo + (1 << 16))
            acc[lo:hi] += fp * np.einsum("ek,ek->e", m[b[lo:hi]], m[a[lo:hi]].conj())
    return 1j * acc


def bond_currents(system, states, f, op=None, sites=None):
    """Bond currents between every pair of coupled sites, each bond once from the site of lower
    index (``bond_currents``, nested.rs:927-1000). With an on-site operator ``op`` (a spin current
    for ``s_z``): ``Re Tr[(O H_ij + H_ij O) G^<_ji]``."""
    _check_f(states, f)
    values = np.asarray(system.values[states.config])
    owner = _owners(system)
    rows = np.repeat(np.arange(system.n, dtype=np.int64), np.diff(system.row_ptr))
    cols = np.asarray(system.cols, dtype=np.int64)
    # Entries the configuration holds (the merged pattern of several configurations keeps zeros).
    keep = (owner[rows] < owner[cols]) & (values != 0)
    r, c, h = rows[keep], cols[keep], values[keep]
    oi, oj = owner[r], owner[c]
    name = (lambda i: sites[i]) if sites is not None else (lambda i: int(i))
    if op is None:
        contrib = 2.0 * h * _lesser_rows(states, f, c, r)
        key = oi * system.n + oj
        uniq, inv = np.unique(key, return_inverse=True)
        tot = np.zeros(len(uniq), np.complex128)
        np.add.at(tot, inv, contrib)
        return [BondCurrent(name(k // system.n), name(k % system.n), float(v.real)) for k, v in zip(uniq, tot)]
    op = np.asarray(op, np.complex128)
    offs = np.asarray(system.site_offsets)
    norb = np.asarray(system.site_orbitals)
    blocks = {}
    for a, b, v, i, j in zip(r, c, h, oi, oj):
        if op.shape[0] != norb[i] or op.shape[0] != norb[j]:
            raise ValueError("the operator acts on the orbitals of a site")
        blk = blocks.setdefault((int(i), int(j)), np.zeros((norb[i], norb[j]), np.complex128))
        blk[a - offs[i], b - offs[j]] += v
    out = []
    for (i, j), hij in sorted(blocks.items()):
        ri = np.arange(offs[i], offs[i] + norb[i])
        rj = np.arange(offs[j], offs[j] + norb[j])
        g = np.zeros((norb[j], norb[i]), np.complex128)  # G^<_ji
        for m, fp in zip(states.leads, f):
            if m.shape[1]:
                g += fp * (m[rj] @ m[ri].conj().T)
        g *= 1j
        w = op @ hij + hij @ op
        out.append(BondCurrent(name(i), name(j), float(np.sum(w * g.T).real)))
    return out


def site_densities(system, states, f, op=None):
    """``Σ_p f_p ψ_p† O ψ_p / 2π`` on each site's orbitals (``site_densities``, nested.rs:1002-1026)."""
    _check_f(states, f)
    offs = np.asarray(system.site_offsets)
    norb = np.asarray(system.site_orbitals)
    out = np.zeros(len(offs))
    op = None if op is None else np.asarray(op, np.complex128)
    for k in np.unique(norb):
        idx = np.nonzero(norb == k)[0]
        if op is not None and op.shape[0] != k:
            raise ValueError("the operator acts on the orbitals of a site")
        rows = offs[idx][:, None] + np.arange(k)[None, :]  # sites x k
        acc = np.zeros(len(idx), np.complex128)
        for m, fp in zip(states.leads, f):
            if m.shape[1] == 0:
                continue
            psi = m[rows]  # sites x k x channels
            if op is None:
                acc += fp * np.sum(np.abs(psi) ** 2, axis=(1, 2))
            else:
                acc += fp * np.einsum("sak,ab,sbk->s", psi.conj(), op, psi)
        out[idx] = acc.real / (2.0 * np.pi)
    return out
