"""ORACLE — test infrastructure only (tests). Multi-terminal transmissions by a dense inverse of
the whole device, as ``MultiTerminal::solve`` and ``MultiSolution::transmission``
(``crates/caroli-green/src/multi.rs:88-111``, ``:178-189``): A = E - H - Σ_p Σ_p (each lead's
self-energy on the orbitals it couples to), G = A^-1, T_pq = Tr[Γ_p G_pq Γ_q G_pq^†]. It uses the
full lead cells (no block decomposition), so it also checks the GPU path's split into independent
blocks and its restricted leads. The reference checks NestedMultiTerminal against MultiTerminal
the same way.
"""
from __future__ import annotations

import numpy as np


def dense_h(system, config=0):
    n = system.n
    h = np.zeros((n, n), np.complex128)
    rows = np.repeat(np.arange(n), np.diff(system.row_ptr))
    np.add.at(h, (rows, np.asarray(system.cols, np.int64)), np.asarray(system.values[config]))
    return h


def surface_self_energy(lead, energy):
    """Σ = V g V^† of an attached lead, g = (E - h00 - Σ_rest)^-1 (multi.rs:43-55), with Σ_rest
    the right self-energy of the lead cell from the mode solver."""
    from caroli_gb300.leads import LeadSolver

    rest = LeadSolver(lead.h00, lead.h01).self_energies(energy)[1]
    m = lead.h00.shape[0]
    g = np.linalg.inv(energy * np.eye(m) - lead.h00 - rest)
    return lead.coupling @ g @ lead.coupling.conj().T


def transmissions(system, leads, energy, config=0):
    """T[p][q] of the device `system` (its H values of `config`) with the full attached leads."""
    a = energy * np.eye(system.n) - dense_h(system, config)
    sig = []
    for l in leads:
        s = surface_self_energy(l, energy)
        a[np.ix_(l.orbitals, l.orbitals)] -= s
        sig.append(s)
    g = np.linalg.inv(a)
    nl = len(leads)
    t = np.zeros((nl, nl))
    for p in range(nl):
        gp = 1j * (sig[p] - sig[p].conj().T)
        for q in range(nl):
            gq = 1j * (sig[q] - sig[q].conj().T)
            gpq = g[np.ix_(leads[p].orbitals, leads[q].orbitals)]
            t[p, q] = float(np.real(np.trace(gp @ gpq @ gq @ gpq.conj().T)))
    return t


def spectral(system, leads, energy, config=0):
    """G Γ_p G^† (dense, whole device) of every lead: the spectral function the scattering states
    of lead p carry, ψ_p ψ_p^† (nested_multi.rs:376-381)."""
    a = energy * np.eye(system.n) - dense_h(system, config)
    sig = []
    for l in leads:
        s = surface_self_energy(l, energy)
        a[np.ix_(l.orbitals, l.orbitals)] -= s
        sig.append(s)
    g = np.linalg.inv(a)
    out = []
    for l, s in zip(leads, sig):
        gam = np.zeros((system.n, system.n), np.complex128)
        gam[np.ix_(l.orbitals, l.orbitals)] = 1j * (s - s.conj().T)
        out.append(g @ gam @ g.conj().T)
    return out


def sector_transmissions(system, leads, energy, labels, tags, config=0):
    """t[k][l] = Tr[Γ_k G Γ_l G^†] between (lead, sector) labels (nested_multi.rs:226-295) on the
    whole device: Γ_(p,a) = V_p P_a i(g_p - g_p^†) P_a V_p^† with P_a the projector on the cell
    orbitals of lead p tagged a (`tags[p]`, one tag per cell orbital)."""
    from caroli_gb300.leads import LeadSolver

    a_mat = energy * np.eye(system.n) - dense_h(system, config)
    gcell = []
    for l in leads:
        rest = LeadSolver(l.h00, l.h01).self_energies(energy)[1]
        m = l.h00.shape[0]
        g = np.linalg.inv(energy * np.eye(m) - l.h00 - rest)
        a_mat[np.ix_(l.orbitals, l.orbitals)] -= l.coupling @ g @ l.coupling.conj().T
        gcell.append(g)
    gfull = np.linalg.inv(a_mat)
    gam = []
    for p, a in labels:
        sel = np.asarray(tags[p]) == a
        gc = 1j * (gcell[p] - gcell[p].conj().T)
        proj = np.where(sel[:, None] & sel[None, :], gc, 0.0)
        gam.append(leads[p].coupling @ proj @ leads[p].coupling.conj().T)
    t = np.zeros((len(labels), len(labels)))
    for k, (p, _) in enumerate(labels):
        for l, (q, _) in enumerate(labels):
            gpq = gfull[np.ix_(leads[p].orbitals, leads[q].orbitals)]
            t[k, l] = float(np.real(np.trace(gam[k] @ gpq @ gam[l] @ gpq.conj().T)))
    return t
