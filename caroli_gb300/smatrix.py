"""Scattering matrix in the basis of the propagating lead modes (``SMatrix``,
``crates/caroli-green/src/smatrix.rs``), as ``kwant.smatrix``.

A lead has cells going away from the device with the hopping ``H1`` and couples to the device
through ``V = <device|H|first cell>``. With ``Σ_rest = H1 F`` (the cells beyond the first) and
``g = (E - H0 - Σ_rest)^-1``:
- an incoming mode φ λ^n of lead q acts on the device as the source V_q s, s = φ λ - g H1^† φ;
- the outgoing wave on the first cell of lead p is ψ_1 = g V_p^† G_pq V_q s (minus g H1^† φ in q);
- its amplitude on an outgoing mode a is the current overlap, S = i λ̄_a [a^† Σ_rest ψ_1 - λ̄_a a^† H1^† ψ_1]
  (``scattering_blocks``, smatrix.rs:138-179), modes normalised to unit current.
G_pq comes from the GPU (``caroli_root_green``: the FP64 root Green's function on the kept
orbitals); the mode algebra is small and stays on the host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SMatrix:
    energy: float
    blocks: list    # blocks[p][q]: outgoing modes of lead p x incoming modes of lead q
    incoming: list  # λ of the incoming modes of each lead
    outgoing: list  # λ of the outgoing modes of each lead

    def transmission(self, p, q):
        """Σ |S_pq|²: from lead q into lead p (a reflection for p = q)."""
        return float(np.sum(np.abs(self.blocks[p][q]) ** 2))

    def full(self):
        """Rows: the outgoing modes of every lead in turn; columns: the incoming ones."""
        return np.block([[self.blocks[p][q] for q in range(len(self.incoming))] for p in range(len(self.outgoing))])


@dataclass
class ScatteringLead:
    """A lead of a block: its positions among the kept orbitals, V, the outward hopping H1 and its
    modes ``(right, λ_right, left, λ_left, Σ_rest)`` (``LeadSolver.modes``) at the energy."""

    at: np.ndarray
    coupling: np.ndarray
    h01: np.ndarray
    modes: tuple
    energy: float


def scattering_blocks(green, leads, h00s, energy):
    """``(incoming, outgoing, blocks)`` of one block from its root Green's function ``green``
    (kept x kept) and its leads (``ScatteringLead`` or None) with their cell Hamiltonians ``h00s``."""
    n = len(leads)
    incoming = [np.zeros(0, complex) if l is None else l.modes[3] for l in leads]
    outgoing = [np.zeros(0, complex) if l is None else l.modes[1] for l in leads]
    blocks = [[np.zeros((len(outgoing[p]), len(incoming[q])), complex) for q in range(n)] for p in range(n)]
    gs = [None if l is None else np.linalg.inv(energy * np.eye(len(h0)) - h0 - l.modes[4])
          for l, h0 in zip(leads, h00s)]
    for q in range(n):
        lq = leads[q]
        if lq is None:
            continue
        phi_in, lam_in = lq.modes[2], lq.modes[3]
        back = gs[q] @ (lq.h01.conj().T @ phi_in)
        source = phi_in * lam_in[None, :] - back
        device_source = lq.coupling @ source
        for p in range(n):
            lp = leads[p]
            if lp is None:
                continue
            gpq = green[np.ix_(lp.at, lq.at)]
            psi1 = gs[p] @ (lp.coupling.conj().T @ (gpq @ device_source))
            if p == q:
                psi1 = psi1 - back
            phi_out, lam_out = lp.modes[0], lp.modes[1]
            a = phi_out.conj().T @ (lp.modes[4] @ psi1)
            b = phi_out.conj().T @ (lp.h01.conj().T @ psi1)
            conj = lam_out.conj()[:, None]
            blocks[p][q] = 1j * conj * (a - conj * b)
    return incoming, outgoing, blocks


def assemble(energy, parts):
    """The scattering matrix of independent blocks: a lead's modes are those of every block in
    turn, and blocks do not mix (``SMatrix::assemble``, smatrix.rs:64-96)."""
    n = len(parts[0][0]) if parts else 0
    incoming = [np.concatenate([pt[0][p] for pt in parts]) for p in range(n)]
    outgoing = [np.concatenate([pt[1][p] for pt in parts]) for p in range(n)]
    blocks = []
    for p in range(n):
        row = []
        for q in range(n):
            out = np.zeros((len(outgoing[p]), len(incoming[q])), complex)
            r0 = c0 = 0
            for pt in parts:
                b = pt[2][p][q]
                out[r0:r0 + b.shape[0], c0:c0 + b.shape[1]] = b
                r0 += len(pt[1][p])
                c0 += len(pt[0][q])
            row.append(out)
        blocks.append(row)
    return SMatrix(float(energy), blocks, incoming, outgoing)
