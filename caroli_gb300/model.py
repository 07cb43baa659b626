"""Tight-binding models and the sparse Hamiltonians the transmission path consumes.

Mirrors ``crates/caroli-model`` of caroli:

- ``Model.sparse_hamiltonian`` builds the CSR ``H`` of a region like ``Model::build`` with the
  ``Triplets`` sink (``caroli-model/src/lib.rs:409-470``, ``:687-701``): the full on-site matrix of
  every site (sublattice term plus site-dependent terms, ``:381-389``), then for every site and
  every hopping both the forward block (site is ``from``, partner at ``+offset``) and the backward
  block (site is ``to``, partner at ``-offset``, adjoint matrix); exact zeros are skipped.
- ``SparseMatrix.from_triplets`` sums duplicates and sorts the columns of each row
  (``caroli-model/src/sparse.rs:21-44``); columns are u32 as on the GPU.
- Presets: ``bhz`` (``presets.rs:28-56``), the Γ matrices (``gamma.rs:25-71``), ``bhz_spin`` and
  ``bhz_exchange`` (``presets.rs:67-80``), the benchmark ``square`` and ``graphene`` models
  (``caroli-bench/src/main.rs:76-93``) and a cubic one.

Everything here is vectorised numpy: the 51 200-orbital BHZ ribbon builds in well under a second.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .lattice import Lattice, Region, Site


def _mat(m, n=None):
    a = np.array(m, dtype=np.complex128)
    if a.ndim == 0:
        a = a.reshape(1, 1)
    if n is not None and a.shape != (n, n):
        raise ValueError(f"matrix of shape {a.shape}, expected {(n, n)}")
    return a


@dataclass
class Hopping:
    """``<(R, from)| H |(R + offset, to)> = matrix``; the reverse hop is added automatically."""

    frm: int
    to: int
    offset: tuple
    matrix: np.ndarray


class SparseMatrix:
    """Square complex CSR matrix (``caroli-model/src/sparse.rs:11-53``)."""

    def __init__(self, n, row_ptr, cols, vals):
        self.n = int(n)
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.cols = np.ascontiguousarray(cols, dtype=np.uint32)
        self.vals = np.ascontiguousarray(vals, dtype=np.complex128)

    @staticmethod
    def from_triplets(n, rows, cols, vals):
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        vals = np.asarray(vals, dtype=np.complex128)
        if len(rows) and (rows.max() >= n or cols.max() >= n or rows.min() < 0 or cols.min() < 0):
            raise ValueError("entry outside the matrix")
        key = rows * n + cols
        order = np.argsort(key, kind="stable")
        key, vals = key[order], vals[order]
        uniq, start = np.unique(key, return_index=True)
        summed = np.add.reduceat(vals, start) if len(vals) else vals
        r = uniq // n
        c = uniq % n
        row_ptr = np.zeros(n + 1, dtype=np.int64)
        np.add.at(row_ptr, r + 1, 1)
        row_ptr = np.cumsum(row_ptr)
        return SparseMatrix(n, row_ptr, c.astype(np.uint32), summed)

    def nnz(self):
        return len(self.vals)

    def row(self, r):
        a, b = self.row_ptr[r], self.row_ptr[r + 1]
        return zip(self.cols[a:b].astype(np.int64), self.vals[a:b])

    def to_dense(self):
        m = np.zeros((self.n, self.n), dtype=np.complex128)
        rows = np.repeat(np.arange(self.n), np.diff(self.row_ptr))
        np.add.at(m, (rows, self.cols.astype(np.int64)), self.vals)
        return m

    def with_values(self, vals):
        return SparseMatrix(self.n, self.row_ptr, self.cols, vals)


class OnSiteMap:
    """Site-dependent on-site matrices, summed when a site is added twice
    (``caroli-disorder/src/lib.rs:134-150``)."""

    def __init__(self):
        self.map = {}

    def add(self, site: Site, m):
        m = _mat(m)
        if site in self.map:
            self.map[site] = self.map[site] + m
        else:
            self.map[site] = m.copy()

    def __call__(self, site):
        return self.map.get(site)


class Model:
    """Tight-binding model on a lattice (``caroli-model/src/lib.rs:189-470``)."""

    def __init__(self, lattice: Lattice):
        self.lattice = lattice
        self.onsite_m = [np.zeros((s.orbitals, s.orbitals), np.complex128) for s in lattice.sublattices]
        self.hoppings: list[Hopping] = []
        self.extra = []
        self.hopping_terms = []

    def clone(self):
        m = Model(self.lattice)
        m.onsite_m = [x.copy() for x in self.onsite_m]
        m.hoppings = list(self.hoppings)
        m.extra = list(self.extra)
        m.hopping_terms = list(self.hopping_terms)
        return m

    def onsite(self, sub, matrix):
        self.onsite_m[sub] = _mat(matrix, self.lattice.sublattices[sub].orbitals)
        return self

    def hopping(self, frm, to, offset, matrix):
        subs = self.lattice.sublattices
        m = np.array(matrix, dtype=np.complex128)
        if m.ndim == 0:
            m = m.reshape(1, 1)
        if m.shape != (subs[frm].orbitals, subs[to].orbitals):
            raise ValueError("hopping matrix of the wrong shape")
        offset = tuple(int(x) for x in (list(offset) + [0, 0, 0])[:3])
        if offset == (0, 0, 0) and frm == to:
            raise ValueError("an on-site term is not a hopping")
        self.hoppings.append(Hopping(frm, to, offset, m))
        return self

    def with_onsite_term(self, term):
        """A callable ``site -> matrix | None`` (disorder, potentials), e.g. an ``OnSiteMap``."""
        m = self.clone()
        m.extra.append(term)
        return m

    def with_hopping_term(self, term):
        """A callable ``(from_site, to_site, t) -> matrix | None`` (bond disorder)."""
        m = self.clone()
        m.hopping_terms.append(term)
        return m

    def with_peierls(self, phase):
        """Peierls phases: the block <i|H|j> times exp(i phase(r_i, r_j)) (``Model::with_peierls``,
        ``caroli-model/src/lib.rs:276-280``, ``:369-378``), ``r`` the sites' positions."""
        lat = self.lattice

        def term(frm, to, t):
            return t * np.exp(1j * phase(lat.position(frm), lat.position(to)))

        return self.with_hopping_term(term)

    def with_field(self, b):
        """A uniform field b z in the Landau gauge A = (-b y, 0, 0) (``gauge::landau_x``,
        ``caroli-model/src/lib.rs:157-164``): invariant along x, so for leads along x."""
        return self.with_peierls(landau_x(b))

    def onsite_matrix(self, site: Site):
        m = self.onsite_m[site.sub].copy()
        for term in self.extra:
            v = term(site)
            if v is not None:
                m = m + _mat(v)
        return m

    def _hop_matrix(self, hop, frm_site, to_site):
        m = hop.matrix
        for term in self.hopping_terms:
            v = term(frm_site, to_site, m)
            if v is not None:
                m = _mat(v) if np.ndim(v) else np.array([[v]], np.complex128)
        return m

    # -- builders ---------------------------------------------------------------------------
    def _onsite_blocks(self, region: Region):
        """Per-site full on-site matrices as a list aligned with the region."""
        if not self.extra:
            return [self.onsite_m[s.sub] for s in region.sites]
        return [self.onsite_matrix(s) for s in region.sites]

    def _couplings(self, a: Region, b: Region):
        """Hopping blocks from sites of ``a`` to sites of ``b``: forward and backward ends of
        every hopping (``lib.rs:532-553``). Yields ``(i, j, matrix)`` with ``i`` in ``a``."""
        if len(a) == 0 or len(b) == 0:
            return
        cells_a, subs_a = a.cells, a.subs
        keys_b = _site_keys(b.cells, b.subs)
        order = np.argsort(keys_b)
        sorted_keys = keys_b[order]
        for hop in self.hoppings:
            off = np.array(hop.offset, dtype=np.int64)
            for sign, sel_sub, partner_sub, adjoint in ((1, hop.frm, hop.to, False), (-1, hop.to, hop.frm, True)):
                idx = np.nonzero(subs_a == sel_sub)[0]
                if len(idx) == 0:
                    continue
                pc = cells_a[idx] + sign * off
                pk = _site_keys(pc, np.full(len(idx), partner_sub))
                pos = np.searchsorted(sorted_keys, pk)
                pos = np.minimum(pos, len(sorted_keys) - 1)
                found = sorted_keys[pos] == pk
                # One matrix object per hopping and direction when no term depends on the bond
                # (the builder groups identical blocks by object).
                fixed = hop.matrix.conj().T.copy() if adjoint else hop.matrix
                for i, j in zip(idx[found], order[pos[found]]):
                    if self.hopping_terms:
                        si, sj = a.sites[i], b.sites[j]
                        m = self._hop_matrix(hop, sj, si).conj().T if adjoint else self._hop_matrix(hop, si, sj)
                    else:
                        m = fixed
                    yield int(i), int(j), m

    def sparse_hamiltonian(self, region: Region) -> SparseMatrix:
        rows, cols, vals = [], [], []
        offs = region.offsets()
        orbs = region.site_orbital_counts()
        # On-site blocks, vectorised by orbital count when no site-dependent term applies.
        blocks = self._onsite_blocks(region)
        for i, m in enumerate(blocks):
            o = offs[i]
            nz = np.nonzero(m)
            rows.append(o + nz[0]); cols.append(o + nz[1]); vals.append(m[nz])
        # Hoppings: group identical blocks to build index arrays in bulk.
        hop_i, hop_j, hop_m = [], [], []
        for i, j, m in self._couplings(region, region):
            hop_i.append(i); hop_j.append(j); hop_m.append(m)
        if hop_i:
            hop_i = np.array(hop_i); hop_j = np.array(hop_j)
            # Blocks share few distinct matrices: bucket by identity.
            ids = {}
            bucket = np.array([ids.setdefault(id(m), len(ids)) for m in hop_m])
            mats = {}
            for m in hop_m:
                mats.setdefault(id(m), m)
            for key, b in ids.items():
                m = mats[key]
                sel = bucket == b
                nz = np.nonzero(m)
                ii, jj = hop_i[sel], hop_j[sel]
                r = offs[ii][:, None] + nz[0][None, :]
                c = offs[jj][:, None] + nz[1][None, :]
                rows.append(r.ravel()); cols.append(c.ravel())
                vals.append(np.broadcast_to(m[nz], r.shape).ravel())
        rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
        cols = np.concatenate(cols) if cols else np.zeros(0, np.int64)
        vals = np.concatenate(vals) if vals else np.zeros(0, np.complex128)
        keep = vals != 0
        return SparseMatrix.from_triplets(region.orbitals, rows[keep], cols[keep], vals[keep])

    def hamiltonian(self, region: Region):
        """Dense Hamiltonian of a finite region (open boundaries)."""
        return self.sparse_hamiltonian(region).to_dense()

    def coupling(self, a: Region, b: Region):
        """``<a| H |b>`` between two disjoint regions (rows ``a``, columns ``b``)."""
        h = np.zeros((a.orbitals, b.orbitals), np.complex128)
        oa, ob = a.offsets(), b.offsets()
        for i, j, m in self._couplings(a, b):
            h[oa[i]:oa[i] + m.shape[0], ob[j]:ob[j] + m.shape[1]] += m
        return h

    def hopping_range(self):
        """Largest |offset| of any hopping along each axis, at least 1 (``nested.rs:61-67``)."""
        r = [1, 1, 1]
        for hop in self.hoppings:
            for d in range(3):
                r[d] = max(r[d], abs(hop.offset[d]))
        return r


def _site_keys(cells, subs):
    c = np.asarray(cells, dtype=np.int64) + (1 << 19)
    return ((c[:, 0] << 42) | (c[:, 1] << 22) | (c[:, 2] << 2)) * 64 + np.asarray(subs, dtype=np.int64)


# -- Pauli and Γ matrices (gamma.rs:1-71) --------------------------------------------------------
O, L, I = 0.0, 1.0, 1j


def s0():
    return np.eye(2, dtype=np.complex128)


def sx():
    return np.array([[0, 1], [1, 0]], np.complex128)


def sy():
    return np.array([[0, -1j], [1j, 0]], np.complex128)


def sz():
    return np.array([[1, 0], [0, -1]], np.complex128)


def kron(a, b):
    return np.kron(a, b)


def gamma0():
    return np.eye(4, dtype=np.complex128)


def gamma12():
    return np.diag([1, 1, -1, -1]).astype(np.complex128)


def gamma12p():
    return np.diag([1, -1, -1, 1]).astype(np.complex128)


def gamma13():
    return np.array([[O, O, I, O], [O, O, O, I], [-I, O, O, O], [O, -I, O, O]], np.complex128)


def gamma14():
    return np.array([[O, O, L, O], [O, O, O, -L], [L, O, O, O], [O, -L, O, O]], np.complex128)


def gamma23():
    return np.array([[O, O, L, O], [O, O, O, L], [L, O, O, O], [O, L, O, O]], np.complex128)


def gamma23p():
    return np.array([[O, O, L, O], [O, O, O, -L], [L, O, O, O], [O, -L, O, O]], np.complex128)


def gamma31():
    return np.array([[O, O, -I, O], [O, O, O, -I], [I, O, O, O], [O, I, O, O]], np.complex128)


def gamma31p():
    return np.array([[O, O, -I, O], [O, O, O, I], [I, O, O, O], [O, -I, O, O]], np.complex128)


def gamma33():
    return np.array([[O, L, O, O], [L, O, O, O], [O, O, O, -L], [O, O, -L, O]], np.complex128)


def gamma44():
    return np.array([[O, -I, O, O], [I, O, O, O], [O, O, O, -I], [O, O, I, O]], np.complex128)


def gamma55():
    return np.diag([1, -1, 1, -1]).astype(np.complex128)


def landau_x(b):
    """Peierls phase of A = (-b y, 0, 0) between positions r_i, r_j: -b (y_i + y_j) (x_i - x_j) / 2."""
    return lambda ri, rj: -b * 0.5 * (ri[1] + rj[1]) * (ri[0] - rj[0])


def combine(terms):
    """``Σ_i c_i M_i`` (``caroli-model/src/lib.rs:703-708``)."""
    out = np.zeros_like(terms[0][1], dtype=np.complex128)
    for c, m in terms:
        out = out + complex(c) * m
    return out


@dataclass(frozen=True)
class BhzParams:
    """HgTe quantum-well parameters in units of A/a (``presets.rs:7-26``)."""

    a: float = 1.0
    b: float = -0.376406
    c: float = 0.0
    d: float = -0.280933
    mass: float = -0.137
    lam: float = 0.0


def bhz(p: BhzParams = BhzParams()):
    """BHZ on a square lattice, basis (E1↑, H1↑, E1↓, H1↓) (``presets.rs:28-56``)."""
    onsite = combine([(p.c - 4.0 * p.d, gamma0()), (p.mass - 4.0 * p.b, gamma55())])
    tx = combine([(p.d, gamma0()), (p.b, gamma55()), (-0.5j * p.a, gamma33()), (0.5j * p.lam, gamma13())])
    ty = combine([(p.d, gamma0()), (p.b, gamma55()), (0.5j * p.a, gamma44()), (-0.5j * p.lam, gamma14())])
    return Model(Lattice.square(1.0, 4)).onsite(0, onsite).hopping(0, 0, [1, 0, 0], tx).hopping(0, 0, [0, 1, 0], ty)


def bhz_spin(coupling="opposite-g"):
    """Spin matrices coupled to a classical moment (``presets.rs:67-74``)."""
    if coupling in ("same", "same-g"):
        return [gamma23(), gamma31(), gamma12()]
    if coupling in ("opposite", "opposite-g"):
        return [gamma23p(), gamma31p(), gamma12p()]
    if coupling == "pauli":
        return [sx(), sy(), sz()]
    raise ValueError(f"unknown spin coupling {coupling}")


def bhz_exchange(coupling, j, n):
    sxm, sym, szm = bhz_spin(coupling)
    return combine([(j * n[0], sxm), (j * n[1], sym), (j * n[2], szm)])


def square(t=1.0, orbitals=1):
    """Square lattice with hopping ``-t`` (the benchmark ``square`` model)."""
    e = -t * np.eye(orbitals)
    return Model(Lattice.square(1.0, orbitals)).hopping(0, 0, [1, 0, 0], e).hopping(0, 0, [0, 1, 0], e)


def cubic(t=1.0, orbitals=1):
    """Simple cubic lattice with hopping ``-t`` along x, y and z."""
    e = -t * np.eye(orbitals)
    m = Model(Lattice.cubic(1.0, orbitals))
    for off in ([1, 0, 0], [0, 1, 0], [0, 0, 1]):
        m = m.hopping(0, 0, off, e)
    return m


def graphene(t=1.0):
    """Honeycomb, transport along a zigzag direction (``caroli-bench/src/main.rs:88-91``)."""
    return (
        Model(Lattice.honeycomb(1.0, 1))
        .hopping(0, 1, [0, 0, 0], -t)
        .hopping(0, 1, [0, -1, 0], -t)
        .hopping(0, 1, [1, -1, 0], -t)
    )
