"""Lattices, finite regions and transport slices.

Mirrors ``crates/caroli-lattice/src/lib.rs`` of caroli: a ``Region`` is an ordered set of
``Site`` objects that fixes the orbital order of every matrix built on it (site ``i`` owns the
orbitals ``offset(i) .. offset(i) + site_orbitals(i)``).  ``Region.cuboid`` orders sites with the
first axis slowest and the sublattice fastest (lib.rs:122-140); ``Region.slices`` groups sites by
their cell coordinate along an axis, keeping the region order (lib.rs:185-194).

The site order is what the elimination tree and the front variable lists index, so it must be
identical to the reference's for the same input.
"""
from __future__ import annotations

from dataclasses import dataclass
import math

import numpy as np


@dataclass(frozen=True, order=True)
class Site:
    """A unit cell (three integer coordinates, unused axes 0) and a sublattice index."""

    cell: tuple
    sub: int


@dataclass
class Sublattice:
    name: str
    offset: tuple
    orbitals: int


class Lattice:
    """Bravais lattice with a basis (``caroli-lattice/src/lib.rs:25-87``)."""

    def __init__(self, vectors):
        vectors = [tuple(float(x) for x in v) for v in vectors]
        if not 1 <= len(vectors) <= 3:
            raise ValueError("a lattice has 1, 2 or 3 primitive vectors")
        self.vectors = vectors
        self.sublattices: list[Sublattice] = []

    def with_sublattice(self, name, offset, orbitals):
        if orbitals <= 0:
            raise ValueError("a sublattice carries at least one orbital")
        self.sublattices.append(Sublattice(name, tuple(float(x) for x in offset), int(orbitals)))
        return self

    @staticmethod
    def square(a=1.0, orbitals=1):
        return Lattice([[a, 0.0, 0.0], [0.0, a, 0.0]]).with_sublattice("A", [0.0, 0.0, 0.0], orbitals)

    @staticmethod
    def cubic(a=1.0, orbitals=1):
        return Lattice([[a, 0.0, 0.0], [0.0, a, 0.0], [0.0, 0.0, a]]).with_sublattice("A", [0.0] * 3, orbitals)

    @staticmethod
    def honeycomb(a=1.0, orbitals=1):
        s3 = math.sqrt(3.0)
        return (
            Lattice([[s3 * a, 0.0, 0.0], [0.5 * s3 * a, 1.5 * a, 0.0]])
            .with_sublattice("A", [0.0, 0.0, 0.0], orbitals)
            .with_sublattice("B", [0.0, a, 0.0], orbitals)
        )

    def dim(self):
        return len(self.vectors)

    def position(self, site: Site):
        r = list(self.sublattices[site.sub].offset)
        for n, v in zip(site.cell, self.vectors):
            for c in range(3):
                r[c] += n * v[c]
        return tuple(r)


class Region:
    """Finite ordered set of sites (``caroli-lattice/src/lib.rs:96-208``)."""

    def __init__(self, lattice: Lattice, sites):
        self.lattice = lattice
        self.sites = [Site(tuple(int(c) for c in s.cell), int(s.sub)) for s in sites]
        self._index = {}
        for i, s in enumerate(self.sites):
            if not 0 <= s.sub < len(lattice.sublattices):
                raise ValueError(f"unknown sublattice {s.sub}")
            if s in self._index:
                raise ValueError(f"duplicate site {s}")
            self._index[s] = i
        orbs = np.array([lattice.sublattices[s.sub].orbitals for s in self.sites], dtype=np.int64)
        self._orbs = orbs
        self._offsets = np.concatenate([[0], np.cumsum(orbs)[:-1]]) if len(orbs) else np.zeros(0, np.int64)
        self.orbitals = int(orbs.sum())
        # Arrays for vectorised builders: cells (n, 3) and sublattices (n,).
        self.cells = np.array([s.cell for s in self.sites], dtype=np.int64).reshape(-1, 3)
        self.subs = np.array([s.sub for s in self.sites], dtype=np.int64)

    @staticmethod
    def from_sites(lattice, sites):
        return Region(lattice, sites)

    @staticmethod
    def cuboid(lattice: Lattice, extent):
        """All sites of cells ``0..extent[a]``; first axis slowest, sublattice fastest."""
        dim = lattice.dim()
        n = [int(extent[a]) if a < dim else 1 for a in range(3)]
        nsub = len(lattice.sublattices)
        sites = [
            Site((i, j, k), s)
            for i in range(n[0])
            for j in range(n[1])
            for k in range(n[2])
            for s in range(nsub)
        ]
        return Region(lattice, sites)

    def __len__(self):
        return len(self.sites)

    def index_of(self, site: Site):
        return self._index.get(site)

    def offset(self, i):
        return int(self._offsets[i])

    def site_orbitals(self, i):
        return int(self._orbs[i])

    def offsets(self):
        return self._offsets

    def site_orbital_counts(self):
        return self._orbs

    def slices(self, axis):
        """Slices along ``axis``: by increasing cell coordinate, region order kept."""
        coords = sorted({s.cell[axis] for s in self.sites})
        return [Region(self.lattice, [s for s in self.sites if s.cell[axis] == c]) for c in coords]

    def translated(self, cells):
        return Region(
            self.lattice,
            [Site(tuple(s.cell[a] + cells[a] for a in range(3)), s.sub) for s in self.sites],
        )
