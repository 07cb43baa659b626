"""Host description of a two-terminal system: what the C ABI uploads.

``build_system`` follows ``NestedTwoTerminal::from_model`` (``crates/caroli-green/src/nested.rs:530-610``):

- ``H`` is the device's sparse Hamiltonian on the region (CSR, u32 columns);
- both leads continue the first and last slices along ``axis`` with the clean lead model:
  ``h00 = <cell|H|cell>`` and ``h01 = <cell|H|cell + step>`` of the lead model, checked to be the
  same one cell further along the lead (``gauge.rs:78-98``);
- the tree covers the interior sites (all but the two lead slices, ``nested.rs:559-563``);
- independent blocks of orbitals are the connected components of the nonzero entries of ``H``
  and of the lead matrices (union-find, label = smallest member, ``nested.rs:565-608``); blocks
  without orbitals on both slices are dropped.

Several disorder configurations of one geometry share one description: their CSR patterns are
merged (union of the nonzero positions) and each configuration keeps a value array on the merged
pattern, zero where it has no entry.  Blocks are computed on the merged pattern.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from scipy.sparse import coo_matrix
from scipy.sparse.csgraph import connected_components

from .lattice import Region
from .model import Model, SparseMatrix


@dataclass
class Block:
    """One independent block: its device orbitals on the two lead slices (lead-cell order) and
    the lead matrices restricted to them."""

    left: np.ndarray
    right: np.ndarray
    left_h00: np.ndarray
    left_h01: np.ndarray
    right_h00: np.ndarray
    right_h01: np.ndarray

    def same_lead(self):
        return (
            self.left_h00.shape == self.right_h00.shape
            and np.array_equal(self.left_h00, self.right_h00)
            and np.array_equal(self.left_h01, self.right_h01)
        )


@dataclass
class System:
    n: int
    row_ptr: np.ndarray
    cols: np.ndarray
    values: list  # one complex128 array per configuration, on the merged pattern
    dim: int
    cells: np.ndarray  # (nsites, 3) int64
    site_offsets: np.ndarray
    site_orbitals: np.ndarray
    range: list
    interior: np.ndarray
    labels: np.ndarray  # block index of each orbital, -1 for orbitals of dropped blocks
    blocks: list = field(default_factory=list)
    axis: int = 0

    @property
    def nnz(self):
        return int(self.row_ptr[-1])

    def config_count(self):
        return len(self.values)

    def block_rows(self, b):
        """Orbitals of block ``b`` (sorted)."""
        return np.nonzero(self.labels == b)[0]


def merge_patterns(mats):
    """Union CSR pattern of several matrices of one size, and each one's values on it."""
    n = mats[0].n
    keys = []
    for m in mats:
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(m.row_ptr))
        keys.append(rows * n + m.cols.astype(np.int64))
    union = np.unique(np.concatenate(keys)) if len(mats) > 1 else keys[0]
    rows = union // n
    cols = (union % n).astype(np.uint32)
    row_ptr = np.zeros(n + 1, np.int64)
    np.add.at(row_ptr, rows + 1, 1)
    row_ptr = np.cumsum(row_ptr)
    vals = []
    for m, k in zip(mats, keys):
        v = np.zeros(len(union), np.complex128)
        v[np.searchsorted(union, k)] = m.vals
        vals.append(v)
    return row_ptr, cols, vals


def lead_cell(lead: Model, cell: Region, step, along):
    """``(h00, h01)`` of the lead at ``cell``; checks that one cell further along the lead gives
    the same matrices (``gauge.rs:78-98``)."""
    def pair(c):
        nxt = c.translated(step)
        return lead.hamiltonian(c), lead.coupling(c, nxt)

    h00, h01 = pair(cell)
    h00n, h01n = pair(cell.translated(along))
    tol = 1e-12 * max(np.abs(h00).max(initial=0.0), np.abs(h01).max(initial=0.0))
    if np.abs(h00 - h00n).max(initial=0.0) > tol or np.abs(h01 - h01n).max(initial=0.0) > tol:
        raise ValueError("the lead model changes along the lead")
    return h00, h01


def build_system(devices, lead: Model, region: Region, axis: int, extra: SparseMatrix = None) -> System:
    """The description of ``devices`` (one model per disorder configuration, same geometry).
    ``extra``: entries added to the pattern (zero in every configuration) and counted as couplings
    for the blocks, e.g. the on-site entries that disorder generated on the device can fill."""
    if isinstance(devices, Model):
        devices = [devices]
    for hop in lead.hoppings:
        if abs(hop.offset[axis]) > 1:
            raise ValueError(f"a lead hopping skips a cell along axis {axis}")
    mats = [d.sparse_hamiltonian(region) for d in devices]
    if extra is not None:
        row_ptr, cols, values = merge_patterns(mats + [extra])
        structural = values.pop() != 0
    else:
        row_ptr, cols, values = merge_patterns(mats)
        structural = None
    n = region.orbitals
    slices = region.slices(axis)
    first, last = slices[0], slices[-1]
    step = [0, 0, 0]
    step[axis] = 1
    back = [-x for x in step]
    lh00, lh01 = lead_cell(lead, first, step, back)
    rh00, rh01 = lead_cell(lead, last, step, step)

    def orbitals_of(s: Region):
        out = []
        for site in s.sites:
            i = region.index_of(site)
            o = region.offset(i)
            out.extend(range(o, o + region.site_orbitals(i)))
        return np.array(out, dtype=np.int64)

    left_orbs, right_orbs = orbitals_of(first), orbitals_of(last)
    ends = {first.sites[0].cell[axis], last.sites[0].cell[axis]}
    interior = np.array([i for i, s in enumerate(region.sites) if s.cell[axis] not in ends], dtype=np.int64)

    # Components of the nonzero entries of H (any configuration) and of the lead matrices.
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
    nz = np.zeros(len(cols), bool) if structural is None else structural.copy()
    for v in values:
        nz |= v != 0
    ei, ej = [rows[nz]], [cols[nz].astype(np.int64)]
    for h, orbs in ((lh00, left_orbs), (lh01, left_orbs), (rh00, right_orbs), (rh01, right_orbs)):
        a, b = np.nonzero(h)
        ei.append(orbs[a]); ej.append(orbs[b])
    ei, ej = np.concatenate(ei), np.concatenate(ej)
    graph = coo_matrix((np.ones(len(ei)), (ei, ej)), shape=(n, n))
    _, comp = connected_components(graph, directed=True, connection="weak")
    # Label of a component: its smallest member; blocks in increasing label order.
    smallest = np.full(comp.max() + 1 if n else 0, n, dtype=np.int64)
    np.minimum.at(smallest, comp, np.arange(n))
    order = np.argsort(smallest)
    labels = np.full(n, -1, dtype=np.int32)
    blocks = []
    for c in order:
        mine = comp == c
        kl = np.nonzero(mine[left_orbs])[0]
        kr = np.nonzero(mine[right_orbs])[0]
        if len(kl) == 0 or len(kr) == 0:
            continue
        labels[mine] = len(blocks)
        blocks.append(
            Block(
                left=left_orbs[kl],
                right=right_orbs[kr],
                left_h00=lh00[np.ix_(kl, kl)],
                left_h01=lh01[np.ix_(kl, kl)],
                right_h00=rh00[np.ix_(kr, kr)],
                right_h01=rh01[np.ix_(kr, kr)],
            )
        )
    return System(
        n=n,
        row_ptr=row_ptr,
        cols=cols,
        values=values,
        dim=region.lattice.dim(),
        cells=region.cells.copy(),
        site_offsets=np.asarray(region.offsets(), np.int64),
        site_orbitals=np.asarray(region.site_orbital_counts(), np.int64),
        range=devices[0].hopping_range(),
        interior=interior,
        labels=labels,
        blocks=blocks,
        axis=axis,
    )
