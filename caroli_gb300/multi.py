"""``NestedMultiTerminal``: devices with any number of leads, T_pq between every pair.

Mirrors ``caroli_green::NestedMultiTerminal`` (``crates/caroli-green/src/nested_multi.rs``) and the
lead attachment of ``MultiTerminal`` (``crates/caroli-green/src/multi.rs``):

- each lead continues an interface slice outward with the clean lead model; it couples to every
  device orbital its first cell reaches (``attach_leads``, multi.rs:113-140);
- sites with an orbital coupled to a lead stay at the root of the elimination tree; the others
  form the tree (nested_multi.rs:64-77);
- independent blocks are the connected components of the device, the lead cells and their
  couplings; each block keeps the part of every lead it reaches (:79-146);
- Σ_p = V_p g_p V_p^† with the surface Green's function g_p = (z - h00 - Σ_rest)^-1 of lead p
  (multi.rs:43-55), once per distinct lead (:188-224);
- T_pq = Tr[Γ_p G_pq Γ_q G_pq^†] from the root inverse on the kept orbitals (:337-364), on the GPU
  (``caroli_multi_transmissions``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.sparse import coo_matrix
from scipy.sparse.csgraph import connected_components

from . import _native
from .lattice import Region
from .leads import GreenError, LeadSolver
from .model import Model
from .nested import context
from .precision import Precision
from .system import Block, System, merge_patterns


@dataclass
class Interface:
    """One lead's interface: the device sites of the slice and the lattice step pointing away
    from the device (``Interface``, multi.rs:68-73)."""

    slice: Region
    outward: tuple


@dataclass
class AttachedLead:
    """A semi-infinite lead: cell Hamiltonian, coupling to the next cell outward, the device
    orbitals its first cell couples to and that coupling (``AttachedLead``, multi.rs:14-25)."""

    h00: np.ndarray
    h01: np.ndarray
    orbitals: np.ndarray
    coupling: np.ndarray
    cell: np.ndarray = None  # indices of these cell orbitals in the full lead cell (a block's part)


def attach_leads(lead: Model, region: Region, interfaces) -> list:
    """The leads of ``interfaces`` on ``region`` (multi.rs:113-140, without a magnetic field)."""
    out = []
    for itf in interfaces:
        step = tuple(int(c) for c in itf.outward) + (0,) * (3 - len(itf.outward))
        first = itf.slice.translated(step)
        if any(region.index_of(s) is not None for s in first.sites):
            raise ValueError("the first lead cell overlaps the device")
        skip = lead.coupling(itf.slice, itf.slice.translated(tuple(2 * c for c in step)))
        if np.abs(skip).max(initial=0.0) != 0.0:
            raise ValueError("a lead hopping reaches beyond the next cell")
        h00 = lead.hamiltonian(itf.slice)
        h01 = lead.coupling(itf.slice, first)
        v = lead.coupling(region, first)
        orbitals = np.nonzero(np.any(v != 0, axis=1))[0].astype(np.int64)
        out.append(AttachedLead(h00, h01, orbitals, v[orbitals]))
    return out


@dataclass
class MultiSelfEnergies:
    """Σ_p of every block and lead at one energy (None where a block does not reach a lead)."""

    energy: float
    blocks: list  # [[Σ_p or None per lead] per block]


class NestedMultiTerminal:
    def __init__(self, system: System, block_leads, nleads, device: int = 0):
        self.system = system
        self.block_leads = block_leads  # [[AttachedLead or None per lead] per block]
        self.nleads = nleads
        self.device = device
        self.sites = None
        self._plan = None
        self._slot_of = {}
        # One mode solver per distinct lead cell (nested_multi.rs:126-145).
        self._solvers = []
        cache = []
        for leads in block_leads:
            row = []
            for l in leads:
                if l is None:
                    row.append(None)
                    continue
                twin = next((s for (h0, h1, s) in cache if np.array_equal(h0, l.h00) and np.array_equal(h1, l.h01)),
                            None)
                if twin is None:
                    twin = LeadSolver(l.h00, l.h01)
                    cache.append((l.h00, l.h01, twin))
                row.append(twin)
            self._solvers.append(row)

    # -- construction (nested_multi.rs:61-153) -----------------------------------------------
    @staticmethod
    def from_model(device_model, lead, region, interfaces, device=0):
        return NestedMultiTerminal.from_models([device_model], lead, region, interfaces, device)

    @staticmethod
    def from_models(device_models, lead, region, interfaces, device=0):
        """One system per disorder configuration of the same geometry and leads."""
        mats = [d.sparse_hamiltonian(region) for d in device_models]
        row_ptr, cols, values = merge_patterns(mats)
        n = region.orbitals
        leads = attach_leads(lead, region, interfaces)
        coupled = np.zeros(n, bool)
        for l in leads:
            coupled[l.orbitals] = True
        offs = region.offsets()
        norb = region.site_orbital_counts()
        interior = np.array([i for i in range(len(region)) if not coupled[offs[i]:offs[i] + norb[i]].any()],
                            dtype=np.int64)
        # Components over the device orbitals, then the orbitals of each lead cell.
        offsets, total = [], n
        for l in leads:
            offsets.append(total)
            total += l.h00.shape[0]
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
        nz = np.zeros(len(cols), bool)
        for v in values:
            nz |= v != 0
        ei, ej = [rows[nz]], [cols[nz].astype(np.int64)]
        for l, off in zip(leads, offsets):
            for m in (l.h00, l.h01):
                a, b = np.nonzero(m)
                ei.append(off + a)
                ej.append(off + b)
            a, b = np.nonzero(l.coupling)
            ei.append(l.orbitals[a])
            ej.append(off + b)
        ei, ej = np.concatenate(ei), np.concatenate(ej)
        graph = coo_matrix((np.ones(len(ei)), (ei, ej)), shape=(total, total))
        _, comp = connected_components(graph, directed=True, connection="weak")
        smallest = np.full(comp.max() + 1 if total else 0, total, dtype=np.int64)
        np.minimum.at(smallest, comp, np.arange(total))
        labels = np.full(n, -1, dtype=np.int32)
        blocks, block_leads = [], []
        for c in np.argsort(smallest):
            mine = comp == c
            bl = []
            for l, off in zip(leads, offsets):
                kc = np.nonzero(mine[off:off + l.h00.shape[0]])[0]
                kd = np.nonzero(mine[l.orbitals])[0]
                if len(kc) == 0 or len(kd) == 0:
                    bl.append(None)
                    continue
                bl.append(AttachedLead(l.h00[np.ix_(kc, kc)], l.h01[np.ix_(kc, kc)], l.orbitals[kd],
                                       l.coupling[np.ix_(kd, kc)], kc))
            if all(x is None for x in bl):
                continue
            labels[mine[:n]] = len(blocks)
            kept = np.unique(np.concatenate([x.orbitals for x in bl if x is not None]))
            empty = np.zeros((0, 0), np.complex128)
            blocks.append(Block(left=kept, right=np.zeros(0, np.int64), left_h00=empty, left_h01=empty,
                                right_h00=empty, right_h01=empty))
            block_leads.append(bl)
        system = System(n=n, row_ptr=row_ptr, cols=cols, values=values, dim=region.lattice.dim(),
                        cells=region.cells.copy(), site_offsets=np.asarray(offs, np.int64),
                        site_orbitals=np.asarray(norb, np.int64), range=device_models[0].hopping_range(),
                        interior=interior, labels=labels, blocks=blocks, axis=0)
        out = NestedMultiTerminal(system, block_leads, len(leads), device)
        out.sites = list(region.sites)
        out._region = region
        # For each lead, the index of every orbital of its cell within its site (nested_multi.rs:147-150).
        out.orbital_kinds = [[o for i in range(len(itf.slice)) for o in range(itf.slice.site_orbitals(i))]
                             for itf in interfaces]
        return out

    def lead_count(self):
        return self.nleads

    def region(self):
        """The device region (orbital layout of the scattering states, nested_multi.rs:512-515)."""
        return getattr(self, "_region", None)

    def block_count(self):
        return len(self.system.blocks)

    def config_count(self):
        return self.system.config_count()

    # -- self-energies (nested_multi.rs:188-224, multi.rs:43-55) ---------------------------------
    def surfaces(self, energy):
        """Surface Green's functions g of every block's leads (None where a block has no part of
        a lead), once per distinct lead cell (nested_multi.rs:201-224)."""
        z = complex(energy, 0.0)
        out = []
        for leads, solvers in zip(self.block_leads, self._solvers):
            row, done = [], {}
            for l, s in zip(leads, solvers):
                if l is None:
                    row.append(None)
                    continue
                if id(s) not in done:
                    rest = s.self_energies(energy)[1]
                    m = l.h00.shape[0]
                    done[id(s)] = np.linalg.inv(z * np.eye(m) - l.h00 - rest)
                row.append(done[id(s)])
            out.append(row)
        return out

    def self_energies(self, energy) -> MultiSelfEnergies:
        out = []
        for leads, gs in zip(self.block_leads, self.surfaces(energy)):
            out.append([None if l is None else l.coupling @ g @ l.coupling.conj().T for l, g in zip(leads, gs)])
        return MultiSelfEnergies(float(energy), out)

    def sector_transmissions(self, energy, sectors, config=0, precision=Precision.DOUBLE):
        """Transmissions between sectors of the leads (``sector_transmissions``,
        nested_multi.rs:226-295): ``sectors[p]`` labels the orbitals of each site of lead p (e.g.
        ``[0, 0, 1, 1]`` for the two spins of BHZ) or is None for the lead as a whole. Returns
        ``(labels, t)``: ``labels`` the (lead, sector) of each row and column, ``t[k][l]`` from
        label l into label k."""
        if len(sectors) != self.nleads:
            raise ValueError("one sector labelling per lead")

        def label(p, cell_orbital):
            return 0 if sectors[p] is None else sectors[p][self.orbital_kinds[p][cell_orbital]]

        labels = []
        for p, kinds in enumerate(self.orbital_kinds):
            labels += [(p, a) for a in sorted({label(p, o) for o in range(len(kinds))})]
        sigma = self.self_energies(energy)
        surf = self.surfaces(energy)
        gam = []
        for leads, gs in zip(self.block_leads, surf):
            row = [None] * len(labels)
            for p, (l, g) in enumerate(zip(leads, gs)):
                if l is None:
                    continue
                tags = np.array([label(p, o) for o in l.cell])
                for m in (l.h00, l.h01):
                    if np.any((tags[:, None] != tags[None, :]) & (m != 0)):
                        raise ValueError(f"the Hamiltonian of lead {p} couples different sectors")
                gamma = 1j * (g - g.conj().T)
                for k, (lead, sec) in enumerate(labels):
                    if lead != p:
                        continue
                    sel = tags == sec
                    proj = np.where(sel[:, None] & sel[None, :], gamma, 0.0)
                    row[k] = l.coupling @ proj @ l.coupling.conj().T
            gam.append(row)
        slot = self._slot(sigma)
        t, st = self.plan().multi_sector(slot, config, int(precision), [lab[0] for lab in labels], gam)
        if st != _native.OK:
            raise GreenError("Singular", f"solve status {st} at E = {energy}")
        return labels, t

    # -- GPU plumbing ---------------------------------------------------------------------------
    def plan(self):
        if self._plan is None:
            p = _native.Plan(context(self.device), self.system)
            p.upload_values(self.system.values)
            ptr, orbs = [0], []
            for leads in self.block_leads:
                for l in leads:
                    if l is not None:
                        orbs.extend(l.orbitals.tolist())
                    ptr.append(len(orbs))
            p.multi_leads(self.nleads, ptr, orbs)
            self._plan = p
        return self._plan

    def _slot(self, sigma: MultiSelfEnergies):
        key = id(sigma)
        if key not in self._slot_of or self._slot_of[key][1] is not sigma:
            slot = len(self._slot_of)
            self.plan().upload_multi_sigma(slot, sigma.energy, sigma.blocks)
            self._slot_of[key] = (slot, sigma)
        return self._slot_of[key][0]

    # -- transmissions (nested_multi.rs:163-186) -------------------------------------------------
    def solve_batch(self, sigmas, configs, precision=Precision.DOUBLE):
        """``(T, status)``: T[i] is the nleads x nleads matrix of pair i (from lead q into lead p
        at T[i][p, q])."""
        slots = [self._slot(s) for s in sigmas]
        return self.plan().multi_solve(slots, configs, int(precision), self.nleads)

    def transmissions_with_precision(self, energy, precision=Precision.DOUBLE, config=0):
        t, st = self.solve_batch([self.self_energies(energy)], [config], precision)
        if st[0] != _native.OK:
            raise GreenError("Singular", f"solve status {st[0]} at E = {energy}")
        return t[0]

    def transmissions(self, energy, config=0):
        """``T[p][q] = Tr[Γ_p G_pq Γ_q G_pq^†]`` from lead q into lead p at ``energy``."""
        return self.transmissions_with_precision(energy, Precision.DOUBLE, config)

    def transmissions_batch(self, energies, configs=None, precision=Precision.DOUBLE):
        """T matrices of every (energy, configuration) pair in one GPU batch; a failed point is a
        ``GreenError`` in its place."""
        if configs is None:
            configs = [0] * len(energies)
        sig = {}
        for e in energies:
            if float(e) not in sig:
                sig[float(e)] = self.self_energies(e)
        t, st = self.solve_batch([sig[float(e)] for e in energies], configs, precision)
        return [t[i] if st[i] == _native.OK else GreenError("Singular", f"solve status {st[i]} at E = {e}")
                for i, e in enumerate(energies)]

    # -- scattering matrix (nested_multi.rs:440-495) --------------------------------------------
    def smatrix(self, energy, config=0):
        """Scattering matrix in the basis of the propagating lead modes, from the FP64 root Green's
        function on the GPU (``caroli_root_green``)."""
        from .smatrix import ScatteringLead, assemble, scattering_blocks

        sigma = self.self_energies(energy)
        slot = self._slot(sigma)
        kept = [len(b.left) for b in self.system.blocks]
        greens, st = self.plan().root_green([slot], [config], kept)
        if st[0] != _native.OK:
            raise GreenError("Singular", f"solve status {st[0]} at E = {energy}")
        parts = []
        for blk, leads, solvers, g in zip(self.system.blocks, self.block_leads, self._solvers, greens[0]):
            kept_orbs = np.asarray(blk.left)
            done, sl, h00s = {}, [], []
            for l, s in zip(leads, solvers):
                if l is None:
                    sl.append(None)
                    h00s.append(None)
                    continue
                if id(s) not in done:
                    done[id(s)] = s.modes(energy)
                sl.append(ScatteringLead(np.searchsorted(kept_orbs, l.orbitals), l.coupling, l.h01, done[id(s)],
                                         energy))
                h00s.append(l.h00)
            parts.append(scattering_blocks(g, sl, h00s, energy))
        return assemble(energy, parts)

    # -- scattering states (nested_multi.rs:382-438) and what is built from them --------------
    def scattering_states_batch(self, energies, configs=None):
        """``ScatteringStates`` (one ψ_p per lead) of each (energy, configuration) pair in one GPU
        batch; a failed point is a ``GreenError`` in its place."""
        from .leads import gamma_root
        from .states import ScatteringStates

        if configs is None:
            configs = [0] * len(energies)
        sig = {}
        for e in energies:
            if float(e) not in sig:
                sig[float(e)] = self.self_energies(e)
        sigmas = [sig[float(e)] for e in energies]
        slots = [self._slot(s) for s in sigmas]
        roots = {id(s): [[None if x is None else gamma_root(x) for x in blk] for blk in s.blocks] for s in sigmas}
        outs, st = self.plan().multi_scattering_states(slots, configs, [roots[id(s)] for s in sigmas],
                                                       self.system.n, self.nleads)
        res = []
        for psi, code, e, c in zip(outs, st, energies, configs):
            if code != _native.OK:
                res.append(GreenError("Singular", f"solve status {code} at E = {e}"))
            else:
                res.append(ScatteringStates(float(e), psi, int(c)))
        return res

    def scattering_states(self, energy, config=0):
        """``ψ_p = G W_p`` on every device orbital for every lead (nested_multi.rs:382)."""
        out = self.scattering_states_batch([energy], [config])[0]
        if isinstance(out, GreenError):
            raise out
        return out

    def bond_currents(self, states, f):
        """``2 Re Tr[H_ij G^<_ji]`` of every bond, one occupation per lead (nested_multi.rs:497)."""
        from . import states as st

        return st.bond_currents(self.system, states, f, None, self.sites)

    def operator_currents(self, states, f, op):
        from . import states as st

        return st.bond_currents(self.system, states, f, op, self.sites)

    def site_densities(self, states, f, op=None):
        from . import states as st

        return st.site_densities(self.system, states, f, op)


def lead_voltages(t, currents, ground):
    """Lead voltages in linear response (Landauer–Büttiker) from the transmissions ``t[p][q]`` and
    the currents into the device, lead ``ground`` at zero (``lead_voltages``, multi.rs:148-171):
    I_p = Σ_q (T_qp V_p - T_pq V_q)."""
    t = np.asarray(t, float)
    n = len(t)
    currents = np.asarray(currents, float)
    if currents.shape != (n,):
        raise ValueError("one current per lead")
    if abs(currents.sum()) > 1e-12 * max(np.abs(currents).sum(), 1.0):
        raise ValueError("the currents must add up to zero")

    def g(p, q):
        return sum(t[r][p] for r in range(n) if r != p) if p == q else -t[p][q]

    free = [p for p in range(n) if p != ground]
    a = np.array([[g(i, j) for j in free] for i in free])
    v = np.linalg.solve(a, currents[free])
    out = np.zeros(n)
    out[free] = v
    return out
