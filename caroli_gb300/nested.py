"""``NestedTwoTerminal``: the drop-in host face of the GB300 transmission path.

Mirrors the public API of ``caroli_green::NestedTwoTerminal`` (``crates/caroli-green/src/nested.rs``):

=============================  ==========================================================
reference                      here
=============================  ==========================================================
``from_model`` :530            ``NestedTwoTerminal.from_model`` (and ``from_models`` for a
                               batch of disorder configurations of one geometry)
``block_count`` :613           ``block_count``
``transmission`` :618          ``transmission``
``transmissions`` :623         ``transmissions`` (one batched GPU launch sequence)
``transmissions_checked`` :630 ``transmissions_checked``
``self_energies`` :652         ``self_energies`` -> ``LeadSelfEnergies``
``transmission_with`` :682     ``transmission_with``
``transmission_with_precision``  ``transmission_with_precision``
  :688
``scattering_states`` :851     ``scattering_states`` (and ``scattering_states_batch``)
``bond_currents`` :903         ``bond_currents``, ``operator_currents``
``site_densities`` :916        ``site_densities``
=============================  ==========================================================

The elimination and the trace run on the GPU through ``libcaroli_gb300.so``; the lead
self-energies are computed on the host (``leads.py``), once per energy, and reused for every
configuration as the reference does (``self_energies`` doc, nested.rs:643-651). A failed solve
raises ``GreenError("Singular", …)`` as ``GreenError::Singular`` (nested.rs:798-800).
"""
from __future__ import annotations

import contextlib
import math
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _native
from . import states as _states
from .states import ScatteringStates
from .leads import GreenError, LeadSolver, gamma_root
from .precision import Precision, PrecisionOptions, checked
from .system import System, build_system


@dataclass
class LeadSelfEnergies:
    """Self-energies of every block at one energy (``nested.rs:436-459``)."""

    energy: float
    blocks: list  # [(Σ_L, Σ_R)] per block

    def key(self):
        return id(self)

    def w_right(self):
        """Per block, W_R with W_R W_R^† = Γ_R (the mixed path's right-hand sides)."""
        if not hasattr(self, "_w_right"):
            self._w_right = [gamma_root(sr) for _, sr in self.blocks]
        return self._w_right

    def w_left(self):
        """Per block, W_L with W_L W_L^† = Γ_L (the sources of the left lead's scattering states)."""
        if not hasattr(self, "_w_left"):
            self._w_left = [gamma_root(sl) for sl, _ in self.blocks]
        return self._w_left


@dataclass
class ModeSelfEnergies:
    """Self-energies of every block at one energy, to be formed on the GPU from the leads' modes
    (``caroli_sigma_from_modes``): per block ``(1/λ_L, λ_R, open channels, channel weights)`` of
    leads with a scalar coupling (the definite fast path of ``modes.rs:540-710``)."""

    energy: float
    blocks: list

    def key(self):
        return id(self)


_CONTEXTS = {}


def context(device=0):
    """The shared device context of ``device`` (created on first use)."""
    if device not in _CONTEXTS:
        _CONTEXTS[device] = _native.Context(device)
    return _CONTEXTS[device]


class NestedTwoTerminal:
    def __init__(self, system: System, device: int = 0):
        self.system = system
        self.device = device
        self._solvers = []
        for b in system.blocks:
            left = LeadSolver(b.left_h00, b.left_h01)
            right = left if b.same_lead() else LeadSolver(b.right_h00, b.right_h01)
            self._solvers.append((left, right))
        self._plan = None
        self._slot_of = {}
        self.sites = None  # the region's sites, when built from a region (names of bond ends)

    # -- construction -------------------------------------------------------------------------
    @staticmethod
    def from_model(device_model, lead, region, axis, device=0):
        out = NestedTwoTerminal(build_system([device_model], lead, region, axis), device)
        out.sites = list(region.sites)
        out._region = region
        return out

    @staticmethod
    def from_models(device_models, lead, region, axis, device=0):
        """One system per disorder configuration of the same geometry and leads."""
        out = NestedTwoTerminal(build_system(list(device_models), lead, region, axis), device)
        out.sites = list(region.sites)
        out._region = region
        return out

    @staticmethod
    def from_disorder(clean_model, lead, region, axis, entries, nconfigs, first_config=0, device=0):
        """``nconfigs`` disorder configurations of the CLI's ``[[disorder]]`` entries
        (``caroli-cli/src/build.rs:251-310``; the dicts of ``disorder.disordered``) generated on the
        GPU (``caroli_values_generate``): configuration c is the CLI's configuration
        ``first_config + c``. The pattern holds every on-site entry the entries can fill."""
        from . import disorder as dis
        from .model import SparseMatrix

        n = region.orbitals
        offs = region.offsets()
        norb = region.site_orbital_counts()
        touched = {}
        for d in entries:
            if d["kind"] == "anderson":
                for k in set(int(x) for x in norb):
                    touched.setdefault(k, np.zeros((k, k), bool))[np.arange(k), np.arange(k)] = True
            elif d["kind"] == "magnetic":
                mom = d.get("moments", dis.Moments.isotropic())
                spin = [np.asarray(m, np.complex128) for m in d["spin"]]
                k = spin[0].shape[0]
                # n = z exactly for m_z = 1 or a zero cone: only S_z can fill entries.
                only_z = (mom.kind == "polarized" and mom.mz == 1.0) or (mom.kind == "cone" and mom.theta0 == 0.0)
                used = spin[2:] if only_z else spin
                mask = touched.setdefault(k, np.zeros((k, k), bool))
                for m in used:
                    mask |= m != 0
            else:
                raise ValueError(f"unknown disorder {d['kind']}")
        rows, cols = [], []
        for i in range(len(region)):
            mask = touched.get(int(norb[i]))
            if mask is None:
                continue
            a, b = np.nonzero(mask)
            rows.append(offs[i] + a)
            cols.append(offs[i] + b)
        rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
        cols = np.concatenate(cols) if cols else np.zeros(0, np.int64)
        extra = SparseMatrix.from_triplets(n, rows, cols, np.ones(len(rows), np.complex128))
        system = build_system([clean_model], lead, region, axis, extra=extra)
        out = NestedTwoTerminal(system, device)
        out.sites = list(region.sites)
        out._region = region
        out._disorder = (entries, int(nconfigs), int(first_config))
        return out

    def generated_values(self, config):
        """H values of configuration ``config`` as the device holds them (on the system's pattern)."""
        return self.plan().download_values(config, self.system.nnz)

    def block_count(self):
        return len(self.system.blocks)

    def region(self):
        """The device region (orbital layout of the scattering states, nested.rs:920-923), or None
        for a system not built from a region."""
        return getattr(self, "_region", None)

    def config_count(self):
        if getattr(self, "_disorder", None) is not None:
            return self._disorder[1]
        return self.system.config_count()

    # -- self-energies ------------------------------------------------------------------------
    def self_energies(self, energy) -> LeadSelfEnergies:
        blocks = []
        for left, right in self._solvers:
            sl, sr_same, _ = left.self_energies(energy)
            sr = sr_same if right is left else right.self_energies(energy)[1]
            blocks.append((sl, sr))
        return LeadSelfEnergies(float(energy), blocks)

    def self_energies_many(self, energies, threads=None, errors=False):
        """``self_energies`` at many energies, spread over host threads (the reference maps its
        energies in parallel, ``NestedTwoTerminal::transmissions``, nested.rs:622-626): each
        energy's eigenproblems run in LAPACK, which releases the interpreter lock, with the BLAS
        limited to one thread per worker so that the workers do not oversubscribe the cores.
        ``threads`` defaults to the host's cores when ``threadpoolctl`` can set that limit, else to
        one (multithreaded BLAS under several workers was measured slower than one worker). With
        ``errors`` an energy whose modes fail gives its ``GreenError`` in place instead of raising."""
        energies = list(energies)
        try:
            from threadpoolctl import threadpool_limits
        except ImportError:
            threadpool_limits = None

        def one(e):
            try:
                return self.self_energies(e)
            except GreenError as err:
                if errors:
                    return err
                raise

        if threads is None:
            threads = (os.cpu_count() or 1) if threadpool_limits is not None else 1
        threads = max(1, min(int(threads), len(energies)))
        if threads == 1:
            return [one(e) for e in energies]
        limit = threadpool_limits(1) if threadpool_limits is not None else contextlib.nullcontext()
        with limit, ThreadPoolExecutor(max_workers=threads) as pool:
            return list(pool.map(one, energies))

    def self_energies_broadened(self, energy, eta) -> LeadSelfEnergies:
        """Σ at E + iη with the device at the real E (``SelfEnergyMethod::ModesBroadened``,
        caroli-green/src/lib.rs:49-66): no propagating lead mode, as the thesis codes compute it."""
        z = complex(energy, eta)
        blocks = []
        for left, right in self._solvers:
            sl, sr_same, _ = left.self_energies(z)
            sr = sr_same if right is left else right.self_energies(z)[1]
            blocks.append((sl, sr))
        return LeadSelfEnergies(float(energy), blocks)

    def transmission_thesis(self, sigma, config=0):
        """Tr[Re(Γ_L) G Re(Γ_R) G^†]: the thesis' transmission, broadenings truncated to their
        element-wise real part (caroli-validation/src/thesis.rs:84-95), FP64 on the GPU."""
        slot = self._slot(sigma)
        re = [(np.real(1j * (sl - sl.conj().T)).astype(np.complex128),
               np.real(1j * (sr - sr.conj().T)).astype(np.complex128)) for sl, sr in sigma.blocks]
        self.plan().gamma_override(slot, re)
        try:
            t, st, _ = self.plan().solve([slot], [config], int(Precision.DOUBLE))
        finally:
            # The slot no longer holds the exact Γ: the next use of `sigma` uploads a fresh slot.
            self._slot_of[id(sigma)] = (slot, None)
        return _result(t[0], st[0], sigma.energy)

    # -- GPU plumbing -------------------------------------------------------------------------
    def plan(self):
        if self._plan is None:
            self._plan = _native.Plan(context(self.device), self.system)
            if getattr(self, "_disorder", None) is not None:
                self._generate(*self._disorder)
            else:
                self._plan.upload_values(self.system.values)
        return self._plan

    def _generate(self, entries, nconfigs, first_config):
        from . import disorder as dis

        structs, keep = [], []
        for k, d in enumerate(entries):
            seed = int(d.get("seed", 1 + 1000 * k))
            if d["kind"] == "anderson":
                structs.append(_native.Disorder(kind=_native.ANDERSON, seed=seed, strength=float(d["strength"])))
                continue
            mom = d.get("moments", dis.Moments.isotropic())
            kinds = {"isotropic": _native.MOMENTS_ISOTROPIC, "polarized": _native.MOMENTS_POLARIZED,
                     "cone": _native.MOMENTS_CONE}
            param = mom.mz if mom.kind == "polarized" else (-(1.0 - math.cos(mom.theta0)) if mom.kind == "cone" else 0.0)
            spin = np.ascontiguousarray(np.stack([np.asfortranarray(m, np.complex128).ravel(order="F")
                                                  for m in d["spin"]]))
            keep.append(spin)
            structs.append(_native.Disorder(kind=_native.MAGNETIC, moments=kinds[mom.kind], seed=seed,
                                            concentration=float(d["concentration"]), exchange=float(d["exchange"]),
                                            moment_param=float(param), orbitals=int(spin.shape[1] ** 0.5 + 0.5),
                                            spin=spin.ctypes.data))
        self._plan.generate_values(self.system.values[0], structs, nconfigs, first_config)
        del keep

    def leads_on_device(self):
        """Whether every block's leads have a scalar coupling ``h01 = s c 1`` (square and cubic
        leads): their self-energies can then be formed on the GPU (``self_energies_on_device``)."""
        return all(l.cell is not None and r.cell is not None for l, r in self._solvers)

    def self_energies_on_device(self, energy) -> ModeSelfEnergies:
        """The self-energies of ``self_energies(energy)``, classified here per transverse mode
        (O(n) per lead) and formed on the GPU when used: no host products, no eigendecomposition
        of Γ_R, no copies of Σ."""
        if not self.leads_on_device():
            raise ValueError("a lead coupling is not a multiple of the identity")
        blocks = []
        for left, right in self._solvers:
            dl = left.definite_roots(energy)[0]
            _, lam_r, _ = right.definite_roots(energy)
            s, c = right.cell[0], right.cell[1]
            open_ = np.nonzero(lam_r.imag != 0.0)[0]
            weights = np.sqrt(-2.0 * s * c * lam_r.imag[open_])
            blocks.append((dl, lam_r, open_.astype(np.int32), weights))
        return ModeSelfEnergies(float(energy), blocks)

    def _upload_lead_modes(self, plan):
        for b, (left, right) in enumerate(self._solvers):
            for side, solver in ((0, left), (1, right)):
                s, c, _, y = solver.cell
                plan.lead_modes(b, side, y, s * c)

    def _slot(self, sigma):
        if isinstance(sigma, ModeSelfEnergies):
            key = id(sigma)
            if key not in self._slot_of or self._slot_of[key][1] is not sigma:
                plan = self.plan()
                if not getattr(self, "_modes_uploaded", False):
                    self._upload_lead_modes(plan)
                    self._modes_uploaded = True
                slot = len(self._slot_of)
                plan.sigma_from_modes(slot, sigma.energy, sigma.blocks)
                self._slot_of[key] = (slot, sigma)
            return self._slot_of[key][0]
        if len(sigma.blocks) != len(self.system.blocks):
            raise ValueError("self-energies of a system with other blocks")
        for (sl, sr), b in zip(sigma.blocks, self.system.blocks):
            if sl.shape != (len(b.left),) * 2 or sr.shape != (len(b.right),) * 2:
                raise ValueError("self-energies of a system with other leads")
        key = id(sigma)
        if key not in self._slot_of or self._slot_of[key][1] is not sigma:
            slot = len(self._slot_of)
            self.plan().upload_sigma(slot, sigma.energy, sigma.blocks, sigma.w_right())
            self._slot_of[key] = (slot, sigma)
        return self._slot_of[key][0]

    def solve_batch(self, sigmas, configs, precision=Precision.DOUBLE):
        """Raw batched solve: ``(T, status, err)`` arrays for the pairs ``(sigmas[i], configs[i])``."""
        slots = [self._slot(s) for s in sigmas]
        return self.plan().solve(slots, configs, int(precision))

    # -- transmissions ------------------------------------------------------------------------
    def transmission_with_precision(self, sigma, precision=Precision.DOUBLE, config=0):
        t, st, _ = self.solve_batch([sigma], [config], precision)
        return _result(t[0], st[0], sigma.energy)

    def transmission_with(self, sigma, config=0):
        return self.transmission_with_precision(sigma, Precision.DOUBLE, config)

    def transmission(self, energy, config=0):
        return self.transmission_with(self.self_energies(energy), config)

    def transmissions_with(self, sigmas, configs=None, precision=Precision.DOUBLE):
        """T for each ``(sigma, config)`` pair in one batch; failed points are ``GreenError``."""
        if configs is None:
            configs = [0] * len(sigmas)
        t, st, _ = self.solve_batch(sigmas, configs, precision)
        out = []
        for i, s in enumerate(sigmas):
            try:
                out.append(_result(t[i], st[i], s.energy))
            except GreenError as e:
                out.append(e)
        return out

    def transmissions(self, energies, config=0, precision=Precision.DOUBLE):
        """T at many energies (``NestedTwoTerminal::transmissions``, nested.rs:622-626): the lead
        self-energies on host threads, the solves in one GPU batch; an energy whose self-energies
        or solve fail is a ``GreenError`` in its place."""
        sigmas = self.self_energies_many(energies, errors=True)
        ok = [i for i, s in enumerate(sigmas) if not isinstance(s, GreenError)]
        out = list(sigmas)
        if ok:
            for i, r in zip(ok, self.transmissions_with([sigmas[i] for i in ok], [config] * len(ok), precision)):
                out[i] = r
        return out

    def set_parameter_derivatives(self, derivs):
        """dH/dp for gradient parameters: ``derivs[c][k]`` = values of dH/dp_k of configuration c
        on the system's CSR pattern (e.g. the exchange term divided by J for dT/dJ)."""
        self.plan().upload_derivs(derivs)

    def transmissions_with_grad(self, sigmas, configs=None):
        """``(T, status, dT/dV, dT/dp)``: dT/dV for every orbital's on-site potential (n per point)
        and dT/dp for the parameters of ``set_parameter_derivatives``; mixed precision refined in
        FP64 (no reference counterpart: the adjoint of ``transmission_with``)."""
        if configs is None:
            configs = [0] * len(sigmas)
        slots = [self._slot(s) for s in sigmas]
        return self.plan().solve_grad(slots, configs, self.system.n)

    def transmission_with_grad(self, sigma, config=0):
        t, st, dv, dp = self.transmissions_with_grad([sigma], [config])
        _result(t[0], st[0], sigma.energy)
        return float(t[0]), dv[0], dp[0]

    # -- scattering states (nested.rs:851-1020) ----------------------------------------------
    def scattering_states_batch(self, sigmas, configs=None):
        """Scattering states of each ``(sigma, config)`` pair in one GPU batch; a failed point is a
        ``GreenError`` in its place."""
        if configs is None:
            configs = [0] * len(sigmas)
        if any(not isinstance(s, LeadSelfEnergies) for s in sigmas):
            raise TypeError("scattering states take host self-energies (self_energies)")
        slots = [self._slot(s) for s in sigmas]
        outs, st = self.plan().scattering_states(slots, configs, [s.w_left() for s in sigmas],
                                                 [s.w_right() for s in sigmas], self.system.n)
        res = []
        for (pl, pr), code, s, c in zip(outs, st, sigmas, configs):
            try:
                _result(0.0, code, s.energy)
                res.append(ScatteringStates(s.energy, [pl, pr], int(c)))
            except GreenError as e:
                res.append(e)
        return res

    def scattering_states_with(self, sigma, config=0):
        out = self.scattering_states_batch([sigma], [config])[0]
        if isinstance(out, GreenError):
            raise out
        return out

    def scattering_states(self, energy, config=0):
        """``ψ_p = G W_p`` on every orbital for both leads at ``energy`` (nested.rs:851-899)."""
        return self.scattering_states_with(self.self_energies(energy), config)

    def bond_currents(self, states, f):
        """``2 Re Tr[H_ij G^<_ji]`` of every bond (nested.rs:903-906)."""
        return _states.bond_currents(self.system, states, f, None, self.sites)

    def operator_currents(self, states, f, op):
        """``Re Tr[(O H_ij + H_ij O) G^<_ji]`` of every bond (nested.rs:910-912)."""
        return _states.bond_currents(self.system, states, f, op, self.sites)

    def site_densities(self, states, f, op=None):
        """``Σ_p f_p ψ_p† O ψ_p / 2π`` of every site (nested.rs:916-918)."""
        return _states.site_densities(self.system, states, f, op)

    # -- scattering matrix (nested.rs:717-752) -------------------------------------------------
    def smatrix(self, energy, config=0):
        """Scattering matrix in the basis of the propagating lead modes (left lead 0, right lead
        1), from the FP64 root Green's function on the GPU (``caroli_root_green``)."""
        from .leads import LeadSolver
        from .smatrix import ScatteringLead, assemble, scattering_blocks

        sigma = self.self_energies(energy)
        slot = self._slot(sigma)
        kept = []
        for blk in self.system.blocks:
            same = np.array_equal(blk.left, blk.right)
            kept.append(len(blk.left) + (0 if same else len(blk.right)))
        greens, st = self.plan().root_green([slot], [config], kept)
        if st[0] != _native.OK:
            raise GreenError("Singular", f"solve status {st[0]} at E = {energy}")
        parts = []
        for blk, g in zip(self.system.blocks, greens[0]):
            nl, nr = len(blk.left), len(blk.right)
            rpos = 0 if np.array_equal(blk.left, blk.right) else nl
            left_out = blk.left_h01.conj().T  # cells going away from the device: -axis
            lm = LeadSolver(blk.left_h00, left_out).modes(energy)
            rm = LeadSolver(blk.right_h00, blk.right_h01).modes(energy)
            leads = [ScatteringLead(np.arange(nl), left_out, left_out, lm, energy),
                     ScatteringLead(np.arange(rpos, rpos + nr), blk.right_h01, blk.right_h01, rm, energy)]
            parts.append(scattering_blocks(g, leads, [blk.left_h00, blk.right_h00], energy))
        return assemble(energy, parts)

    # -- transmission eigenvalues (nested.rs:753-780) --------------------------------------
    def transmission_eigenvalues_batch(self, sigmas, configs=None):
        """Transmission eigenvalues of each ``(sigma, config)`` pair, decreasing: the squared
        singular values of t = W_L^† G_LR W_R of every block (t from the GPU, the small SVD here);
        a failed point is a ``GreenError``."""
        if configs is None:
            configs = [0] * len(sigmas)
        slots = [self._slot(s) for s in sigmas]
        nr = [len(b.right) for b in self.system.blocks]
        ts, st = self.plan().transmission_matrices(slots, configs, [s.w_left() for s in sigmas], nr)
        out = []
        for tb, code, s in zip(ts, st, sigmas):
            if code != _native.OK:
                out.append(GreenError("Singular", f"solve status {code} at E = {s.energy}"))
                continue
            taus = np.concatenate([np.linalg.svd(t, compute_uv=False) ** 2 if t.size else np.zeros(0) for t in tb])
            out.append(np.sort(taus)[::-1])
        return out

    def transmission_eigenvalues(self, energy, config=0):
        out = self.transmission_eigenvalues_batch([self.self_energies(energy)], [config])[0]
        if isinstance(out, GreenError):
            raise out
        return out

    def fano_factor(self, energy, config=0):
        """F = Σ τ (1 - τ) / Σ τ (nested.rs:773-780)."""
        taus = self.transmission_eigenvalues(energy, config)
        return float(np.sum(taus * (1.0 - taus)) / np.sum(taus))

    def transmissions_checked(self, energies, options: PrecisionOptions, config=0):
        sigmas = {float(e): self.self_energies(e) for e in energies}

        def run(points, precision):
            return self.transmissions_with([sigmas[float(e)] for e in points], [config] * len(points), precision)

        return checked(list(energies), options, run)


def solve_systems(items, precision=Precision.MIXED):
    """``(T, status, err)`` for ``(system, sigma, config)`` items of possibly different systems
    (sizes, trees, leads) in one GPU batch; every system must be on the same device. The
    reference calls ``transmission_with`` system by system (nested.rs:682)."""
    if not items:
        return np.zeros(0), np.zeros(0, np.int32), np.zeros(0)
    device = items[0][0].device
    if any(s.device != device for s, _, _ in items):
        raise ValueError("solve_systems: systems on different devices")
    plans = [s.plan() for s, _, _ in items]
    slots = [s._slot(sig) for s, sig, _ in items]
    configs = [c for _, _, c in items]
    return context(device).solve_multi(plans, slots, configs, int(precision))


def _result(t, status, energy):
    if status == _native.OK:
        return float(t)
    if status in (_native.SINGULAR, _native.NONFINITE):
        raise GreenError("Singular", f"lead self-energy or root singular near E = {energy}")
    if status == _native.REFINE_STALLED:
        raise GreenError("NoConvergence", f"refinement stalled at E = {energy}")
    raise GreenError("Singular", f"solve status {status} at E = {energy}")
