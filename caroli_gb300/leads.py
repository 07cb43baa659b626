"""Lead modes and mode-matching self-energies (host input to the transmission path).

The nested-dissection path takes ``Σ_L``, ``Σ_R`` as inputs (``NestedTwoTerminal::transmission_with``,
``crates/caroli-green/src/nested.rs:682``); caroli computes them by mode matching
(``crates/caroli-green/src/modes.rs``).  This module computes the same retarded self-energies on
the host with LAPACK (numpy/scipy), by a formulation of its own:

- the Bloch problem ``(h01^† λ^-1 + h00 - E + h01 λ) φ = 0`` of a lead cell (``h01 = <j|H|j+1>``)
  is linearised as the ``2n`` pencil ``A v = λ B v`` with ``v = (ψ_j, ψ_{j+1})``; with a
  well-conditioned ``h01`` (BHZ) it is solved as the standard eigenproblem of ``B^-1 A`` (five times
  faster than the QZ of the pencil, Σ equal to ~1e-13), else (graphene's rank-deficient coupling)
  by QZ;
- modes with ``|λ| < 1`` and propagating modes with positive current go right, the others left;
  the current of a propagating group is ``J_pq = i(λ_q φ_p^† h01 φ_q - λ_p^* φ_p^† h01^† φ_q)``,
  diagonalised within degenerate groups (the reference's rule, ``modes.rs:400-446``);
- with ``V`` the right-going vectors, ``Σ_R = h01 V_bot V_top^-1``; with ``W`` the left-going ones,
  ``Σ_L = h01^† W_top W_bot^-1`` (any basis of the subspaces gives the same ``Σ``);
- a rank-deficient coupling (graphene's zigzag cell: only half of a slice's sites couple to the
  next cell) is reduced to a ``2r`` pencil, ``r = rank h01``, before the eigenproblem (below,
  ``_reduced``): 8x fewer flops than the ``2n`` pencil and no infinite eigenvalues, so it is a
  standard eigenproblem instead of a QZ;
- a Hermitian scalar coupling ``h01 = s c 1`` (square and cubic leads) takes the fast path of
  ``modes.rs:540-710``: one eigen-decomposition of ``h00``, reused at every energy;
- band edges and surface bound states are retried at ``E + δ``, ``δ`` in ``{0, 1e-9 … 1e-6}``
  times the bandwidth scale (``modes.rs:49-50``, ``:129-145``).

``Σ`` is the mathematically unique retarded self-energy, so it agrees with the reference's
``sigma_left``/``sigma_right`` to rounding; the tests pin it against the reference's published
transmissions and against Lopez-Sancho decimation.
"""
from __future__ import annotations

import threading

import numpy as np
import scipy.linalg as sla

UNIT_TOL = 1e-6
DEGENERATE_TOL = 1e-7
VELOCITY_TOL = 1e-8
DEFECTIVE_TOL = 1e-7
SINGULAR_TOL = 1e-11
SHIFTS = (0.0, 1e-9, 1e-8, 1e-7, 1e-6)
RANK_TOL = 1e-12  # singular values of h01 below this fraction of the largest are dropped


class GreenError(Exception):
    """Mirror of ``GreenError`` (``crates/caroli-green/src/lib.rs:34-47``)."""

    def __init__(self, kind, detail=""):
        super().__init__(f"{kind}: {detail}" if detail else kind)
        self.kind = kind


def _row_norm(m):
    return float(np.abs(m).sum(axis=1).max()) if m.size else 0.0


def _hermitian(m, tol=1e-14):
    return np.abs(m - m.conj().T).max() <= tol * max(np.abs(m).max(), 0.0) if m.size else True


def _inv_cond(m):
    if m.shape[0] == 0:
        return 1.0
    s = np.linalg.svd(m, compute_uv=False)
    return float(s.min() / s.max()) if s.max() > 0 else 0.0


class LeadSolver:
    """Energy-independent part of a lead's mode problem (``ModeSolver``, ``modes.rs:514-538``)."""

    def __init__(self, h00, h01):
        self.h00 = np.array(h00, dtype=np.complex128)
        self.h01 = np.array(h01, dtype=np.complex128)
        n = self.h00.shape[0]
        self.n = n
        self.scale = max(_row_norm(self.h00) + 2.0 * _row_norm(self.h01), np.finfo(float).tiny)
        # h01^-1 when the coupling is well conditioned (the general path then solves a standard
        # eigenproblem), else None (QZ of the pencil).
        self.h01_inv = None
        if n and np.abs(self.h01).max() > 0 and _inv_cond(self.h01) > 1e-6:
            self.h01_inv = np.linalg.inv(self.h01)
        # Rank-deficient couplings: h01 = u v^† with u, v of r < n columns (the reduced pencil).
        self.uv = None
        if n and self.h01_inv is None and np.abs(self.h01).max() > 0:
            uu, sv, vh = np.linalg.svd(self.h01)
            r = int(np.sum(sv > RANK_TOL * sv[0]))
            if r < n:
                root = np.sqrt(sv[:r])
                self.uv = (uu[:, :r] * root[None, :], vh[:r].conj().T * root[None, :])
        # The modes of the last general or reduced solve, per thread: energies may be solved on
        # several host threads at once (NestedTwoTerminal.self_energies_many).
        self._tls = threading.local()
        self.cell = None
        if n and np.abs(self.h01).max() > 0 and _hermitian(self.h00) and _hermitian(self.h01):
            c = self.h01[0, 0].real
            if c != 0 and np.abs(self.h01 - c * np.eye(n)).max() <= 1e-14 * abs(c):
                s = 1.0 if c > 0 else -1.0
                theta, y = np.linalg.eigh(0.5 * (self.h00 + self.h00.conj().T))
                self.cell = (s, abs(c), theta, y)

    def self_energies(self, energy):
        """``(Σ_L, Σ_R, energy used)`` at the real ``energy`` (shifted off band edges)."""
        last = GreenError("Eigen")
        for shift in SHIFTS:
            e = energy + shift * self.scale
            try:
                if self.cell is not None:
                    return self._definite(e) + (e,)
                if self.uv is not None:
                    return self._reduced(e) + (e,)
                return self._general(e) + (e,)
            except GreenError as err:
                last = err
            except (np.linalg.LinAlgError, ValueError) as err:
                last = GreenError("Eigen", str(err))
        raise last

    def definite_roots(self, energy):
        """For a scalar coupling ``h01 = s c 1``: ``(1/λ_L, λ_R, energy used)`` per mode of the cell
        eigenvectors ``self.cell[3]`` (shifted off band edges as ``self_energies``), so that
        ``Σ_L = s c Y diag(1/λ_L) Y^†`` and ``Σ_R = s c Y diag(λ_R) Y^†``."""
        if self.cell is None:
            raise ValueError("the lead coupling is not a multiple of the identity")
        last = GreenError("Eigen")
        for shift in SHIFTS:
            e = energy + shift * self.scale
            try:
                lam_l, lam_r = self._definite_roots(e)
                return 1.0 / lam_l, lam_r, e
            except GreenError as err:
                last = err
        raise last

    def modes(self, energy):
        """Propagating modes at ``energy`` (shifted off band edges as ``self_energies``), each
        carrying unit current (``LeadModes``, modes.rs:52-76), for a lead whose cells go away from
        the device with ``h01``: ``(right_modes, right_lambdas, left_modes, left_lambdas, Σ_rest,
        energy used)``; right = outgoing (away from the device), left = incoming, Σ_rest = h01 F the
        self-energy of the cells beyond the first."""
        last = GreenError("Eigen")
        for shift in SHIFTS:
            e = energy + shift * self.scale
            try:
                if self.cell is not None:
                    sig = self._definite(e)
                    s, c, theta, y = self.cell
                    lam_l, lam_r = self._definite_roots(e)
                    prop = np.nonzero(lam_r.imag != 0.0)[0]
                    flux = y[:, prop] / np.sqrt(c) / np.sqrt(2.0 * np.abs(lam_r.imag[prop]))[None, :]
                    return flux, lam_r[prop], flux.copy(), lam_l[prop], sig[1], e
                sig = self._reduced(e) if self.uv is not None else self._general(e)
                (rm, rl), (lm, ll) = self._tls.last_modes
                return rm, rl, lm, ll, sig[1], e
            except GreenError as err:
                last = err
            except (np.linalg.LinAlgError, ValueError) as err:
                last = GreenError("Eigen", str(err))
        raise last

    # -- h01 = s c 1: one Hermitian problem ------------------------------------------------------
    def _definite(self, e):
        s, c, theta, y = self.cell
        lam_l, lam_r = self._definite_roots(e)
        # Σ_R = h01 F_+ with F_+ = Y λ_R Y†;  Σ_L = h01† F_-^-1 with F_-^-1 = Y λ_L^-1 Y†.
        sig_r = (s * c) * (y * lam_r) @ y.conj().T
        sig_l = (s * c) * (y * (1.0 / lam_l)) @ y.conj().T
        return sig_l, sig_r

    def _definite_roots(self, e):
        s, c, theta, y = self.cell
        mu = -(theta - e) / (s * c)
        lam_r = np.empty(len(mu), np.complex128)
        lam_l = np.empty(len(mu), np.complex128)
        for k, m in enumerate(mu):
            if abs(m) < 2.0:
                root = complex(m / 2.0, np.sqrt(4.0 - m * m) / 2.0)
                if 2.0 * root.imag < DEGENERATE_TOL:
                    raise GreenError("Singular", f"subband edge near E = {e}")
                # Current J = -2 s c Im λ: the root with s Im λ < 0 goes right.
                r, l = (root, root.conjugate()) if s < 0 else (root.conjugate(), root)
                if abs(2.0 * r.imag / c) < VELOCITY_TOL * self.scale:
                    raise GreenError("Singular", f"subband edge near E = {e}")
                lam_r[k], lam_l[k] = r, l
            else:
                big = (m + np.sign(m) * np.sqrt(m * m - 4.0)) / 2.0
                if abs(big) <= 1.0 + UNIT_TOL:
                    raise GreenError("Singular", f"subband edge near E = {e}")
                lam_r[k], lam_l[k] = 1.0 / big, big
        return lam_l, lam_r

    # -- general coupling: the 2n pencil ---------------------------------------------------------
    def _general(self, e):
        n = self.n
        h00, h01 = self.h00, self.h01
        eye = np.eye(n, dtype=np.complex128)
        zero = np.zeros((n, n), np.complex128)
        a = np.block([[zero, eye], [-h01.conj().T, e * eye - h00]])
        b = np.block([[eye, zero], [zero, h01]])
        if self.h01_inv is not None:
            # A well-conditioned coupling: the standard eigenproblem of B^-1 A has the same
            # eigenpairs and costs a third of the QZ iteration of the pencil.
            hi = self.h01_inv
            m = np.block([[zero, eye], [-hi @ h01.conj().T, hi @ (e * eye - h00)]])
            alpha, vr = np.linalg.eig(m)
            beta = np.ones_like(alpha)
        else:
            w, vr = sla.eig(a, b, homogeneous_eigvals=True, right=True)
            alpha, beta = w[0], w[1]
        mod_a, mod_b = np.abs(alpha), np.abs(beta)
        right_ev = mod_a < (1.0 - UNIT_TOL) * mod_b
        left_ev = mod_a > (1.0 + UNIT_TOL) * mod_b
        prop = ~(right_ev | left_ev)
        with np.errstate(divide="ignore", invalid="ignore"):
            lam = np.where(mod_b > 0, alpha / np.where(mod_b > 0, beta, 1.0), np.inf)
        vr = vr / np.linalg.norm(vr, axis=0)

        right_vecs, left_vecs = [], []
        right_modes, left_modes = [], []  # (unit-current φ, λ) of the propagating modes
        pidx = np.nonzero(prop)[0]
        # Degenerate propagating groups by single linkage.
        groups = []
        for k in pidx:
            placed = False
            for g in groups:
                if any(abs(lam[k] - lam[j]) < DEGENERATE_TOL for j in g):
                    g.append(k)
                    placed = True
                    break
            if not placed:
                groups.append([k])
        for g in groups:
            v = vr[:, g]
            phi = v[:n]
            lg = lam[g]
            gram = v.conj().T @ v
            if _inv_cond(gram) < DEFECTIVE_TOL ** 2:
                raise GreenError("Singular", f"Jordan block (subband edge) near E = {e}")
            a_ = phi.conj().T @ (h01 @ phi)
            b_ = phi.conj().T @ (h01.conj().T @ phi)
            cur = 1j * (a_ * lg[None, :] - lg.conj()[:, None] * b_)
            cur = 0.5 * (cur + cur.conj().T)
            vel, coef = sla.eigh(cur, gram)
            newv = v @ coef
            for k in range(len(g)):
                ph = newv[:n, k]
                vk = vel[k] / max(np.vdot(ph, ph).real, np.finfo(float).tiny)
                if not np.isfinite(vk) or abs(vk) < VELOCITY_TOL * self.scale:
                    raise GreenError("Singular", f"subband edge near E = {e}")
                (right_vecs if vk > 0 else left_vecs).append(newv[:, k])
                (right_modes if vk > 0 else left_modes).append((ph / np.sqrt(abs(vel[k])), lg.mean()))
        def stack(ms):
            if not ms:
                return np.zeros((n, 0), np.complex128), np.zeros(0, np.complex128)
            return np.array([m[0] for m in ms]).T, np.array([m[1] for m in ms])

        self._tls.last_modes = (stack(right_modes), stack(left_modes))
        nr = int(right_ev.sum()) + len(right_vecs)
        nl = int(left_ev.sum()) + len(left_vecs)
        if nr != n or nl != n:
            raise GreenError("ModeCount", f"{nr} right-going and {nl} left-going, expected {n}")
        vr_right = np.concatenate([vr[:, right_ev]] + [np.array(right_vecs).T.reshape(2 * n, -1)], axis=1)
        vr_left = np.concatenate([vr[:, left_ev]] + [np.array(left_vecs).T.reshape(2 * n, -1)], axis=1)
        if _inv_cond(vr_right) < 1e-10 or _inv_cond(vr_left) < 1e-10:
            vr_right, vr_left = self._schur_bases(a, b, vr_right[:, right_ev.sum():], vr_left[:, left_ev.sum():])
        top, bot = vr_right[:n], vr_right[n:]
        if _inv_cond(top) < SINGULAR_TOL:
            raise GreenError("Singular", f"lead surface bound state near E = {e}")
        sig_r = h01 @ np.linalg.solve(top.T, bot.T).T
        top, bot = vr_left[:n], vr_left[n:]
        if _inv_cond(bot) < SINGULAR_TOL:
            raise GreenError("Singular", f"lead surface bound state near E = {e}")
        sig_l = h01.conj().T @ np.linalg.solve(bot.T, top.T).T
        return sig_l, sig_r

    # -- rank-deficient coupling: the 2r pencil ----------------------------------------------------
    def _reduced(self, e):
        """Σ_L, Σ_R of a coupling h01 = u v^† of rank r < n.

        With a = v^† φ, b = u^† φ the Bloch equation reads (h00 - E) φ = -λ u a - λ^-1 v b. A
        stabilised resolvent G = (h00 - E + s(u u^† + v v^†))^-1, s = i (invertible unless a state
        of the cell at E is decoupled from both neighbours), gives φ = G[u(s b - λ a) + v(s a - b/λ)],
        and projecting on v^† and u^† gives, for x = (a, y), y = b / λ, the 2r pencil R x = λ L x:
            R = [[1 - s v^†Gv, v^†Gv], [-s u^†Gv, u^†Gv]],
            L = [[-v^†Gu, s v^†Gu], [-u^†Gu, s u^†Gu - 1]].
        Its 2r eigenvalues are the finite, non-zero λ of the 2n problem; the n - r modes with λ = 0
        span null(u^†) and those with λ = ∞ null(v^†). So with (A, Y) the reduced vectors of the r
        right-going modes, Σ_R = h01 F = u A Y^-1 u^†, and with those of the r left-going ones,
        Σ_L = h01^† F^-1 = v Y A^-1 v^† (both basis-independent). Propagating modes are split by
        their current i(λ_q φ_p^† h01 φ_q - λ_p^* φ_p^† h01^† φ_q) as in ``_general``, on φ rebuilt
        from the reduced vector.
        """
        n = self.n
        u, v = self.uv
        r = u.shape[1]
        h01 = self.h01
        s = 1j
        eye_r = np.eye(r, dtype=np.complex128)
        uvm = np.concatenate([u, v], axis=1)
        gmat = self.h00 - e * np.eye(n) + s * (uvm @ uvm.conj().T)
        if _inv_cond(gmat) < 1e-13:
            raise GreenError("Eigen", f"decoupled cell state near E = {e}")
        guv = np.linalg.solve(gmat, uvm)
        gu, gv = guv[:, :r], guv[:, r:]
        ugu, ugv = u.conj().T @ gu, u.conj().T @ gv
        vgu, vgv = v.conj().T @ gu, v.conj().T @ gv
        rmat = np.block([[eye_r - s * vgv, vgv], [-s * ugv, ugv]])
        lmat = np.block([[-vgu, s * vgu], [-ugu, s * ugu - eye_r]])
        cl, cr = _inv_cond(lmat), _inv_cond(rmat)
        std = None  # the standard matrix of the pencil, and whether its eigenvalues are 1/λ
        if cl >= cr and cl > 1e-10:
            std = (np.linalg.solve(lmat, rmat), False)
            lam, x = np.linalg.eig(std[0])
        elif cr > 1e-10:
            std = (np.linalg.solve(rmat, lmat), True)
            mu, x = np.linalg.eig(std[0])
            with np.errstate(divide="ignore", invalid="ignore"):
                lam = np.where(np.abs(mu) > 1e-13 * np.abs(mu).max(), 1.0 / mu, np.inf)
        else:
            w, x = sla.eig(rmat, lmat, homogeneous_eigvals=True, right=True)
            with np.errstate(divide="ignore", invalid="ignore"):
                lam = np.where(np.abs(w[1]) > 0, w[0] / np.where(np.abs(w[1]) > 0, w[1], 1.0), np.inf)
        x = x / np.linalg.norm(x, axis=0)
        mod = np.abs(lam)
        right_ev = mod < 1.0 - UNIT_TOL
        left_ev = mod > 1.0 + UNIT_TOL
        prop = ~(right_ev | left_ev)

        def phi_of(xs, ls):
            """φ of reduced vectors (a, y) with eigenvalues λ (finite, non-zero)."""
            a, y = xs[:r], xs[r:]
            return gu @ (s * ls[None, :] * y - ls[None, :] * a) + gv @ (s * a - y)

        right_x, left_x = [], []
        right_modes, left_modes = [], []
        pidx = np.nonzero(prop)[0]
        groups = []
        for k in pidx:
            for g in groups:
                if any(abs(lam[k] - lam[j]) < DEGENERATE_TOL for j in g):
                    g.append(k)
                    break
            else:
                groups.append([k])
        for g in groups:
            lg = lam[g]
            phi = phi_of(x[:, g], lg)
            # The 2n vectors (φ, λφ) of _general: the same metric within the group.
            gram = (1.0 + np.abs(lg.mean()) ** 2) * (phi.conj().T @ phi)
            if _inv_cond(gram) < DEFECTIVE_TOL ** 2:
                raise GreenError("Singular", f"Jordan block (subband edge) near E = {e}")
            a_ = phi.conj().T @ (h01 @ phi)
            b_ = phi.conj().T @ (h01.conj().T @ phi)
            cur = 1j * (a_ * lg[None, :] - lg.conj()[:, None] * b_)
            cur = 0.5 * (cur + cur.conj().T)
            vel, coef = sla.eigh(cur, gram)
            newx = x[:, g] @ coef
            newphi = phi @ coef
            for k in range(len(g)):
                ph = newphi[:, k]
                vk = vel[k] / max(np.vdot(ph, ph).real, np.finfo(float).tiny)
                if not np.isfinite(vk) or abs(vk) < VELOCITY_TOL * self.scale:
                    raise GreenError("Singular", f"subband edge near E = {e}")
                (right_x if vk > 0 else left_x).append(newx[:, k])
                (right_modes if vk > 0 else left_modes).append((ph / np.sqrt(abs(vel[k])), lg.mean()))

        def stack(ms):
            if not ms:
                return np.zeros((n, 0), np.complex128), np.zeros(0, np.complex128)
            return np.array([m[0] for m in ms]).T, np.array([m[1] for m in ms])

        self._tls.last_modes = (stack(right_modes), stack(left_modes))
        nr = int(right_ev.sum()) + len(right_x)
        nl = int(left_ev.sum()) + len(left_x)
        if nr != r or nl != r:
            raise GreenError("ModeCount", f"{nr} right-going and {nl} left-going, expected {r}")
        xr = np.concatenate([x[:, right_ev]] + [np.array(right_x).T.reshape(2 * r, -1)], axis=1)
        xl = np.concatenate([x[:, left_ev]] + [np.array(left_x).T.reshape(2 * r, -1)], axis=1)
        if _inv_cond(xr) < 1e-4 or _inv_cond(xl) < 1e-4:
            # Nearly parallel evanescent vectors (zigzag edge states, from W ~ 30 on): orthonormal
            # bases of the evanescent subspaces from ordered Schur forms instead (Σ then satisfies
            # its Dyson equation to ~1e-13 where the eigenvectors leave ~1e-7).
            pr, pl = xr[:, right_ev.sum():], xl[:, left_ev.sum():]
            if std is None:
                xr, xl = self._schur_bases(rmat, lmat, pr, pl)
            else:
                m_std, inv = std
                inside = (lambda z: abs(z) > 1.0 / (1.0 - UNIT_TOL)) if inv else (lambda z: abs(z) < 1.0 - UNIT_TOL)
                outside = (lambda z: abs(z) < 1.0 / (1.0 + UNIT_TOL)) if inv else (lambda z: abs(z) > 1.0 + UNIT_TOL)
                _, zi, ki = sla.schur(m_std, output="complex", sort=inside)
                _, zo, ko = sla.schur(m_std, output="complex", sort=outside)
                xr = np.concatenate([zi[:, :ki], pr], axis=1)
                xl = np.concatenate([zo[:, :ko], pl], axis=1)
        a_r, y_r = xr[:r], xr[r:]
        if _inv_cond(y_r) < SINGULAR_TOL:
            raise GreenError("Singular", f"lead surface bound state near E = {e}")
        sig_r = u @ np.linalg.solve(y_r.T, a_r.T).T @ u.conj().T
        a_l, y_l = xl[:r], xl[r:]
        if _inv_cond(a_l) < SINGULAR_TOL:
            raise GreenError("Singular", f"lead surface bound state near E = {e}")
        sig_l = v @ np.linalg.solve(a_l.T, y_l.T).T @ v.conj().T
        return sig_l, sig_r

    @staticmethod
    def _schur_bases(a, b, prop_right, prop_left):
        """Orthonormal bases of the evanescent subspaces from the ordered QZ decomposition, for
        pencils whose eigenvectors are too close to parallel."""
        def first(sort):
            _, _, alpha, beta, _, z = sla.ordqz(a, b, sort=sort, output="complex")
            k = int(sum(sort(x, y) for x, y in zip(alpha, beta)))
            return z[:, :k]

        inside = lambda x, y: abs(x) < (1.0 - UNIT_TOL) * abs(y)
        outside = lambda x, y: abs(x) > (1.0 + UNIT_TOL) * abs(y)
        right = np.concatenate([first(inside), prop_right], axis=1)
        left = np.concatenate([first(outside), prop_left], axis=1)
        return right, left


def broadening(sigma):
    """``Γ = i(Σ - Σ†)`` (``crates/caroli-green/src/lib.rs:67-71``)."""
    return 1j * (sigma - sigma.conj().T)


def gamma_root(sigma, cut=1e-12):
    """``W`` with ``W W† = Γ``: eigenvectors of ``Γ`` with eigenvalues above ``cut`` times the
    largest, scaled by their square roots (``nested.rs:1036-1047`` cuts at 1e-12). The mixed
    transmission takes its right-hand sides from here: T = Σ_j x_j^† Γ_L x_j with x = G W_R
    differs from the full-Γ trace only by the dropped eigenvalues (rounding noise of Σ, which may
    be slightly negative), a few 1e-10 at worst on the reference's benchmark problems."""
    g = broadening(sigma)
    g = 0.5 * (g + g.conj().T)
    vals, vecs = np.linalg.eigh(g)
    top = np.abs(vals).max() if len(vals) else 0.0
    keep = vals > cut * top
    return vecs[:, keep] * np.sqrt(vals[keep])[None, :]
