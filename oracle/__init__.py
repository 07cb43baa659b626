"""ORACLE — test infrastructure only (tests, ``__graft_entry__.smoke`` and the CPU-baseline leg
of ``bench.py``). The product package ``caroli_gb300`` never imports this module.

``liboracle.so`` is a C++ restatement of caroli's nested-dissection transmission
(``crates/caroli-green/src/nested.rs``); see ``nested_oracle.cpp`` for the line-by-line map.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "nested_oracle.cpp")):
            build()
        L = ctypes.CDLL(_LIB)
        P = ctypes.c_void_p
        L.oracle_build.restype = ctypes.c_int
        L.oracle_build.argtypes = [ctypes.c_int64, P, P, ctypes.c_int64, ctypes.c_int, P, P, P, P, ctypes.c_int64, P,
                                   ctypes.c_int, P, P, P, P, P, ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_solve.argtypes = [P, ctypes.c_int, ctypes.c_double, P, P, P, ctypes.c_int, P, P, P]
        L.oracle_solve_batch.restype = ctypes.c_int
        L.oracle_solve_batch.argtypes = [P, ctypes.c_int64, P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_free.argtypes = [P]
        L.oracle_tree_info.argtypes = [P, ctypes.c_int, P, P, P]
        L.oracle_tree_fronts.argtypes = [P, ctypes.c_int, ctypes.c_int64, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """FP64 (or c32-fronts) CPU transmission of a ``caroli_gb300.nested.System`` description."""

    def __init__(self, system):
        L = lib()
        s = system
        self.system = s
        self._keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            self._keep.append(a)
            return a

        row_ptr = arr(s.row_ptr, np.int64)
        cols = arr(s.cols, np.uint32)
        cells = arr(s.cells, np.int64)
        offs = arr(s.site_offsets, np.int64)
        norbs = arr(s.site_orbitals, np.int64)
        rng = arr(s.range, np.int64)
        interior = arr(s.interior, np.int64)
        labels = arr(s.labels, np.int32)
        lp = arr(np.cumsum([0] + [len(b.left) for b in s.blocks]), np.int64)
        rp = arr(np.cumsum([0] + [len(b.right) for b in s.blocks]), np.int64)
        lf = arr(np.concatenate([b.left for b in s.blocks]) if s.blocks else [], np.int64)
        rt = arr(np.concatenate([b.right for b in s.blocks]) if s.blocks else [], np.int64)
        h = ctypes.c_void_p()
        rc = L.oracle_build(s.n, _p(row_ptr), _p(cols), len(norbs), s.dim, _p(cells), _p(offs), _p(norbs), _p(rng),
                            len(interior), _p(interior), len(s.blocks), _p(labels), _p(lp), _p(lf), _p(rp), _p(rt),
                            ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("oracle_build failed")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_free(self.h)
            self.h = None

    def tree_info(self, block):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        lib().oracle_tree_info(self.h, block, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def tree_fronts(self, block):
        nodes = self.tree_info(block)[0]
        n = np.zeros(nodes, np.int32)
        ne = np.zeros(nodes, np.int32)
        lib().oracle_tree_fronts(self.h, block, nodes, _p(n), _p(ne))
        return n, ne

    def solve_block(self, block, energy, vals, sigma_l, sigma_r, precision=0, want_g=False):
        """``(status, T, G_LR or None, delayed count)`` for one block."""
        vals = np.ascontiguousarray(vals, np.complex128)
        sl = np.asfortranarray(sigma_l, np.complex128)
        sr = np.asfortranarray(sigma_r, np.complex128)
        t = np.zeros(1)
        nl, nr = sl.shape[0], sr.shape[0]
        g = np.zeros((nl, nr), np.complex128, order="F") if want_g else None
        nd = np.zeros(1, np.int64)
        st = lib().oracle_solve(self.h, block, energy, _p(vals), _p(sl), _p(sr), precision, _p(t),
                                _p(g) if want_g else None, _p(nd))
        return st, float(t[0]), g, int(nd[0])

    def transmission(self, energy, vals, sigmas, precision=0):
        """Sum over blocks; ``sigmas[b] = (Σ_L, Σ_R)``. Raises on a singular block."""
        total = 0.0
        for b, (sl, sr) in enumerate(sigmas):
            st, t, _, _ = self.solve_block(b, energy, vals, sl, sr, precision)
            if st != 0:
                raise RuntimeError(f"oracle status {st} at E = {energy}, block {b}")
            total += t
        return total

    def solve_batch(self, blocks, energies, vals_list, sl_list, sr_list, precision=0, threads=0):
        """Independent block solves on OpenMP threads; returns ``(T, status)`` arrays."""
        cnt = len(blocks)
        blocks = np.ascontiguousarray(blocks, np.int32)
        energies = np.ascontiguousarray(energies, np.float64)
        vals_list = [np.ascontiguousarray(v, np.complex128) for v in vals_list]
        sl_list = [np.asfortranarray(v, np.complex128) for v in sl_list]
        sr_list = [np.asfortranarray(v, np.complex128) for v in sr_list]
        ptr = lambda xs: np.array([x.ctypes.data for x in xs], dtype=np.uintp)
        pv, pl, pr = ptr(vals_list), ptr(sl_list), ptr(sr_list)
        t = np.zeros(cnt)
        st = np.zeros(cnt, np.int32)
        lib().oracle_solve_batch(self.h, cnt, _p(blocks), _p(energies), _p(pv), _p(pl), _p(pr), precision, threads,
                                 _p(t), _p(st))
        return t, st
