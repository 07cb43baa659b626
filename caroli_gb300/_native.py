"""ctypes binding of ``libcaroli_gb300.so`` (the C ABI of ``include/caroli_gb300.h``).

The library is built in-tree (``caroli_gb300/_build``) by ``__graft_entry__.build()``. There is no
fallback: without the library every GPU entry point raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcaroli_gb300.so")

OK, PIVOT_DELAYED, SINGULAR, NONFINITE, REFINE_STALLED, TIMEOUT = 0, 1, 2, 3, 4, 5
EINVAL, ENOMEM, ECUDA, EUNAVAILABLE = 16, 17, 18, 19
DOUBLE, SINGLE, MIXED = 0, 1, 2

# Every symbol the header declares, with its ctypes signature.
P = ctypes.c_void_p
I64 = ctypes.c_int64
SIGNATURES = {
    "caroli_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "caroli_ctx_destroy": (None, [P]),
    "caroli_last_error": (ctypes.c_char_p, [P]),
    "caroli_plan_upload": (ctypes.c_int, [P, I64, P, P, I64, ctypes.c_int, P, P, P, P, I64, P, ctypes.c_int, P, P, P,
                                          P, P, ctypes.POINTER(ctypes.c_int)]),
    "caroli_plan_info": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P]),
    "caroli_plan_fronts": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, I64, P, P, P, P]),
    "caroli_values_upload": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P]),
    "caroli_sigma_upload": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, P, P, P, P]),
    "caroli_solve_batch": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, P, P, P]),
    "caroli_last_timing": (ctypes.c_int, [P, P, P]),
    "caroli_last_stats": (ctypes.c_int, [P, P, P]),
    "caroli_last_phases": (ctypes.c_int, [P, P, P, P]),
    "caroli_region_begin": (ctypes.c_int, [P]),
    "caroli_region_end": (ctypes.c_int, [P, P, P]),
    "caroli_solve_batch_noalloc": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P]),
    "caroli_derivs_upload": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P]),
    "caroli_transmission_with_grad": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]),
    "caroli_kernel_classes": (ctypes.c_int, []),
    "caroli_last_job_info": (ctypes.c_int, [P, I64, P, P, P, P]),
    "caroli_last_refine_steps": (ctypes.c_int, [P, P, P]),
    "caroli_set_refine_options": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    "caroli_set_tensor_cores": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_set_mixed_max_channels": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_set_wait_limit": (ctypes.c_int, [P, ctypes.c_int64]),
    "caroli_set_autotune": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_set_graphs": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_set_schedule": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
    "caroli_set_sweep_columns": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_set_small_threads": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_last_schedule": (ctypes.c_int, [P, P, P, P, P, P, P]),
    "caroli_solve_multi": (ctypes.c_int, [P, ctypes.c_int, P, P, P, ctypes.c_int, P, P, P]),
    "caroli_scattering_states": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P, P, P]),
    "caroli_multi_leads": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P]),
    "caroli_transmission_matrix": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]),
    "caroli_last_job_steps": (ctypes.c_int, [P, ctypes.c_int64, P, P]),
    "caroli_gamma_override": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P]),
    "caroli_root_green": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P]),
    "caroli_multi_scattering_states": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]),
    "caroli_multi_sector_transmissions": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int,
                                                         ctypes.c_int, P, P, P, P]),
    "caroli_values_generate": (ctypes.c_int, [P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int]),
    "caroli_lead_modes": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P,
                                         ctypes.c_double]),
    "caroli_sigma_from_modes": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, P, P, P, P, P]),
    "caroli_values_download": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P]),
    "caroli_multi_sigma_upload": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, P]),
    "caroli_multi_transmissions": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, P, P]),
    "caroli_kernel_class_name": (ctypes.c_char_p, [ctypes.c_int]),
    "caroli_probe_kernel": (ctypes.c_int, [P, ctypes.c_int]),
    "caroli_kernel_stats": (ctypes.c_int, [P, ctypes.c_int, P, P, P, P, ctypes.c_int]),
}

_lib = None


ANDERSON, MAGNETIC = 0, 1
MOMENTS_ISOTROPIC, MOMENTS_POLARIZED, MOMENTS_CONE = 0, 1, 2


class Disorder(ctypes.Structure):
    """``caroli_disorder`` of the C ABI."""

    _fields_ = [("kind", ctypes.c_int32), ("moments", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("strength", ctypes.c_double), ("concentration", ctypes.c_double), ("exchange", ctypes.c_double),
                ("moment_param", ctypes.c_double), ("orbitals", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("spin", ctypes.c_void_p)]


class NativeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"caroli_gb300 native error {code}: {msg}")
        self.code = code


def load():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError(EUNAVAILABLE, f"{LIB_PATH} is missing: build the CUDA library first")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Context:
    """A device context (``caroli_ctx``)."""

    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        rc = lib.caroli_ctx_create(device, ctypes.byref(h))
        if rc != OK:
            why = "no usable CUDA device" if rc == EUNAVAILABLE else lib.caroli_last_error(None).decode()
            raise NativeError(rc, f"caroli_ctx_create: {why}")
        self.h = h
        self.lib = lib

    def check(self, rc):
        if rc != OK:
            raise NativeError(rc, self.lib.caroli_last_error(self.h).decode())

    def region_begin(self):
        self.check(self.lib.caroli_region_begin(self.h))

    def region_end(self):
        ms, n = ctypes.c_double(), ctypes.c_int64()
        self.check(self.lib.caroli_region_end(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_refine_options(self, max_iters=6, tol=1e-10, inner_tol=1e-10):
        """Mixed-precision refinement controls (``caroli_set_refine_options``)."""
        self.check(self.lib.caroli_set_refine_options(self.h, int(max_iters), float(tol), float(inner_tol)))

    def set_tensor_cores(self, enable=True):
        """f32 rank-32 updates on the tcgen05 tensor cores (True) or the CUDA cores."""
        self.check(self.lib.caroli_set_tensor_cores(self.h, 1 if enable else 0))

    def set_mixed_max_channels(self, channels=96):
        """Mixed-precision block solves with more sources than ``channels`` take the FP64 path."""
        self.check(self.lib.caroli_set_mixed_max_channels(self.h, int(channels)))

    def set_autotune(self, enable=True):
        """The f32 factorization's schedule picked per plan set by timing trials (default on)."""
        self.check(self.lib.caroli_set_autotune(self.h, 1 if enable else 0))

    def set_schedule(self, small_max=96, update_mode=1):
        """The schedule used while the autotuner is off (see caroli_set_schedule)."""
        self.check(self.lib.caroli_set_schedule(self.h, int(small_max), int(update_mode)))

    def set_sweep_columns(self, min_columns=32):
        """Batches with this many right-hand-side columns sweep on the tensor cores."""
        self.check(self.lib.caroli_set_sweep_columns(self.h, int(min_columns)))

    def set_small_threads(self, threads=512):
        """Threads of a CTA factoring a front of 64 to 96 variables (256 or 512)."""
        self.check(self.lib.caroli_set_small_threads(self.h, int(threads)))

    def set_graphs(self, enable=True):
        """Replay a repeated batch's factorization as a CUDA graph (default on)."""
        self.check(self.lib.caroli_set_graphs(self.h, 1 if enable else 0))

    def last_schedule(self):
        """The last batch's schedule: small_max, the update mode (2: tensor cores with the split
        Schur GEMM, 1: tensor-core rank-32 updates, 0: CUDA cores), tuned, the trial times (ms) of
        (48, 64, 96) x (2, 1, 0), graph replays and captures so far."""
        sm, tc, tu = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        ms = np.zeros(9)
        rep, cap = ctypes.c_int64(), ctypes.c_int64()
        self.check(self.lib.caroli_last_schedule(self.h, ctypes.byref(sm), ctypes.byref(tc), ctypes.byref(tu), ptr(ms),
                                                 ctypes.byref(rep), ctypes.byref(cap)))
        return {"small_max": sm.value, "update_mode": tc.value, "tuned": bool(tu.value),
                "trial_ms": [None if np.isnan(x) else float(x) for x in ms], "graph_replays": rep.value,
                "graph_captures": cap.value}

    def set_wait_limit(self, polls=-1):
        """Polls of a tensor-core pipeline wait before it gives up (negative: the default)."""
        self.check(self.lib.caroli_set_wait_limit(self.h, int(polls)))

    def solve_multi(self, plans, slots, configs, precision=DOUBLE):
        """T for instances of several plans of this context in one batch (``caroli_solve_multi``)."""
        ids = np.ascontiguousarray([p.id for p in plans], np.int32)
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        n = len(ids)
        t = np.zeros(n)
        st = np.zeros(n, np.int32)
        err = np.zeros(n)
        self.check(self.lib.caroli_solve_multi(self.h, n, ptr(ids), ptr(slots), ptr(configs), precision, ptr(t),
                                               ptr(st), ptr(err)))
        return t, st, err

    def kernel_classes(self):
        return [self.lib.caroli_kernel_class_name(k).decode() for k in range(self.lib.caroli_kernel_classes())]

    def probe(self, kclass):
        self.check(self.lib.caroli_probe_kernel(self.h, kclass))

    def kernel_stats(self, kclass, reset=False):
        n, f, b, ms = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.check(self.lib.caroli_kernel_stats(self.h, kclass, ctypes.byref(n), ctypes.byref(f), ctypes.byref(b),
                                                ctypes.byref(ms), int(reset)))
        return {"launches": n.value, "flops": f.value, "bytes": b.value, "ms": ms.value}

    def close(self):
        if self.h:
            self.lib.caroli_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """A system uploaded to a context (``caroli_plan_upload``) with its values and Σ slots."""

    def __init__(self, ctx: Context, system):
        self.ctx = ctx
        s = system
        self._keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            self._keep.append(a)
            return a

        lp = arr(np.cumsum([0] + [len(b.left) for b in s.blocks]), np.int64)
        rp = arr(np.cumsum([0] + [len(b.right) for b in s.blocks]), np.int64)
        lf = arr(np.concatenate([b.left for b in s.blocks]) if s.blocks else [], np.int64)
        rt = arr(np.concatenate([b.right for b in s.blocks]) if s.blocks else [], np.int64)
        pid = ctypes.c_int()
        ctx.check(ctx.lib.caroli_plan_upload(
            ctx.h, s.n, ptr(arr(s.row_ptr, np.int64)), ptr(arr(s.cols, np.uint32)), len(s.site_offsets), s.dim,
            ptr(arr(s.cells, np.int64)), ptr(arr(s.site_offsets, np.int64)), ptr(arr(s.site_orbitals, np.int64)),
            ptr(arr(s.range, np.int64)), len(s.interior), ptr(arr(s.interior, np.int64)), len(s.blocks),
            ptr(arr(s.labels, np.int32)), ptr(lp), ptr(lf), ptr(rp), ptr(rt), ctypes.byref(pid)))
        self.id = pid.value
        self._keep = []
        self.nblocks = len(s.blocks)
        self.slots = {}

    def info(self, block):
        vals = [ctypes.c_int64() for _ in range(5)]
        self.ctx.check(self.ctx.lib.caroli_plan_info(self.ctx.h, self.id, block, *[ctypes.byref(v) for v in vals]))
        return dict(zip(["fronts", "max_n", "max_ne", "root_n", "arena_elems"], [v.value for v in vals]))

    def fronts(self, block):
        """``(n, ne, level)`` arrays of the block's tree fronts (post-order)."""
        cnt = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_plan_fronts(self.ctx.h, self.id, block, 0, None, None, None,
                                                       ctypes.byref(cnt)))
        n = np.zeros(cnt.value, np.int32); ne = np.zeros(cnt.value, np.int32); lv = np.zeros(cnt.value, np.int32)
        self.ctx.check(self.ctx.lib.caroli_plan_fronts(self.ctx.h, self.id, block, cnt.value, ptr(n), ptr(ne), ptr(lv),
                                                       ctypes.byref(cnt)))
        return n, ne, lv

    def upload_values(self, values):
        """H values of every configuration: an (nconfigs, nnz) complex128 array (used in place
        when C-contiguous) or a list of per-configuration arrays."""
        if isinstance(values, np.ndarray) and values.ndim == 2 and values.dtype == np.complex128 \
                and values.flags.c_contiguous:
            v = values
        else:
            v = np.ascontiguousarray(np.stack(values), dtype=np.complex128)
        self.ctx.check(self.ctx.lib.caroli_values_upload(self.ctx.h, self.id, v.shape[0], ptr(v)))

    def upload_sigma(self, slot, energy, sigmas, w_right=None):
        """Σ of every block; ``w_right[b]`` (nr x channels) with W W^† = Γ_R, or None."""
        ls = [np.asfortranarray(sl, dtype=np.complex128) for sl, _ in sigmas]
        rs = [np.asfortranarray(sr, dtype=np.complex128) for _, sr in sigmas]
        pl = np.array([a.ctypes.data for a in ls], dtype=np.uintp)
        pr = np.array([a.ctypes.data for a in rs], dtype=np.uintp)
        pw = ch = None
        if w_right is not None:
            ws = [np.asfortranarray(w, dtype=np.complex128) for w in w_right]
            pw = np.array([w.ctypes.data if w.size else 0 for w in ws], dtype=np.uintp)
            ch = np.array([w.shape[1] for w in ws], dtype=np.int32)
            self._keep_w = ws
        self.ctx.check(self.ctx.lib.caroli_sigma_upload(self.ctx.h, self.id, slot, energy, ptr(pl), ptr(pr),
                                                        ptr(pw), ptr(ch)))

    def solve(self, slots, configs, precision=DOUBLE):
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        n = len(slots)
        t = np.zeros(n)
        st = np.zeros(n, np.int32)
        err = np.zeros(n)
        self.ctx.check(self.ctx.lib.caroli_solve_batch(self.ctx.h, self.id, n, ptr(slots), ptr(configs), precision,
                                                       ptr(t), ptr(st), ptr(err)))
        return t, st, err

    def last_stats(self):
        fb, it = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_last_stats(self.ctx.h, ctypes.byref(fb), ctypes.byref(it)))
        return fb.value, it.value

    def last_refine_steps(self):
        """(GMRES steps summed over the block solves, steps the batch launched) of the last solve."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_last_refine_steps(self.ctx.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def last_phases(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.ctx.lib.caroli_last_phases(self.ctx.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def upload_derivs(self, derivs):
        """``derivs[c][k]``: dH/dp_k values of configuration c on the pattern."""
        d = np.ascontiguousarray(np.asarray(derivs, dtype=np.complex128))
        nparams = d.shape[1] if d.ndim == 3 else 0
        self.ctx.check(self.ctx.lib.caroli_derivs_upload(self.ctx.h, self.id, nparams, ptr(d) if nparams else None))
        self.nparams = nparams

    def solve_grad(self, slots, configs, n):
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt = len(slots)
        t = np.zeros(cnt)
        st = np.zeros(cnt, np.int32)
        dv = np.zeros((cnt, n))
        npar = getattr(self, "nparams", 0)
        dp = np.zeros((cnt, max(npar, 1)))
        self.ctx.check(self.ctx.lib.caroli_transmission_with_grad(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs),
                                                                  ptr(t), ptr(st), ptr(dv), ptr(dp) if npar else None))
        return t, st, dv, dp[:, :npar]

    def scattering_states(self, slots, configs, w_left, w_right, n):
        """ψ_L, ψ_R (n x channels, complex128) of each instance: ``w_left[i][b]``, ``w_right[i][b]``
        are the lead factors of block b (``caroli_scattering_states``). Returns ``(states, status)``
        with ``states[i] = (ψ_L, ψ_R)``."""
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt = len(slots)
        keep = []

        def table(ws):
            mats = [np.asfortranarray(w, dtype=np.complex128) for per in ws for w in per]
            keep.extend(mats)
            p = np.array([m.ctypes.data if m.size else 0 for m in mats] or [0], dtype=np.uintp)
            c = np.array([m.shape[1] for m in mats] or [0], dtype=np.int32)
            return p, c

        pl, cl = table(w_left)
        pr, cr = table(w_right)
        nb = self.nblocks
        outs = []
        for i in range(cnt):
            a = np.zeros((n, int(cl[i * nb:(i + 1) * nb].sum())), np.complex128, order="F")
            b = np.zeros((n, int(cr[i * nb:(i + 1) * nb].sum())), np.complex128, order="F")
            outs.append((a, b))
        po_l = np.array([a.ctypes.data if a.size else 0 for a, _ in outs] or [0], dtype=np.uintp)
        po_r = np.array([b.ctypes.data if b.size else 0 for _, b in outs] or [0], dtype=np.uintp)
        st = np.zeros(max(cnt, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_scattering_states(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs),
                                                             ptr(pl), ptr(cl), ptr(pr), ptr(cr), ptr(po_l), ptr(po_r),
                                                             ptr(st)))
        return outs, st[:cnt]

    def lead_modes(self, block, side, y, sc):
        """Cell eigenvectors of a block's lead with a scalar coupling (``caroli_lead_modes``)."""
        y = np.asfortranarray(y, dtype=np.complex128)
        self.ctx.check(self.ctx.lib.caroli_lead_modes(self.ctx.h, self.id, block, side, y.shape[0], ptr(y), sc))

    def sigma_from_modes(self, slot, energy, blocks):
        """``blocks[b] = (1/λ_L, λ_R, channel modes, channel weights)`` (``caroli_sigma_from_modes``)."""
        keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x if len(x) else np.zeros(1), dtype=dt)
            keep.append(a)
            return a

        dl = np.array([arr(b[0], np.complex128).ctypes.data for b in blocks], dtype=np.uintp)
        dr = np.array([arr(b[1], np.complex128).ctypes.data for b in blocks], dtype=np.uintp)
        nc = np.array([len(b[2]) for b in blocks], dtype=np.int32)
        cm = np.array([arr(b[2], np.int32).ctypes.data for b in blocks], dtype=np.uintp)
        cw = np.array([arr(b[3], np.float64).ctypes.data for b in blocks], dtype=np.uintp)
        self.ctx.check(self.ctx.lib.caroli_sigma_from_modes(self.ctx.h, self.id, slot, energy, ptr(dl), ptr(dr),
                                                            ptr(nc), ptr(cm), ptr(cw)))

    def generate_values(self, clean_values, entries, nconfigs, first_config=0):
        """H values of ``nconfigs`` configurations generated on the device
        (``caroli_values_generate``): ``entries`` is a list of ``Disorder`` with the spin matrices
        kept alive by the caller."""
        clean = np.ascontiguousarray(clean_values, np.complex128)
        arr = (Disorder * max(len(entries), 1))(*entries)
        self.ctx.check(self.ctx.lib.caroli_values_generate(self.ctx.h, self.id, ptr(clean), len(entries),
                                                           ctypes.cast(arr, ctypes.c_void_p), nconfigs, first_config))

    def download_values(self, config, nnz):
        out = np.zeros(nnz, np.complex128)
        self.ctx.check(self.ctx.lib.caroli_values_download(self.ctx.h, self.id, config, ptr(out)))
        return out

    def root_green(self, slots, configs, kept_sizes):
        """The FP64 root Green's function on the kept orbitals of every (instance, block)
        (``caroli_root_green``): ``(g, status)`` with ``g[i][b]`` kept x kept."""
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt, nb = len(slots), self.nblocks
        outs = [np.zeros((max(kept_sizes[b], 1), max(kept_sizes[b], 1)), np.complex128, order="F")
                for _ in range(cnt) for b in range(nb)]
        po = np.array([o.ctypes.data for o in outs] or [0], dtype=np.uintp)
        kept = np.zeros(max(cnt * nb, 1), np.int32)
        st = np.zeros(max(cnt, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_root_green(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs), ptr(po),
                                                      ptr(kept), ptr(st)))
        res = []
        for i in range(cnt):
            res.append([outs[i * nb + b][:kept[i * nb + b], :kept[i * nb + b]] for b in range(nb)])
        return res, st[:cnt]

    def transmission_matrices(self, slots, configs, w_left, nr):
        """t = W_L^† G_LR W_R per (instance, block) (``caroli_transmission_matrix``); ``w_left[i][b]``
        and ``nr[b]`` the right slice sizes. Returns ``(t, status)`` with ``t[i][b]`` cl x cr."""
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt = len(slots)
        mats = [np.asfortranarray(w, dtype=np.complex128) for inst in w_left for w in inst]
        pw = np.array([m.ctypes.data if m.size else 0 for m in mats] or [0], dtype=np.uintp)
        cl = np.array([m.shape[1] for m in mats] or [0], dtype=np.int32)
        nb = self.nblocks
        outs = [np.zeros((max(int(cl[q]), 1) * max(int(nr[q % nb]), 1),), np.complex128) for q in range(len(mats))]
        po = np.array([o.ctypes.data for o in outs] or [0], dtype=np.uintp)
        cr = np.zeros(max(len(mats), 1), np.int32)
        st = np.zeros(max(cnt, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_transmission_matrix(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs),
                                                               ptr(pw), ptr(cl), ptr(po), ptr(cr), ptr(st)))
        res = []
        for i in range(cnt):
            row = []
            for b in range(nb):
                q = i * nb + b
                k, c = int(cl[q]), int(cr[q])
                row.append(outs[q][:k * c].reshape((k, c), order="F"))
            res.append(row)
        return res, st[:cnt]

    def multi_leads(self, nleads, lead_ptr, lead_orbitals):
        """Leads of a multi-terminal plan (``caroli_multi_leads``)."""
        lp = np.ascontiguousarray(lead_ptr, np.int64)
        lo = np.ascontiguousarray(lead_orbitals if len(lead_orbitals) else [0], np.int64)
        self.ctx.check(self.ctx.lib.caroli_multi_leads(self.ctx.h, self.id, nleads, ptr(lp), ptr(lo)))
        self.nleads = nleads

    def upload_multi_sigma(self, slot, energy, sigmas):
        """``sigmas[b][p]``: Σ_p of block b on the lead's orbitals, or None."""
        mats = [None if m is None else np.asfortranarray(m, dtype=np.complex128) for row in sigmas for m in row]
        pt = np.array([0 if m is None or m.size == 0 else m.ctypes.data for m in mats] or [0], dtype=np.uintp)
        self.ctx.check(self.ctx.lib.caroli_multi_sigma_upload(self.ctx.h, self.id, slot, energy, ptr(pt)))

    def multi_scattering_states(self, slots, configs, w, n, nleads):
        """``w[i][b][p]``: W of lead p in block b for instance i (np x channels, or None).
        Returns ``(states, status)`` with ``states[i]`` the list of ψ_p (n x channels)."""
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt = len(slots)
        mats = [None if m is None else np.asfortranarray(m, dtype=np.complex128)
                for inst in w for blk in inst for m in blk]
        pw = np.array([0 if m is None or m.size == 0 else m.ctypes.data for m in mats] or [0], dtype=np.uintp)
        ch = np.array([0 if m is None else m.shape[1] for m in mats] or [0], dtype=np.int32)
        nb = self.nblocks
        outs = []
        for i in range(cnt):
            per = []
            for p in range(nleads):
                cols = sum(int(ch[(i * nb + b) * nleads + p]) for b in range(nb))
                per.append(np.zeros((n, cols), np.complex128, order="F"))
            outs.append(per)
        po = np.array([m.ctypes.data if m.size else 0 for per in outs for m in per] or [0], dtype=np.uintp)
        st = np.zeros(max(cnt, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_multi_scattering_states(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs),
                                                                   ptr(pw), ptr(ch), ptr(po), ptr(st)))
        return outs, st[:cnt]

    def multi_sector(self, slot, config, precision, label_lead, gammas):
        """One instance of ``caroli_multi_sector_transmissions``: ``gammas[b][k]`` per block and
        label (or None). Returns ``(t, status)`` with t nlabels x nlabels."""
        nl = len(label_lead)
        mats = [None if g is None else np.asfortranarray(g, dtype=np.complex128) for row in gammas for g in row]
        pg = np.array([0 if m is None or m.size == 0 else m.ctypes.data for m in mats] or [0], dtype=np.uintp)
        ll = np.ascontiguousarray(label_lead, np.int32)
        sl = np.array([slot], np.int32)
        cf = np.array([config], np.int32)
        t = np.zeros((nl, nl))
        st = np.zeros(1, np.int32)
        self.ctx.check(self.ctx.lib.caroli_multi_sector_transmissions(self.ctx.h, self.id, 1, ptr(sl), ptr(cf),
                                                                      precision, nl, ptr(ll), ptr(pg), ptr(t),
                                                                      ptr(st)))
        return t, int(st[0])

    def multi_solve(self, slots, configs, precision, nleads):
        slots = np.ascontiguousarray(slots, np.int32)
        configs = np.ascontiguousarray(configs, np.int32)
        cnt = len(slots)
        t = np.zeros((max(cnt, 1), nleads, nleads))
        st = np.zeros(max(cnt, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_multi_transmissions(self.ctx.h, self.id, cnt, ptr(slots), ptr(configs),
                                                               precision, ptr(t), ptr(st)))
        return t[:cnt], st[:cnt]

    def gamma_override(self, slot, gammas):
        """``gammas[b] = (Γ_L, Γ_R)`` replacing the slot's trace broadenings (``caroli_gamma_override``)."""
        gl = [np.asfortranarray(a, dtype=np.complex128) for a, _ in gammas]
        gr = [np.asfortranarray(b, dtype=np.complex128) for _, b in gammas]
        pl = np.array([a.ctypes.data for a in gl], dtype=np.uintp)
        pr = np.array([b.ctypes.data for b in gr], dtype=np.uintp)
        self.ctx.check(self.ctx.lib.caroli_gamma_override(self.ctx.h, self.id, slot, ptr(pl), ptr(pr)))

    def last_job_steps(self):
        """GMRES steps of each block solve of the last batch (``caroli_last_job_steps``)."""
        cnt = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_last_job_steps(self.ctx.h, 0, None, ctypes.byref(cnt)))
        out = np.zeros(max(cnt.value, 1), np.int32)
        self.ctx.check(self.ctx.lib.caroli_last_job_steps(self.ctx.h, cnt.value, ptr(out), ctypes.byref(cnt)))
        return out[:cnt.value]

    def last_job_info(self):
        cnt = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_last_job_info(self.ctx.h, 0, None, None, None, ctypes.byref(cnt)))
        it = np.zeros(cnt.value, np.int32); pt = np.zeros(cnt.value, np.int32); st = np.zeros(cnt.value, np.int32)
        self.ctx.check(self.ctx.lib.caroli_last_job_info(self.ctx.h, cnt.value, ptr(it), ptr(pt), ptr(st),
                                                         ctypes.byref(cnt)))
        return it, pt, st

    def last_timing(self):
        ms, launches = ctypes.c_double(), ctypes.c_int64()
        self.ctx.check(self.ctx.lib.caroli_last_timing(self.ctx.h, ctypes.byref(ms), ctypes.byref(launches)))
        return ms.value, launches.value
