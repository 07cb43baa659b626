#!/usr/bin/env python3
"""Benchmark of the GB300 nested-dissection transmission (one JSON line on rank 0).

Workload (the configuration the headline metric is quoted on): BHZ ribbon 200 x 64 sites
(51 200 complex unknowns, two spin blocks of 25 600), magnetic disorder at concentration 0.2 with
exchange J = 0.4, opposite-g spin matrices (s_z tau_z), moments polarised along z, impurities at
seeded random sites (CLI convention: configuration c seeded with 1 + c); 33 energies uniform in
[-0.16, 0.16] x 8 configurations = 264 transmissions per step. Synthetic inputs of that shape
(no dataset is involved); the lead self-energies are computed once per energy on the host and
stay resident, as the reference reuses them for every configuration.

A step is one batched pass of the path over the 264 (energy, configuration) solves:
- ``value``: solves/s of the mixed path (complex-f32 multifrontal factors + FP64 iterative
  refinement to |dT| <= 1e-8), inputs resident in HBM, device time between CUDA events on the
  library's stream (the stream every kernel of the library runs on);
- ``e2e``: the same through the public API with host buffers: every step uploads the H values of
  the 8 configurations and the self-energies of the 33 energies from host memory and reads the
  transmissions back;
- beside them the plain FP64 GPU path on the same batch (the denominator of the target ratio),
  and max |dT| of the mixed path against it.
The arena of a step (~33 GB) is far larger than L2, so no L2 flush is needed between steps.

``--impl reference`` times the reference's CPU path on the host cores: the C++ restatement of
caroli's NestedTwoTerminal (oracle/, FP64, OpenMP over solves), since the reference itself (Rust)
cannot be built here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "T(E) solves/s, mixed+refined vs FP64 GPU at |ΔT|≤1e-8; grad/fwd time ratio"
# Kernel classes whose algorithmic work is counted in flops (the rest in bytes).
FLOP_CLASSES = {"large_front_panel", "large_front_update", "root_inverse", "trace", "refine_residual"}
WORKLOAD = "bhz-magnetic-200x64: BHZ 200x64, magnetic c=0.2 J=0.4 opposite-g polarised, 33 E in [-0.16,0.16] x 8 configs"


def build_workload(length=200, width=64, configs=8, energies=33):
    from caroli_gb300 import NestedTwoTerminal, Region, bhz
    from caroli_gb300.disorder import Moments, disordered
    from caroli_gb300.model import bhz_spin

    m = bhz()
    region = Region.cuboid(m.lattice, [length, width, 0])
    entry = {"kind": "magnetic", "concentration": 0.2, "exchange": 0.4, "moments": Moments.polarized(1.0),
             "spin": bhz_spin("opposite-g")}
    t0 = time.perf_counter()
    devices = [disordered(m, region, [entry], c) for c in range(configs)]
    sys_ = NestedTwoTerminal.from_models(devices, m, region, 0)
    sys_._host_build_s = time.perf_counter() - t0  # the configurations' H values built on the host
    sys_._workload = (m, region, [entry], configs)
    es = np.linspace(-0.16, 0.16, energies)
    sigmas = [sys_.self_energies(e) for e in es]
    pairs = [(s, c) for s in sigmas for c in range(configs)]
    return sys_, sigmas, pairs


def time_generation(sys_, ctx):
    """The workload's configurations generated on the device (caroli_values_generate) instead of
    built on the host and uploaded: device time, and whether the values are the host's exactly."""
    from caroli_gb300 import NestedTwoTerminal

    m, region, entries, configs = sys_._workload
    gen = NestedTwoTerminal.from_disorder(m, m, region, 0, entries, configs)
    gen.plan()  # plan upload and a first generation
    ctx.region_begin()
    gen._generate(*gen._disorder)
    ms, launches = ctx.region_end()
    same_pattern = np.array_equal(gen.system.row_ptr, sys_.system.row_ptr) and np.array_equal(
        gen.system.cols, sys_.system.cols)
    identical = same_pattern and all(np.array_equal(gen.generated_values(c), sys_.system.values[c])
                                     for c in range(configs))
    return {"configs": configs, "device_ms": ms, "launches": int(launches),
            "host_build_s": sys_._host_build_s, "values_identical_to_host": bool(identical),
            "h2d_bytes_saved": int(sum(v.nbytes for v in sys_.system.values))}


class Clocks:
    """nvidia-smi samples of SM clocks and throttle reasons during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "out", "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profiled_traffic(kernel_class):
    """DRAM bytes per step of a kernel class from the committed ncu summary of this workload
    (profiles/launches_mixed_bhz200x64.md), or None."""
    path = os.path.join(ROOT, "profiles", "launches_mixed_bhz200x64.md")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and parts[0] == "traffic" and parts[1] == kernel_class and parts[3] == "GB":
                    return float(parts[2]) * 1e9
    except OSError:
        pass
    return None


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return {"hbm_gbs": p["hbm_gbs"], "bf16_tflops": p["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def fp64_gemm_tflops(n=4096, reps=5):
    """FP64 roof of this GPU, measured here: torch.matmul of two n x n float64 matrices (cuBLAS
    DGEMM, 2 n^3 flops), best of `reps` by CUDA events."""
    import torch

    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def gradient_workload(length=100, width=40, energies=16):
    """BHZ 100 x 40 with Anderson disorder W = 0.02 and magnetic impurities (concentration 0.1,
    J = 0.3, isotropic moments, so the two spin blocks couple: one block of 16 000 orbitals), with
    dH/dJ = H(J = 1) - H(J = 0) on the system's pattern (H is linear in J); 16 energies."""
    from caroli_gb300 import NestedTwoTerminal, Region, bhz
    from caroli_gb300.disorder import Moments, disordered
    from caroli_gb300.model import SparseMatrix, bhz_spin
    from caroli_gb300.system import merge_patterns

    m = bhz()
    region = Region.cuboid(m.lattice, [length, width, 0])

    def entries(j):
        return [{"kind": "anderson", "strength": 0.02},
                {"kind": "magnetic", "concentration": 0.1, "exchange": j, "moments": Moments.isotropic(),
                 "spin": bhz_spin("opposite-g")}]

    sys_ = NestedTwoTerminal.from_models([disordered(m, region, entries(0.3), 0)], m, region, 0)
    h1 = disordered(m, region, entries(1.0), 0).sparse_hamiltonian(region)
    h0 = disordered(m, region, entries(0.0), 0).sparse_hamiltonian(region)
    s = sys_.system
    base = SparseMatrix(s.n, s.row_ptr, s.cols, np.zeros(s.nnz, complex))
    _, _, (v1, v0, _) = merge_patterns([h1, h0, base])
    sys_.set_parameter_derivatives([[v1 - v0]])
    sigmas = [sys_.self_energies(e) for e in np.linspace(-0.16, 0.16, energies)]
    return sys_, sigmas


def time_gradient(steps):
    """Device time of T with dT/dV (every orbital) and dT/dJ over the time of T alone, both on the
    mixed path, on the same 16 points."""
    from caroli_gb300 import Precision
    from caroli_gb300.nested import context

    sys_, sigmas = gradient_workload()
    ctx = context(0)
    cfg = [0] * len(sigmas)
    for _ in range(2):
        sys_.solve_batch(sigmas, cfg, Precision.MIXED)
        sys_.transmissions_with_grad(sigmas, cfg)
    ctx.region_begin()
    for _ in range(steps):
        t_f, st_f, _ = sys_.solve_batch(sigmas, cfg, Precision.MIXED)
    fwd_ms, _ = ctx.region_end()
    ctx.region_begin()
    for _ in range(steps):
        t_g, st_g, dv, dp = sys_.transmissions_with_grad(sigmas, cfg)
    grad_ms, _ = ctx.region_end()
    return {"value": grad_ms / fwd_ms, "fwd_ms_per_step": fwd_ms / steps, "grad_ms_per_step": grad_ms / steps,
            "workload": "BHZ 100x40, Anderson W=0.02 + magnetic c=0.1 J=0.3 isotropic, 16 E; dT/dV (16000) + dT/dJ",
            "max_abs_dT_fwd_vs_grad": float(np.max(np.abs(t_f - t_g))),
            "status_ok": bool((st_g == 0).all() and (st_f == 0).all())}


# ---- The many-ribbon workload: 256 graphene zigzag ribbons of uneven sizes x 64 energies ------------
RIBBONS = ("graphene-ribbons: 256 zigzag ribbons, widths 40-160 x lengths 100-400 cells (xoshiro seed 1), "
           "Anderson W=1.0 (seed 1000003 s + ribbon), 64 E in [-0.5,0.5]; mixed c64 + f64 refinement")


def ribbon_shapes(count, seed):
    """(width, length) of each ribbon: uniform integers in [40, 160] and [100, 400] cells drawn in
    that order from xoshiro256** seed_from_u64(seed)."""
    from caroli_gb300.disorder import Xoshiro256

    rng = Xoshiro256.seed_from_u64(seed)
    return [(rng.integer(40, 160), rng.integer(100, 400)) for _ in range(count)]


def _ribbon_system(args):
    """Pool worker: the System of ribbon r (graphene zigzag, clean leads, Anderson w (u - 1/2) per
    site from seed_from_u64(1 000 003 seed + r), the benchmark's convention of
    caroli-bench/src/main.rs:120-126)."""
    seed, r, width, length, w = args
    from caroli_gb300 import Region, graphene
    from caroli_gb300.disorder import ScalarPotential, bench_disorder
    from caroli_gb300.system import build_system

    clean = graphene()
    region = Region.cuboid(clean.lattice, [length, width, 0])
    pot = bench_disorder(seed, r, length, width, 2, w)
    return build_system([clean.with_onsite_term(ScalarPotential(pot, width, 2, 1))], clean, region, 0)


def _ribbon_sigma(args):
    """Pool worker: the clean zigzag leads' Σ_L, Σ_R and W_R of a width at every energy."""
    width, energies = args
    from caroli_gb300 import NestedTwoTerminal, Region, graphene

    clean = graphene()
    lead = NestedTwoTerminal.from_model(clean, clean, Region.cuboid(clean.lattice, [3, width, 0]), 0)
    out = []
    for e in energies:
        s = lead.self_energies(e)
        out.append((s.energy, s.blocks[0][0], s.blocks[0][1], s.w_right()[0]))
    return width, out


def ribbons_workload(count=256, energies=64, seed=1, w=1.0, processes=None):
    """The ribbons (NestedTwoTerminal each) and, per ribbon width, the LeadSelfEnergies of every
    energy. Host work (model builds, lead modes) runs on a spawn pool before any GPU call."""
    import multiprocessing as mp

    from caroli_gb300 import LeadSelfEnergies, NestedTwoTerminal

    shapes = ribbon_shapes(count, seed)
    es = list(np.linspace(-0.5, 0.5, energies))
    widths = sorted({wd for wd, _ in shapes})
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(processes or os.cpu_count() or 1) as pool:
        # Largest ribbons first so the pool's tail is short.
        order = sorted(range(count), key=lambda r: -shapes[r][0] * shapes[r][1])
        built = pool.map(_ribbon_system, [(seed, r, shapes[r][0], shapes[r][1], w) for r in order], chunksize=1)
        sig = dict(pool.map(_ribbon_sigma, [(wd, es) for wd in sorted(widths, reverse=True)], chunksize=1))
    systems = [None] * count
    for r, s in zip(order, built):
        systems[r] = s
    host_s = time.perf_counter() - t0
    ribbons = [NestedTwoTerminal(s) for s in systems]
    sigmas = {}
    for wd in widths:
        row = []
        for e, sl, sr, wr in sig[wd]:
            lse = LeadSelfEnergies(e, [(sl, sr)])
            lse._w_right = [wr]
            row.append(lse)
        sigmas[wd] = row
    return ribbons, shapes, sigmas, es, host_s


def run_ribbons(args):
    """The many-ribbon workload in one batched launch sequence per step (caroli_solve_multi)."""
    from caroli_gb300 import Precision, solve_systems
    from caroli_gb300.nested import context

    ribbons, shapes, sigmas, es, host_s = ribbons_workload(args.ribbons, args.energies)
    ne = len(es)
    items = [(ribbons[r], sigmas[shapes[r][0]][k], 0) for r in range(len(ribbons)) for k in range(ne)]
    ctx = context(0)
    ctx.set_refine_options(args.refine_max_iters, 1e-10, 1e-10)
    t0 = time.perf_counter()
    solve_systems(items, Precision.MIXED)  # plan and Σ uploads, first factorization
    upload_s = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        solve_systems(items, Precision.MIXED)
    with Clocks(0) as clk:
        ctx.region_begin()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            t_mixed, st_mixed, _ = solve_systems(items, Precision.MIXED)
        ms, launches = ctx.region_end()
        wall = time.perf_counter() - w0
    plan0 = ribbons[0].plan()
    schedule = ctx.last_schedule()
    fallbacks, max_iters = plan0.last_stats()
    # Per block solve of the last step: GMRES steps, outer iterations, perturbed pivots, status.
    j_iters, j_pert, j_stat = plan0.last_job_info()
    j_steps = plan0.last_job_steps()
    job_steps, batch_steps = plan0.last_refine_steps()

    def hist(a, cap):
        a = np.minimum(np.asarray(a), cap)
        vals, cnt = np.unique(a, return_counts=True)
        return {int(v): int(c) for v, c in zip(vals, cnt)}

    refinement = {"max_outer_iterations": int(max_iters), "fp64_recomputed_solves": int(fallbacks),
                  "gmres_steps_total": int(job_steps), "batch_steps": int(batch_steps),
                  "gmres_steps_hist": hist(j_steps, 80), "outer_iterations_hist": hist(j_iters, 10),
                  "perturbed_pivots_hist": hist(j_pert, 32),
                  "mean_steps_unperturbed": float(np.mean(j_steps[j_pert == 0])) if (j_pert == 0).any() else None,
                  "mean_steps_perturbed": float(np.mean(j_steps[j_pert > 0])) if (j_pert > 0).any() else None}
    # FP64 on every 8th energy of every ribbon (the ratio's denominator), and the mixed T there.
    sub = [i for i in range(len(items)) if (i % ne) % 8 == 0]
    sub_items = [items[i] for i in sub]
    solve_systems(sub_items, Precision.DOUBLE)
    ctx.region_begin()
    t_dbl, st_dbl, _ = solve_systems(sub_items, Precision.DOUBLE)
    ms_dbl, _ = ctx.region_end()
    ctx.region_begin()
    t_msub, _, _ = solve_systems(sub_items, Precision.MIXED)
    ms_msub, _ = ctx.region_end()
    dT = np.abs(t_mixed[sub] - t_dbl)
    # End to end: every ribbon's H values uploaded from pinned host memory each step (Σ resident:
    # one copy per ribbon and energy, uploaded once), T read back.
    import torch as _torch

    def pinned(a):
        buf = _torch.empty(a.size, dtype=_torch.complex128, pin_memory=True).numpy()
        buf[...] = a.ravel()
        return buf.reshape(a.shape)

    host_vals = [pinned(np.stack(rb.system.values)) for rb in ribbons]
    h2d = sum(v.nbytes for v in host_vals) + 3 * 4 * len(items)
    d2h = len(items) * (8 + 4 + 8)
    ctx.region_begin()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        for rb, v in zip(ribbons, host_vals):
            rb.plan().upload_values(v)
        solve_systems(items, Precision.MIXED)
    e2e_ms, _ = ctx.region_end()
    e2e_wall = time.perf_counter() - e0
    roof, kernels = (roofline_probe(ctx, lambda: solve_systems(items, Precision.MIXED), ms / args.steps,
                                    traffic_of=lambda name: None) if args.probe else (None, None))
    # CPU baseline: the oracle on one energy of 16 ribbons spread over the sizes.
    cpu = None
    if args.cpu_sample > 0:
        from oracle import Oracle

        pick = list(range(0, len(ribbons), max(1, len(ribbons) // args.cpu_sample)))[:args.cpu_sample]
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        tref = []
        for r in pick:
            s = sigmas[shapes[r][0]][ne // 2]
            t, st = Oracle(ribbons[r].system).solve_batch([0], [s.energy], [ribbons[r].system.values[0]],
                                                          [s.blocks[0][0]], [s.blocks[0][1]], threads=threads)
            tref.append(t[0])
        dt = time.perf_counter() - t0
        idx = [r * ne + ne // 2 for r in pick]
        cpu = {"value": len(pick) / dt, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"{len(pick)} ribbons spread over the sizes at E = {es[ne // 2]:.4f} (one solve at a time, "
                         f"OpenMP inside), {dt:.1f} s wall",
               "max_abs_dT_vs_gpu_mixed": float(np.abs(np.array(tref) - t_mixed[idx]).max())}
    n = len(items)
    line = {
        "metric": METRIC, "value": n * args.steps / (ms * 1e-3), "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 factors + f64 refinement",
        "data": "synthetic (seeded shapes and disorder of the reference's benchmark conventions; no dataset)",
        "config": {"workload": RIBBONS, "solves_per_step": n, "ribbons": len(ribbons),
                   "unknowns_min_max": [int(min(2 * a * b for a, b in shapes)), int(max(2 * a * b for a, b in shapes))],
                   "distinct_widths": len(sigmas), "parallelism": "replicas x1",
                   "l2": "inputs larger than L2 (every ribbon's fronts per step)"},
        "fp64_gpu": {"value": len(sub) / (ms_dbl * 1e-3), "unit": "solves/s", "ms": ms_dbl,
                     "sample": f"every 8th energy of every ribbon ({len(sub)} solves)",
                     "mixed_ms_same_sample": ms_msub},
        "mixed_over_fp64": ms_dbl / ms_msub,
        "max_abs_dT_vs_fp64": float(dT.max()), "median_abs_dT_vs_fp64": float(np.median(dT)),
        "status_ok": bool((st_mixed == 0).all()), "fp64_recomputed_solves": int(fallbacks),
        "refinement": refinement,
        "e2e": {"value": n * args.steps / (e2e_ms * 1e-3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "wall_s": e2e_wall,
                "note": "H values of every ribbon uploaded each step; lead self-energies resident"},
        "gpu_launches": int(launches), "schedule": schedule, "roofline": roof, "kernels_ms_per_step": kernels,
        "clocks": clk.summary(), "wall_s_timed": wall, "host_setup_s": host_s, "first_solve_with_uploads_s": upload_s, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


# ---- The cubic workload: 3D Anderson wire 64 x 32 x 32, W = 16.5, mixed plus gradient ---------------
CUBIC = ("cubic-anderson-64x32x32: 3D cubic 1-orbital t=1, Anderson W=16.5 (CLI seeds), square 32x32 leads, "
         "32 E in [-1,1] x 16 configurations; mixed c64 + f64 refinement, dT/dV of every site")


def cubic_workload(length=64, width=32, depth=32, configs=16):
    from caroli_gb300 import NestedTwoTerminal, Region, cubic
    from caroli_gb300.disorder import disordered

    m = cubic()
    region = Region.cuboid(m.lattice, [length, width, depth])
    devices = [disordered(m, region, [{"kind": "anderson", "strength": 16.5, "seed": 1}], c) for c in range(configs)]
    return NestedTwoTerminal.from_models(devices, m, region, 0)


def run_cubic(args):
    """A bounded sample of the cubic workload (its 512 solves take minutes in FP64): the energies
    `--cubic-energies` of the 32-point grid x `--configs` configurations, mixed and FP64 on the same
    solves, the gradient (dT/dV of all 65 536 sites) on them, and the oracle on a few."""
    from caroli_gb300 import Precision
    from caroli_gb300.nested import context

    shape = [int(x) for x in args.cubic_shape.split(",")]
    sys_ = cubic_workload(*shape, configs=args.configs)
    grid = np.linspace(-1.0, 1.0, 32)
    pick = [int(k) for k in args.cubic_energies.split(",")]
    sigmas = [sys_.self_energies_on_device(grid[k]) for k in pick]
    pairs = [(s, c) for s in sigmas for c in range(args.configs)]
    S, C = [p[0] for p in pairs], [p[1] for p in pairs]
    ctx = context(0)
    ctx.set_mixed_max_channels(args.mixed_max_channels)
    plan = sys_.plan()
    for _ in range(args.warmup):
        sys_.solve_batch(S, C, Precision.MIXED)
    with Clocks(0) as clk:
        ctx.region_begin()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            t_mixed, st_mixed, _ = sys_.solve_batch(S, C, Precision.MIXED)
        ms, launches = ctx.region_end()
        wall = time.perf_counter() - w0
    phases = plan.last_phases()
    schedule = ctx.last_schedule()
    fallbacks, max_iters = plan.last_stats()
    steps_job, steps_batch = plan.last_refine_steps()
    ctx.region_begin()
    t_dbl, st_dbl, _ = sys_.solve_batch(S, C, Precision.DOUBLE)
    ms_dbl, _ = ctx.region_end()
    dT = np.abs(t_mixed - t_dbl)
    # Gradient on the same solves (host self-energies: the adjoint needs Σ^† on the device too,
    # which the slot holds either way).
    ctx.region_begin()
    t_g, st_g, dv, dp = sys_.transmissions_with_grad(S, C)
    ms_grad, _ = ctx.region_end()
    roof, kernels = roofline_probe(ctx, lambda: sys_.solve_batch(S, C, Precision.MIXED), ms / args.steps,
                                   traffic_of=lambda name: None)
    # The slice products of the refinement (the dominant class here) run in FP64, on the FP64 pipe:
    # their roof is FP64 GEMM throughput, measured in this run beside the tensor-core figure above.
    roof64 = None
    if roof["kernel"] == "refine_residual":
        peak64 = fp64_gemm_tflops()
        roof64 = {"kernel": roof["kernel"], "bound": "fp64", "achieved": roof["achieved"], "peak": peak64,
                  "unit": "TFLOP/s", "frac": roof["achieved"] / peak64,
                  "note": "peak = torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5, measured in this run"}
    cpu = None
    if args.cpu_sample > 0:
        from oracle import Oracle

        hs = sys_.self_energies(grid[pick[0]])
        threads = os.cpu_count() or 1
        orc = Oracle(sys_.system)
        t0 = time.perf_counter()
        tref, st = orc.solve_batch([0] * args.cpu_sample, [hs.energy] * args.cpu_sample,
                                   [sys_.system.values[c] for c in range(args.cpu_sample)],
                                   [hs.blocks[0][0]] * args.cpu_sample, [hs.blocks[0][1]] * args.cpu_sample,
                                   threads=threads)
        dt = time.perf_counter() - t0
        cpu = {"value": args.cpu_sample / dt, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} configurations at E = {hs.energy:.4f}, {dt:.1f} s wall",
               "max_abs_dT_vs_gpu_mixed": float(np.abs(tref - t_mixed[:args.cpu_sample]).max())}
    n = len(pairs)
    line = {
        "metric": METRIC, "value": n * args.steps / (ms * 1e-3), "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 factors + f64 refinement",
        "data": "synthetic (seeded Anderson disorder of the reference's CLI conventions; no dataset)",
        "config": {"workload": CUBIC, "solves_per_step": n, "sample": f"energies {pick} of 32 x {args.configs} "
                   "configurations", "unknowns": sys_.system.n, "lead_channels": [int(len(s.blocks[0][2])) for s in sigmas],
                   "parallelism": "replicas x1", "l2": "inputs larger than L2 (fronts ~1.3 GB per solve)"},
        "fp64_gpu": {"value": n / (ms_dbl * 1e-3), "unit": "solves/s", "ms_per_step": ms_dbl},
        "mixed_over_fp64": ms_dbl / (ms / args.steps),
        "max_abs_dT_vs_fp64": float(dT.max()), "max_rel_dT_vs_fp64": float((dT / np.maximum(np.abs(t_dbl), 1e-300)).max()),
        "phases_ms": {"factor": phases[0], "root": phases[1], "refinement": phases[2]},
        "refinement": {"max_iterations": max_iters, "fp64_recomputed_solves": fallbacks, "gmres_steps": steps_job,
                       "batch_steps": steps_batch},
        "gradient": {"grad_ms": ms_grad, "grad_fwd_ratio": ms_grad / (ms / args.steps),
                     "max_abs_dT_fwd_vs_grad": float(np.abs(t_g - t_mixed).max()),
                     "status_ok": bool((st_g == 0).all()), "sites": int(sys_.system.n)},
        "status_ok": bool((st_mixed == 0).all() and (st_dbl == 0).all()),
        "gpu_launches": int(launches), "schedule": schedule, "roofline": roof, "roofline_fp64": roof64,
        "kernels_ms_per_step": kernels, "clocks": clk.summary(), "wall_s_timed": wall, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def roofline_probe(ctx, step, step_ms, traffic_of):
    """Per-kernel-class device time of one untimed step (each class probed launch by launch on its
    own pass); the dominant class against its roof."""
    names = ctx.kernel_classes()
    probe = {}
    for k, name in enumerate(names):
        for q in range(len(names)):
            ctx.kernel_stats(q, reset=True)
        ctx.probe(k)
        step()
        ctx.probe(-1)
        stt = ctx.kernel_stats(k)
        probe[name] = {"ms": stt["ms"], "flops": stt["flops"], "bytes": stt["bytes"], "launches": stt["launches"]}
    dom = max(probe.items(), key=lambda kv: kv[1]["ms"])
    pk = peaks()
    d = dom[1]
    traffic = traffic_of(dom[0])
    if dom[0] in FLOP_CLASSES:
        achieved = d["flops"] / (d["ms"] * 1e-3) / 1e12
        roof = {"kernel": dom[0], "bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": traffic, "note": f"peak = {pk['source']} bf16 dense"}
    else:
        achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9
        roof = {"kernel": dom[0], "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": traffic, "note": f"peak = {pk['source']} HBM copy"}
    roof["per"] = "step (all launches of the class in one step)"
    roof["algorithmic"] = d["bytes"] if roof["bound"] == "hbm" else d["flops"]
    roof["ms_per_step"] = d["ms"]
    roof["launches_per_step"] = d["launches"]
    roof["share_of_step"] = d["ms"] / step_ms
    kernels = {k: {"ms": round(v["ms"], 3), "launches": v["launches"]} for k, v in probe.items() if v["launches"]}
    return roof, kernels


def cpu_baseline(sys_, pairs, sample, threads):
    """The oracle (C++ restatement of the reference's CPU path) on `sample` instances."""
    from oracle import Oracle

    orc = Oracle(sys_.system)
    sub = pairs[:sample]
    nb = sys_.block_count()
    blocks, energies, vals, sls, srs = [], [], [], [], []
    for s, c in sub:
        for b in range(nb):
            blocks.append(b)
            energies.append(s.energy)
            vals.append(sys_.system.values[c])
            sls.append(s.blocks[b][0])
            srs.append(s.blocks[b][1])
    t0 = time.perf_counter()
    t, st = orc.solve_batch(blocks, energies, vals, sls, srs, precision=0, threads=threads)
    dt = time.perf_counter() - t0
    tsum = t.reshape(len(sub), nb).sum(axis=1)
    return len(sub) / dt, dt, tsum


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return world, rank, local, dist, torch
    return world, rank, local, None, None


def barrier(dist, torch):
    if dist is not None:
        dist.barrier()


def reduce_max(x, dist, torch):
    if dist is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    from caroli_gb300 import Precision
    from caroli_gb300.nested import context

    world, rank, local, dist, torch = dist_setup(args)
    sys_, sigmas, pairs = build_workload(args.length, args.width, args.configs, args.energies)
    sys_.device = local
    plan = sys_.plan()
    ctx = context(local)
    S = [p[0] for p in pairs]
    C = [p[1] for p in pairs]
    nsolve = len(pairs)
    for _ in range(args.warmup):
        sys_.solve_batch(S, C, Precision.MIXED)
    if args.profile_run:
        # One step of the mixed path and nothing else (for a profiler's launch list).
        sys_.solve_batch(S, C, Precision.MIXED)
        print(json.dumps({"profile_run": True, "solves": nsolve, "launches": plan.last_timing()[1]}))
        return
    # Timed region: K steps of the mixed path, inputs resident.
    barrier(dist, torch)
    with Clocks(local) as clk:
        ctx.region_begin()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            t_mixed, st_mixed, err_mixed = sys_.solve_batch(S, C, Precision.MIXED)
        ms, launches = ctx.region_end()
        wall = time.perf_counter() - w0
    barrier(dist, torch)
    ms_max = reduce_max(ms, dist, torch)
    schedule = ctx.last_schedule()  # the autotuner's choice for this batch, graph replays so far
    fallbacks, max_iters = plan.last_stats()
    iters, perturbed, jstat = plan.last_job_info()
    # Plain FP64 GPU path on the same batch (one step after one warm-up).
    sys_.solve_batch(S, C, Precision.DOUBLE)
    ctx.region_begin()
    t_dbl, st_dbl, _ = sys_.solve_batch(S, C, Precision.DOUBLE)
    ms_dbl, _ = ctx.region_end()
    dT = np.abs(t_mixed - t_dbl)
    # End to end through the public API from host buffers: the step's inputs (H values of every
    # configuration, Σ_L, Σ_R and W_R of every energy) sit in pinned host memory, column-major as
    # the C ABI reads them, and are copied to the device inside the timed region every step.
    import torch as _torch

    def pinned(a, order="C"):
        a = np.asarray(a)
        buf = _torch.empty(a.size, dtype=_torch.complex128, pin_memory=True).numpy()
        out = buf.reshape(a.shape, order=order)
        out[...] = a
        return out

    values = pinned(np.stack(sys_.system.values))
    host_sigma = [([(pinned(a, "F"), pinned(b, "F")) for a, b in s.blocks], [pinned(w, "F") for w in s.w_right()])
                  for s in sigmas]
    h2d = values.nbytes + sum(sum(a.nbytes + b.nbytes for a, b in bl) + sum(w.nbytes for w in ws)
                              for bl, ws in host_sigma)
    h2d += 2 * 4 * nsolve
    d2h = nsolve * (8 + 4 + 8)
    def e2e_step():
        plan.upload_values(values)
        for s, (bl, ws) in zip(sigmas, host_sigma):
            plan.upload_sigma(sys_._slot_of[id(s)][0], s.energy, bl, ws)
        sys_.solve_batch(S, C, Precision.MIXED)

    for _ in range(max(1, args.warmup)):  # untimed: the FP64 comparison above replaced the cached task lists
        e2e_step()
    ctx.region_begin()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_ms, _ = ctx.region_end()
    e2e_wall = time.perf_counter() - e0
    gen = time_generation(sys_, ctx) if rank == 0 else None
    # Per-kernel probe (untimed pass per class): the dominant kernel and its roofline.
    names = ctx.kernel_classes()
    probe = {}
    for k, name in enumerate(names):
        for q in range(len(names)):
            ctx.kernel_stats(q, reset=True)
        ctx.probe(k)
        sys_.solve_batch(S, C, Precision.MIXED)
        ctx.probe(-1)
        stt = ctx.kernel_stats(k)
        probe[name] = {"ms": stt["ms"], "flops": stt["flops"], "bytes": stt["bytes"], "launches": stt["launches"]}
    dom = max(probe.items(), key=lambda kv: kv[1]["ms"])
    pk = peaks()
    d = dom[1]
    traffic = profiled_traffic(dom[0])
    if dom[0] in FLOP_CLASSES:
        achieved = d["flops"] / (d["ms"] * 1e-3) / 1e12
        roof = {"kernel": dom[0], "bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": traffic,
                "note": f"peak = {pk['source']} bf16 dense"}
    else:
        achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9
        roof = {"kernel": dom[0], "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": traffic, "note": f"peak = {pk['source']} HBM copy"}
    roof["per"] = "step (all launches of the class in one step); traffic from the committed ncu launch list"
    roof["algorithmic"] = d["bytes"] if roof["bound"] == "hbm" else d["flops"]
    roof["ms_per_step"] = d["ms"]
    roof["launches_per_step"] = d["launches"]
    roof["share_of_step"] = d["ms"] / (ms_max / args.steps)
    kernels = {k: {"ms": round(v["ms"], 3), "launches": v["launches"]} for k, v in probe.items() if v["launches"]}
    grad = None
    if rank == 0 and args.gradient:
        grad = time_gradient(args.steps)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_sample > 0:
        threads = os.cpu_count() or 1
        rate, dt, tcpu = cpu_baseline(sys_, pairs, args.cpu_sample, threads)
        cpu = {"value": rate, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} of the step's {nsolve} solves (both blocks each), {dt:.1f} s wall",
               "max_abs_dT_vs_gpu_fp64": float(np.abs(tcpu - t_dbl[:args.cpu_sample]).max())}
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    value = world * nsolve * args.steps / (ms_max * 1e-3)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64 factors + f64 refinement",
        "data": "synthetic (seeded disorder of the reference's CLI conventions; no dataset)",
        "config": {"workload": WORKLOAD, "solves_per_step": nsolve, "blocks": sys_.block_count(),
                   "unknowns": sys_.system.n, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (arena ~33 GB per step)"},
        "fp64_gpu": {"value": nsolve / (ms_dbl * 1e-3), "unit": "solves/s", "ms_per_step": ms_dbl},
        "mixed_over_fp64": ms_dbl / (ms_max / args.steps),
        "max_abs_dT_vs_fp64": float(dT.max()),
        "median_abs_dT_vs_fp64": float(np.median(dT)),
        "refinement": {"max_iterations": max_iters, "fp64_recomputed_solves": fallbacks,
                       "median_iterations": float(np.median(iters)) if len(iters) else None,
                       "perturbed_pivots_total": int(perturbed.sum()) if len(perturbed) else 0},
        "grad_fwd_ratio": grad["value"] if grad else None,
        "gradient": grad,
        "e2e": {"value": nsolve * args.steps / (e2e_ms * 1e-3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "wall_s": e2e_wall},
        "gpu_launches": int(launches),
        "schedule": schedule,
        "inputs_on_device": gen,
        "roofline": roof,
        "kernels_ms_per_step": kernels,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import Oracle

    sys_, sigmas, pairs = build_workload(args.length, args.width, args.configs, args.energies)
    threads = os.cpu_count() or 1
    sample = args.ref_sample
    for _ in range(args.warmup):
        cpu_baseline(sys_, pairs, max(1, sample // 4), threads)
    times = []
    for k in range(args.steps):
        rate, dt, _ = cpu_baseline(sys_, pairs, sample, threads)
        times.append(dt)
    total = sum(times)
    value = sample * args.steps / total
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "impl": "reference",
        "data": "synthetic (same workload as the GPU arm)",
        "config": {"workload": WORKLOAD, "solves_per_step": sample, "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the workload's {len(pairs)} solves per step, FP64, OpenMP over solves"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--length", type=int, default=200)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--configs", type=int, default=8)
    ap.add_argument("--energies", type=int, default=33)
    ap.add_argument("--cpu-sample", type=int, default=264)
    ap.add_argument("--ref-sample", type=int, default=264)
    ap.add_argument("--profile-run", action="store_true", help="warm-up steps and one step, no timing (profilers)")
    ap.add_argument("--no-gradient", dest="gradient", action="store_false", help="skip the grad/fwd measurement")
    ap.add_argument("--workload", default="bhz", choices=["bhz", "ribbons", "cubic"],
                    help="bhz: the headline BHZ 200x64 magnetic batch; ribbons: 256 graphene ribbons x 64 E; "
                         "cubic: a sample of the 64x32x32 Anderson wire")
    ap.add_argument("--ribbons", type=int, default=256)
    ap.add_argument("--cubic-energies", default="8,16,23", help="indices into the cubic workload's 32 energies")
    ap.add_argument("--cubic-shape", default="64,32,32", help="length, width, depth of the cubic wire (a smaller "
                    "one for profiler captures)")
    ap.add_argument("--mixed-max-channels", type=int, default=100000)
    ap.add_argument("--refine-max-iters", type=int, default=6, help="outer refinement steps (caroli_set_refine_options)")
    ap.add_argument("--no-probe", dest="probe", action="store_false", help="skip the per-kernel-class probe passes")
    args = ap.parse_args()
    if args.workload == "cubic":
        if args.configs == 8:
            args.configs = 2
        if args.cpu_sample == 264:
            args.cpu_sample = 2
        run_cubic(args)
    elif args.workload == "ribbons":
        if args.energies == 33:
            args.energies = 64
        if args.cpu_sample == 264:
            args.cpu_sample = 16
        run_ribbons(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
