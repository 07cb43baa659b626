"""Test systems: the reference's benchmark problems (benchmarks/transport.toml with the disorder of
caroli-bench/src/main.rs:118-126) and the workloads of the GB300 path."""
from __future__ import annotations

import json
import os

import numpy as np

from caroli_gb300 import NestedTwoTerminal, Region, bhz, cubic, graphene, square
from caroli_gb300.disorder import Moments, ScalarPotential, bench_disorder, disordered
from caroli_gb300.model import bhz_spin

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CLEAN = {"square": square, "bhz": bhz, "graphene": graphene}
PROBLEMS = {"square-clean": ("square", None, None), "square-anderson": ("square", 1, 2.0),
            "bhz-anderson": ("bhz", 2, 0.5), "graphene-anderson": ("graphene", 4, 1.0)}


def bench_golden():
    with open(os.path.join(GOLDEN, "bench_transmissions.json")) as f:
        return json.load(f)["results"]


def bench_problem(name, width, length=None):
    """The device and lead models and region of a benchmark problem (L = W by default)."""
    model_name, seed, w = PROBLEMS[name]
    clean = CLEAN[model_name]()
    length = length or width
    region = Region.cuboid(clean.lattice, [length, width, 0])
    if seed is None:
        return clean, clean, region
    subs = len(clean.lattice.sublattices)
    orb = clean.lattice.sublattices[0].orbitals
    pot = bench_disorder(seed, width, length, width, subs, w)
    return clean.with_onsite_term(ScalarPotential(pot, width, subs, orb)), clean, region


def bench_system(name, width):
    dev, lead, region = bench_problem(name, width)
    return NestedTwoTerminal.from_model(dev, lead, region, 0)


def clean_bhz_ribbon(length=16, width=10):
    """Config: clean BHZ ribbon with leads of the same model (ti_conductance.rs:20-24)."""
    m = bhz()
    return NestedTwoTerminal.from_model(m, m, Region.cuboid(m.lattice, [length, width, 0]), 0)


def magnetic_bhz(length, width, configs, concentration=0.2, exchange=0.4, moments=None, spin="opposite-g",
                 anderson=None):
    """BHZ ribbon with CLI-style [[disorder]] entries (caroli-cli/src/build.rs:251-310), one system
    per configuration: magnetic impurities at a concentration over all sites, and optionally an
    Anderson entry first."""
    m = bhz()
    region = Region.cuboid(m.lattice, [length, width, 0])
    entries = []
    if anderson is not None:
        entries.append({"kind": "anderson", "strength": anderson})
    entries.append({"kind": "magnetic", "concentration": concentration, "exchange": exchange,
                    "moments": moments or Moments.polarized(1.0), "spin": bhz_spin(spin)})
    devices = [disordered(m, region, entries, c) for c in range(configs)]
    return NestedTwoTerminal.from_models(devices, m, region, 0)


def cubic_wire(length, width, depth, w=16.5, configs=1, seed=1):
    """Cubic Anderson wire, leads of the clean cubic model along x."""
    m = cubic()
    region = Region.cuboid(m.lattice, [length, width, depth])
    devices = []
    for c in range(configs):
        entries = [{"kind": "anderson", "strength": w, "seed": seed}]
        devices.append(disordered(m, region, entries, c))
    return NestedTwoTerminal.from_models(devices, m, region, 0)


def oracle_T(sys_, sigma, config=0, precision=0):
    from oracle import Oracle

    if not hasattr(sys_, "_oracle"):
        sys_._oracle = Oracle(sys_.system)
    return sys_._oracle.transmission(sigma.energy, sys_.system.values[config], sigma.blocks, precision)


def gradient_bhz(length, width, configs=1, anderson=0.02, concentration=0.1, exchange=0.3, moments=None,
                 spin="opposite-g"):
    """The gradient workload's physics on a ribbon: Anderson disorder W (entry 0) and magnetic
    impurities (entry 1, isotropic moments by default, as the CLI), with dH/dJ per configuration:
    the exchange term at J = 1 (H is linear in J)."""
    from caroli_gb300.system import merge_patterns

    m = bhz()
    region = Region.cuboid(m.lattice, [length, width, 0])
    mom = moments or Moments.isotropic()

    def entries(j):
        return [{"kind": "anderson", "strength": anderson},
                {"kind": "magnetic", "concentration": concentration, "exchange": j, "moments": mom,
                 "spin": bhz_spin(spin)}]

    devices = [disordered(m, region, entries(exchange), c) for c in range(configs)]
    sys_ = NestedTwoTerminal.from_models(devices, m, region, 0)
    derivs = []
    for c in range(configs):
        h1 = disordered(m, region, entries(1.0), c).sparse_hamiltonian(region)
        h0 = disordered(m, region, entries(0.0), c).sparse_hamiltonian(region)
        # Both on the system's merged pattern.
        from caroli_gb300.model import SparseMatrix
        base = SparseMatrix(sys_.system.n, sys_.system.row_ptr, sys_.system.cols, np.zeros(sys_.system.nnz, complex))
        _, _, (v1, v0, _) = merge_patterns([h1, h0, base])
        derivs.append([v1 - v0])
    return sys_, derivs


def graphene_ribbons(count, seed=1, widths=(8, 24), lengths=(12, 40), w=1.0, pick=None):
    """Graphene zigzag ribbons of uneven sizes, as the many-ribbon workload draws them (widths and
    lengths from xoshiro seed_from_u64(seed), Anderson w(u - 0.5) per site from
    seed_from_u64(1 000 003 seed + ribbon), the benchmark's convention of caroli-bench/src/main.rs:124).
    Returns the NestedTwoTerminal of each ribbon, or of the ribbons `pick` of the `count` drawn."""
    from caroli_gb300.disorder import Xoshiro256

    rng = Xoshiro256.seed_from_u64(seed)
    shapes = [(rng.integer(*widths), rng.integer(*lengths)) for _ in range(count)]
    out = []
    for r in (range(count) if pick is None else pick):
        width, length = shapes[r]
        clean = graphene()
        region = Region.cuboid(clean.lattice, [length, width, 0])
        subs = len(clean.lattice.sublattices)
        pot = bench_disorder(seed, r, length, width, subs, w)
        device = clean.with_onsite_term(ScalarPotential(pot, width, subs, 1))
        out.append(NestedTwoTerminal.from_model(device, clean, region, 0))
    return out


def cross_geometry(lattice, w):
    """A w x w square with arms of length w / 4 on its four edges and the interfaces of their
    leads (left, right, bottom, top): the benchmark's "cross" (caroli-bench/src/main.rs:128-153)."""
    from caroli_gb300 import Interface, Region
    from caroli_gb300.lattice import Site

    arm = w // 4
    subs = len(lattice.sublattices)

    def sites(cells):
        return [Site((x, y, 0), s) for (x, y) in cells for s in range(subs)]

    cells = [(x, y) for x in range(-arm, w + arm) for y in range(-arm, w + arm) if 0 <= x < w or 0 <= y < w]
    column = lambda x: Region.from_sites(lattice, sites([(x, y) for y in range(w)]))
    row = lambda y: Region.from_sites(lattice, sites([(x, y) for x in range(w)]))
    interfaces = [Interface(column(-arm), (-1, 0, 0)), Interface(column(w + arm - 1), (1, 0, 0)),
                  Interface(row(-arm), (0, -1, 0)), Interface(row(w + arm - 1), (0, 1, 0))]
    return Region.from_sites(lattice, sites(cells)), interfaces


def cross_problem(width, model="square", seed=5, anderson=1.0):
    """The square-cross benchmark problem (benchmarks/transport.toml:54-62): Anderson disorder
    w (u - 0.5) per site of the bounding box from xoshiro seed_from_u64(seed * 1 000 003 + W),
    index (x ny + y) subs + sub from the box's corner (caroli-bench/src/main.rs:108-125)."""
    from caroli_gb300 import NestedMultiTerminal

    clean = CLEAN[model]() if model in CLEAN else model
    region, interfaces = cross_geometry(clean.lattice, width)
    arm = width // 4
    nx = ny = width + 2 * arm
    subs = len(clean.lattice.sublattices)
    orb = clean.lattice.sublattices[0].orbitals
    pot = bench_disorder(seed, width, nx, ny, subs, anderson)
    dev = clean.with_onsite_term(ScalarPotential(pot, ny, subs, orb, origin=(-arm, -arm)))
    return dev, clean, region, interfaces


def cross_system(width, model="square", seed=5, anderson=1.0):
    from caroli_gb300 import NestedMultiTerminal

    dev, clean, region, interfaces = cross_problem(width, model, seed, anderson)
    return NestedMultiTerminal.from_model(dev, clean, region, interfaces)


def thesis_ribbon(case, coupling_j):
    """The thesis' conductance-2t setup (caroli-validation/tests/ti_conductance_disorder.rs:24-40,
    src/thesis.rs:53-82): BHZ 16 x 10 with one clean lead slice at each end, 24 magnetic
    impurities drawn from gfortran seed 12345 in the central 8 x 10 region (x fastest), moments
    along z (cone of zero angle) or isotropic, exchange J (n . S) with the case's spin coupling."""
    from caroli_gb300.disorder import MagneticImpurities, Moments, Xoshiro256
    from caroli_gb300.lattice import Site

    nx, ny, nx_imp = 16, 10, 8
    spin, coupling = {"ti-cond2t-same-g": (1, "same-g"), "ti-cond2t-isotropic": (0, "same-g"),
                      "ti-cond2t-opposite-g": (1, "opposite-g")}[case]
    x0 = 1 + (nx - nx_imp) // 2
    region_imp = [Site((x0 + x, y, 0), 0) for y in range(ny) for x in range(nx_imp)]
    n_imp = int(0.3 * nx_imp * ny)
    moments = Moments.isotropic() if spin == 0 else Moments.cone(0.0)
    imp = MagneticImpurities.generate(Xoshiro256.gfortran(12345), region_imp, n_imp, moments)
    clean = bhz()
    dev = bhz().with_onsite_term(imp.exchange(coupling_j, bhz_spin(coupling)))
    return NestedTwoTerminal.from_model(dev, clean, Region.cuboid(clean.lattice, [nx + 2, ny, 0]), 0)
