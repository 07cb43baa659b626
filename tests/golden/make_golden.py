"""Generates the golden fixtures of tests/golden from caroli's own published results.

Run in a checkout that has the caroli sources at REFERENCE (read-only input):
    python tests/golden/make_golden.py /path/to/caroli
It reads
- benchmarks/results/Mac-mini-de-Arnaud.jsonl: the nested-dissection (code "caroli") and RGF
  ("caroli-rgf") transmissions of the benchmark problems of benchmarks/transport.toml (for the
  four-terminal square-cross, the twelve T_pq with p != q of each energy, p-major);
- reference/baseline/golden/ti-cond2t-clean/{axes,cond}_00.dat: the thesis conductance of the
  clean BHZ 16 x 10 ribbon (Fortran unformatted records, int32-framed float64);
- crates/caroli-disorder/src/rng.rs: nothing (the RNG known answers are in the test itself).
- reference/baseline/golden/ti-cond2t-{same-g,isotropic,opposite-g}: the thesis conductance of the
  same ribbon with magnetic impurities;
and writes tests/golden/bench_transmissions.json, ti_cond2t_clean.json and ti_cond2t_disorder.json.
"""
import json
import os
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def records(path):
    b = open(path, "rb").read()
    i, out = 0, []
    while i < len(b):
        (n,) = struct.unpack("<i", b[i:i + 4])
        i += 4
        out.append(list(struct.unpack("<%dd" % (n // 8), b[i:i + n])))
        i += n + 4
    return out


def main(ref):
    rows = [json.loads(l) for l in open(os.path.join(ref, "benchmarks/results/Mac-mini-de-Arnaud.jsonl"))]
    bench = {}
    for r in rows:
        if r.get("mode", "single") != "single" or r.get("code") not in ("caroli", "caroli-rgf"):
            continue
        if r["problem"] not in ("bhz-anderson", "graphene-anderson", "square-anderson", "square-clean",
                                "square-cross"):
            continue
        if r["width"] not in (32, 64):
            continue
        key = f"{r['code']}/{r['problem']}/{r['width']}"
        bench.setdefault(key, {"energies": r["energies"], "runs": []})["runs"].append(r["transmissions"])
    with open(os.path.join(HERE, "bench_transmissions.json"), "w") as f:
        json.dump({"source": "benchmarks/results/Mac-mini-de-Arnaud.jsonl (caroli, commit 53d13c9 and later)",
                   "problems": {"square-clean": {"seed": None, "anderson": None},
                                "square-anderson": {"seed": 1, "anderson": 2.0},
                                "bhz-anderson": {"seed": 2, "anderson": 0.5},
                                "graphene-anderson": {"seed": 4, "anderson": 1.0},
                                "square-cross": {"seed": 5, "anderson": 1.0, "geometry": "cross",
                                                 "order": "T_pq for p != q, p-major"}},
                   "results": bench}, f, indent=1)
    g = os.path.join(ref, "reference/baseline/golden/ti-cond2t-clean")
    axes = records(os.path.join(g, "axes_00.dat"))[0]
    cond = records(os.path.join(g, "cond_00.dat"))[0]
    nu, ne = 3, 13
    with open(os.path.join(HERE, "ti_cond2t_clean.json"), "w") as f:
        json.dump({"source": "reference/baseline/golden/ti-cond2t-clean (thesis conductance-2t, BHZ 16x10)",
                   "energies": axes[nu:], "conductance": [cond[ie * nu] for ie in range(ne)]}, f, indent=1)
    # The magnetic-impurity cases: axes = 3 exchange couplings then 5 energies, cond(Nu, Ne)
    # column-major (caroli-validation/tests/ti_conductance_disorder.rs:16-22).
    cases = {}
    for case in ("ti-cond2t-same-g", "ti-cond2t-isotropic", "ti-cond2t-opposite-g"):
        g = os.path.join(ref, "reference/baseline/golden", case)
        axes = records(os.path.join(g, "axes_00.dat"))[0]
        cond = records(os.path.join(g, "cond_00.dat"))[0]
        cases[case] = {"couplings": axes[:3], "energies": axes[3:], "cond": cond}
    with open(os.path.join(HERE, "ti_cond2t_disorder.json"), "w") as f:
        json.dump({"source": "reference/baseline/golden/ti-cond2t-{same-g,isotropic,opposite-g} (thesis "
                             "conductance-2t: BHZ 16x10 + one lead slice at each end, 24 impurities, gfortran "
                             "seed 12345, Σ at E + 1e-5 i, Re Γ trace); cond[iu + 3 ie]",
                   "cases": cases}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the caroli source tree>")
    main(sys.argv[1])
