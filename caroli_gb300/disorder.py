"""Reproducible disorder: xoshiro256**, Anderson disorder and classical magnetic impurities.

Bit-compatible with ``crates/caroli-disorder`` of caroli:

- ``Xoshiro256`` (``rng.rs:9-81``): ``seed_from_u64`` fills the state with splitmix64
  (``rng.rs:19-33``), ``gfortran``/``gfortran_put`` rebuild gfortran >= 9 seeding (``rng.rs:35-49``),
  ``uniform`` takes the top 53 bits (``rng.rs:65-69``), ``integer`` is ``lo + floor((hi-lo+1) u)``.
- ``choose_sites`` is the partial Fisher-Yates draw of the thesis codes (``lib.rs:14-26``);
  ``Moments.draw`` draws all ``n_z`` first, then all azimuths (``lib.rs:53-64``).
- ``Anderson.generate`` draws ``w (u - 1/2)`` per site in order (``lib.rs:110-115``).
- ``disordered`` follows the CLI's ``[[disorder]]`` convention (``caroli-cli/src/build.rs:251-310``):
  entry ``k`` of configuration ``c`` is seeded with ``1 + 1000 k + c``.
- ``bench_disorder`` follows ``caroli-bench/src/main.rs:118-126``: one value per site of the
  bounding box, index ``(x ny + y) subs + sub``, seed ``seed * 1000003 + width``.
"""
from __future__ import annotations

import math

import numpy as np

from .lattice import Region, Site
from .model import Model, OnSiteMap, combine

M64 = (1 << 64) - 1
GFORTRAN_KEYS = (0xBD0C5B6E50C2DF49, 0xD46061CD46E1DF38, 0xBB4F4D4ED6103544, 0x114A583D0756AD39)


def _rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & M64


def splitmix64(state):
    """One splitmix64 step: returns ``(new_state, output)``."""
    state = (state + 0x9E3779B97F4A7C15) & M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return state, z ^ (z >> 31)


class Xoshiro256:
    """xoshiro256** (Blackman & Vigna 2018)."""

    def __init__(self, s):
        self.s = [int(x) & M64 for x in s]

    @staticmethod
    def seed_from_u64(seed):
        sm = int(seed) & M64
        out = []
        for _ in range(4):
            sm, v = splitmix64(sm)
            out.append(v)
        return Xoshiro256(out)

    @staticmethod
    def gfortran_put(put):
        w = [int(x) & 0xFFFFFFFF for x in put]
        raw = [w[7] | w[6] << 32, w[5] | w[4] << 32, w[3] | w[2] << 32, w[1] | w[0] << 32]
        return Xoshiro256([raw[i] ^ GFORTRAN_KEYS[i] for i in range(4)])

    @staticmethod
    def gfortran(seed):
        return Xoshiro256.gfortran_put([seed] * 8)

    def next_u64(self):
        s = self.s
        result = (_rotl((s[1] * 5) & M64, 7) * 9) & M64
        t = (s[1] << 17) & M64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = _rotl(s[3], 45)
        return result

    def uniform(self):
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def uniforms(self, n):
        return np.array([self.uniform() for _ in range(n)], dtype=np.float64)

    def integer(self, lo, hi):
        return lo + int((hi - lo + 1) * self.uniform())


def choose_sites(rng: Xoshiro256, candidates, n):
    if n > len(candidates):
        raise ValueError(f"{n} impurities for {len(candidates)} sites")
    tab = list(range(len(candidates)))
    for i in range(n):
        r = rng.integer(i + 1, len(candidates)) - 1
        tab[i], tab[r] = tab[r], tab[i]
    return [candidates[k] for k in tab[:n]]


class Moments:
    """Axisymmetric unit-moment distributions (``lib.rs:28-65``)."""

    def __init__(self, kind="isotropic", theta0=0.0, mz=1.0):
        self.kind, self.theta0, self.mz = kind, theta0, mz

    @staticmethod
    def isotropic():
        return Moments("isotropic")

    @staticmethod
    def polarized(mz):
        if not 0.0 <= mz <= 1.0:
            raise ValueError(f"polarisation mz = {mz} outside [0, 1]")
        return Moments("polarized", mz=mz)

    @staticmethod
    def cone(theta0):
        return Moments("cone", theta0=theta0)

    def nz(self, u):
        if self.kind == "isotropic":
            return 2.0 * u - 1.0
        if self.kind == "cone":
            return -(1.0 - math.cos(self.theta0)) * u + 1.0
        return 2.0 * (1.0 - self.mz) * u + 2.0 * self.mz - 1.0

    def draw(self, rng, n):
        nz = [self.nz(u) for u in rng.uniforms(n)]
        phi = [2.0 * math.pi * u for u in rng.uniforms(n)]
        out = []
        for z, p in zip(nz, phi):
            perp = math.sqrt(1.0 - z * z)
            out.append((perp * math.cos(p), perp * math.sin(p), z))
        return out


class MagneticImpurities:
    def __init__(self, sites, moments):
        self.sites, self.moments = sites, moments

    @staticmethod
    def generate(rng, candidates, n, moments: Moments):
        sites = choose_sites(rng, candidates, n)
        return MagneticImpurities(sites, moments.draw(rng, n))

    def exchange(self, j, s):
        """``J (n_x S_x + n_y S_y + n_z S_z)`` on each impurity site (``lib.rs:88-100``)."""
        out = OnSiteMap()
        for site, n in zip(self.sites, self.moments):
            out.add(site, j * (s[0] * n[0] + s[1] * n[1] + s[2] * n[2]))
        return out


class Anderson:
    def __init__(self, sites, energies):
        self.sites, self.energies = sites, energies

    @staticmethod
    def generate(rng, sites, w):
        return Anderson(list(sites), [w * (u - 0.5) for u in rng.uniforms(len(sites))])

    def onsite(self, orbitals):
        out = OnSiteMap()
        for site, e in zip(self.sites, self.energies):
            out.add(site, e * np.eye(orbitals, dtype=np.complex128))
        return out


def disordered(model: Model, region: Region, entries, config: int) -> Model:
    """The model with the CLI-style ``[[disorder]]`` entries of configuration ``config``.

    Each entry is a dict with ``kind`` ("anderson": ``strength``; "magnetic": ``concentration``,
    ``exchange``, ``moments`` (a ``Moments``), ``spin`` (three matrices)) and optional ``seed``.
    """
    out = model
    for k, d in enumerate(entries):
        sites = list(region.sites)
        seed = d.get("seed", 1 + 1000 * k) + config
        rng = Xoshiro256.seed_from_u64(seed)
        if d["kind"] == "anderson":
            a = Anderson.generate(rng, sites, d["strength"])
            m = OnSiteMap()
            for s, e in zip(a.sites, a.energies):
                n = region.lattice.sublattices[s.sub].orbitals
                m.add(s, e * np.eye(n, dtype=np.complex128))
        elif d["kind"] == "magnetic":
            n_imp = int(d["concentration"] * len(sites))
            imp = MagneticImpurities.generate(rng, sites, n_imp, d.get("moments", Moments.isotropic()))
            spin = d["spin"]
            m = OnSiteMap()
            j = d["exchange"]
            for s, n in zip(imp.sites, imp.moments):
                m.add(s, combine([(j * n[0], spin[0]), (j * n[1], spin[1]), (j * n[2], spin[2])]))
        else:
            raise ValueError(f"unknown disorder {d['kind']}")
        out = out.with_onsite_term(m)
    return out


def bench_disorder(seed: int, width: int, nx: int, ny: int, subs: int, strength: float):
    """On-site values of the benchmark problems, one per site of the bounding box."""
    rng = Xoshiro256.seed_from_u64(seed * 1_000_003 + width)
    return strength * (rng.uniforms(nx * ny * subs) - 0.5)


class ScalarPotential:
    """On-site term ``v[(x ny + y) subs + sub] * 1`` on every site (``main.rs:229-233``)."""

    def __init__(self, values, ny, subs, orbitals, origin=(0, 0)):
        self.values, self.ny, self.subs, self.orbitals, self.origin = values, ny, subs, orbitals, origin

    def __call__(self, site: Site):
        x, y = site.cell[0] - self.origin[0], site.cell[1] - self.origin[1]
        return self.values[(x * self.ny + y) * self.subs + site.sub] * np.eye(self.orbitals, dtype=np.complex128)
