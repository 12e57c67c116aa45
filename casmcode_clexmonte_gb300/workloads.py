"""Seeded synthetic cluster expansions and Monte Carlo workloads.

The reference benchmarks nothing and ships no public dataset for this path;
these seeded systems stand in for real CASM projects with the shapes, sizes
and value distributions of the five benchmark configurations:

0. FCC A/B (a = 4.0 A), 10x10x10 primitive cells (1000 sites), semi-grand
   canonical, T = 1000 K, dmu = 0, random initial occupation.
1. same CE, canonical, 24^3 = 13824 sites, 128 replicas on a grid of 64
   temperatures in [200, 1200] K x x_B in {0.25, 0.5}.
2. BCC A/B/C (a = 3.2 A, two-site cubic cell), 256 replicas of L^3 cells,
   L in [8, 32] drawn by seed (1024..65536 sites), semi-grand canonical,
   mu_B, mu_C ~ U[-0.3, 0.3] eV, T ~ U[300, 1500] K.
3. FCC A/B with NN1 = 0.08 eV (L1_2 ordering), canonical x_B = 0.25,
   48^3 = 110592 sites, 32 replicas.
4. config 0's CE, 512 replicas of 32^3 plus 4 replicas of 96^3.

FCC cluster expansion (7 functions): empty, point, pairs to the third
neighbour shell, triplets with all edges up to the second shell. ECIs: point
U(-0.1, 0.1), NN1 0.05, NN2 -0.02, NN3 N(0, 0.005), triplets N(0, 0.003) eV.
BCC cluster expansion: pairs to the fourth shell, triplets and quadruplets
with all edges up to the second shell (the BCC first-neighbour graph is
bipartite, so no cluster with only first-neighbour edges exists beyond
pairs), ECIs N(0, 0.01) eV; this gives 27 functions.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .system import ClusterExpansion, bcc_conventional, fcc_prim

FCC_A = 4.0
BCC_A = 3.2


def _shell_cut(a: float, lattice: str, shell: int) -> float:
    """Distance between the n-th and (n+1)-th neighbour shells (Angstrom)."""
    if lattice == "fcc":
        d2 = [0.5, 1.0, 1.5, 2.0, 2.5]  # (r/a)^2 for shells 1..5
    else:
        d2 = [0.75, 1.0, 2.0, 2.75, 3.0]
    return a * 0.5 * (math.sqrt(d2[shell - 1]) + math.sqrt(d2[shell]))


def fcc_binary_ce(seed: int = 0, nn1: float = 0.05) -> ClusterExpansion:
    ce = ClusterExpansion(
        fcc_prim(FCC_A, ("A", "B")),
        {2: _shell_cut(FCC_A, "fcc", 3), 3: _shell_cut(FCC_A, "fcc", 2)},
    )
    assert ce.n_funcs == 7, ce.describe()
    rng = np.random.default_rng(seed)
    eci = np.zeros(7)
    eci[1] = rng.uniform(-0.1, 0.1)
    eci[2] = nn1
    eci[3] = -0.02
    eci[4] = rng.normal(0.0, 0.005)
    eci[5] = rng.normal(0.0, 0.003)
    eci[6] = rng.normal(0.0, 0.003)
    ce.eci = eci
    return ce


def bcc_ternary_ce(seed: int = 2) -> ClusterExpansion:
    cut2 = _shell_cut(BCC_A, "bcc", 2)
    ce = ClusterExpansion(
        bcc_conventional(BCC_A, ("A", "B", "C")),
        {2: _shell_cut(BCC_A, "bcc", 4), 3: cut2, 4: cut2},
    )
    rng = np.random.default_rng(seed)
    eci = rng.normal(0.0, 0.01, ce.n_funcs)
    eci[0] = 0.0
    ce.eci = eci
    return ce


def random_occupation(rng, n_sites: int, n_occ: int) -> np.ndarray:
    return rng.integers(0, n_occ, n_sites).astype(np.int8)


def fixed_composition(rng, n_sites: int, x_b: float) -> np.ndarray:
    """Binary occupation with exactly round(x_b * n_sites) B atoms."""
    occ = np.zeros(n_sites, dtype=np.int8)
    nb = int(round(x_b * n_sites))
    occ[rng.permutation(n_sites)[:nb]] = 1
    return occ


@dataclass
class Workload:
    name: str
    ce: ClusterExpansion
    ensemble: str  # "canonical" | "semigrand_canonical"
    L: list  # per replica (Lx, Ly, Lz)
    temperature: np.ndarray
    param_chem_pot: np.ndarray  # [n_rep, n_occ-1]
    x_b: np.ndarray | None
    occupation: list  # per replica int8 arrays
    seeds: np.ndarray
    n_passes: int
    n_equil: int
    notes: dict = field(default_factory=dict)

    @property
    def n_replicas(self) -> int:
        return len(self.L)

    @property
    def n_sites(self) -> np.ndarray:
        nb = self.ce.prim.n_basis
        return np.array([nb * l[0] * l[1] * l[2] for l in self.L])


def config(index: int, seed: int = 20251203, scale: float = 1.0) -> Workload:
    """The benchmark configurations; ``scale`` < 1 shrinks replica counts and
    pass counts (never supercells) for quick tests."""
    rng = np.random.default_rng(seed + index)
    if index == 0:
        ce = fcc_binary_ce(seed)
        L = [(10, 10, 10)]
        occ = [random_occupation(rng, 1000, 2)]
        return Workload("fcc_binary_10I_sgc", ce, "semigrand_canonical", L,
                        np.array([1000.0]), np.zeros((1, 1)), None, occ,
                        np.array([seed]), max(1, int(1000 * scale)), max(1, int(200 * scale)))
    if index == 1:
        ce = fcc_binary_ce(seed)
        n = max(2, int(128 * scale))
        temps = np.repeat(np.linspace(200.0, 1200.0, n // 2), 2)
        xb = np.tile([0.25, 0.5], n // 2)
        L = [(24, 24, 24)] * n
        occ = [fixed_composition(rng, 24**3, x) for x in xb]
        return Workload("fcc_binary_24I_canonical_x128", ce, "canonical", L, temps,
                        np.zeros((n, 1)), xb, occ, seed * 1000 + np.arange(n),
                        max(1, int(5000 * scale)), max(1, int(1000 * scale)))
    if index == 2:
        ce = bcc_ternary_ce(seed)
        n = max(2, int(256 * scale))
        Ls = rng.integers(8, 33, n)
        L = [(int(l), int(l), int(l)) for l in Ls]
        temps = rng.uniform(300.0, 1500.0, n)
        mu = rng.uniform(-0.3, 0.3, (n, 2))
        occ = [random_occupation(rng, 2 * int(l) ** 3, 3) for l in Ls]
        return Workload("bcc_ternary_8I-32I_sgc_x256", ce, "semigrand_canonical", L, temps, mu,
                        None, occ, seed * 1000 + np.arange(n),
                        max(1, int(2000 * scale)), max(1, int(400 * scale)))
    if index == 3:
        ce = fcc_binary_ce(seed, nn1=0.08)
        n = max(1, int(32 * scale))
        L = [(48, 48, 48)] * n
        occ = [fixed_composition(rng, 48**3, 0.25) for _ in range(n)]
        return Workload("fcc_binary_L12_48I_canonical_x32", ce, "canonical", L,
                        np.full(n, 0.9 * 1000.0), np.zeros((n, 1)), np.full(n, 0.25), occ,
                        seed * 1000 + np.arange(n),
                        max(1, int(2000 * scale)), max(1, int(500 * scale)),
                        notes={"T_c": "estimate 1000 K until a temperature scan replaces it"})
    if index == 4:
        ce = fcc_binary_ce(seed)
        n32 = max(1, int(512 * scale))
        n96 = max(1, int(4 * scale))
        L = [(32, 32, 32)] * n32 + [(96, 96, 96)] * n96
        n = n32 + n96
        temps = np.concatenate([np.tile(np.linspace(300.0, 1500.0, 16), n32 // 16 + 1)[:n32],
                                np.full(n96, 800.0)])
        xb = np.concatenate([np.repeat(np.linspace(0.1, 0.5, 32), n32 // 32 + 1)[:n32],
                             np.full(n96, 0.25)])
        occ = [fixed_composition(rng, l[0] * l[1] * l[2], x) for l, x in zip(L, xb)]
        return Workload("fcc_binary_32I_x512_96I_x4_canonical", ce, "canonical", L, temps,
                        np.zeros((n, 1)), xb, occ, seed * 1000 + np.arange(n),
                        max(1, int(20000 * scale)), max(1, int(2000 * scale)))
    raise ValueError(f"unknown config {index}")
