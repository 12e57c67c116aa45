"""Cluster expansions on a general crystal.

The cubic builder in ``system.py`` covers Bravais lattices whose sites sit on
an integer grid. This module covers every other CASM prim: any lattice, any
number of sublattices, each with its own allowed occupants, as in the
reference's ``Clex_ZrO_Occ`` fixture (hcp Zr with octahedral O/Va
interstitials, ``tests/unit/clexmonte/data/Clex_ZrO_Occ/prim.json``).

* Sites are integral coordinates (b, i, j, k): sublattice b of the unit cell
  at lattice translation (i, j, k), CASM's ``UnitCellCoord``.
* The factor group is found from the lattice and the basis: every integer
  matrix R (fractional coordinates) that keeps the metric, combined with the
  translations that map the basis onto itself with equal occupant lists. An
  operation maps (b, u) to (perm[b], R u + d[b]) with integer d[b].
* Clusters are built only from sublattices with more than one allowed
  occupant (the sites that carry the occupation degree of freedom, as CASM's
  cluster specs do), by the ``periodic_max_length`` rule: every pair of sites
  of a cluster of size n is at most ``max_length[n]`` apart.
* A cluster's canonical form is the smallest, over the factor group, of its
  sorted integral sites translated so that the first site lies in cell 0;
  orbits and decorated-function classes are keyed by it.

The kernel tables keep only the sublattices with a degree of freedom,
renumbered 0, 1, ... in increasing prim order; sublattices with one occupant
never change and enter the composition as constants.
"""

from __future__ import annotations

import itertools
import math
from dataclasses import dataclass

import numpy as np

from .system import ClusterExpansion, FlowerCluster, Orbit


@dataclass
class SiteOp:
    """A factor-group operation on integral site coordinates."""

    R: tuple  # 3x3 integer matrix on fractional coordinates (row tuples)
    perm: tuple  # sublattice b -> perm[b]
    d: tuple  # per sublattice: integer cell shift

    def apply(self, b: int, u) -> tuple:
        R, d = self.R, self.d[b]
        return (
            R[0][0] * u[0] + R[0][1] * u[1] + R[0][2] * u[2] + d[0],
            R[1][0] * u[0] + R[1][1] * u[1] + R[1][2] * u[2] + d[1],
            R[2][0] * u[0] + R[2][1] * u[1] + R[2][2] * u[2] + d[2],
            self.perm[b],
        )


class Crystal:
    """A CASM prim: lattice vectors (rows, Angstrom), fractional basis
    coordinates and the allowed occupants of each basis site."""

    def __init__(self, title: str, lattice, frac, occupants, tol: float = 1e-5):
        self.title = title
        self.lattice = np.asarray(lattice, dtype=np.float64).reshape(3, 3)
        self.frac = np.asarray(frac, dtype=np.float64).reshape(-1, 3)
        self.occupants = [tuple(o) for o in occupants]
        if len(self.occupants) != len(self.frac):
            raise ValueError("one occupant list per basis site")
        self.tol = tol
        self.dof = [b for b, o in enumerate(self.occupants) if len(o) > 1]
        if not self.dof:
            raise ValueError("no sublattice has more than one allowed occupant")
        occ0 = self.occupants[self.dof[0]]
        for b in self.dof:
            if self.occupants[b] != occ0:
                raise ValueError(
                    "sublattices with an occupation degree of freedom must share one occupant list"
                )
        self.ops = factor_group(self.lattice, self.frac, self.occupants, tol)

    @property
    def n_basis(self) -> int:
        return len(self.frac)

    def cart(self, b: int, u) -> np.ndarray:
        return (np.asarray(u, dtype=np.float64) + self.frac[b]) @ self.lattice

    def components(self) -> list:
        """Species in order of first appearance over the basis."""
        out = []
        for o in self.occupants:
            for s in o:
                if s not in out:
                    out.append(s)
        return out

    def fixed_counts(self) -> dict:
        """Species count per unit cell on the sublattices without a degree
        of freedom."""
        out = {}
        for b, o in enumerate(self.occupants):
            if len(o) == 1:
                out[o[0]] = out.get(o[0], 0) + 1
        return out


def factor_group(lattice, frac, occupants, tol: float = 1e-5) -> list:
    """Operations (R, t) with R in the lattice point group (integer matrices
    on fractional coordinates, entries in {-1, 0, 1}, R^T G R = G for the
    metric G) and a translation t that maps every basis site onto a basis
    site with the same occupant list (modulo lattice translations)."""
    A = np.asarray(lattice, dtype=np.float64)
    G = A @ A.T
    cand = np.array(list(itertools.product((-1, 0, 1), repeat=9)), dtype=np.int64).reshape(-1, 3, 3)
    det = np.rint(np.linalg.det(cand.astype(np.float64)))
    cand = cand[np.abs(det) == 1]
    # R acts on column vectors of fractional coordinates: f' = R f, so the
    # Cartesian length is kept iff R^T G R = G (G = A A^T, A rows = vectors)
    M = np.einsum("nji,jk,nkl->nil", cand, G, cand)
    scale = max(1.0, float(np.abs(G).max()))
    Rs = cand[np.all(np.abs(M - G) < tol * scale, axis=(1, 2))]
    frac = np.asarray(frac, dtype=np.float64)
    nb = len(frac)
    ops = []
    for R in Rs:
        rf = frac @ R.T
        for b1 in range(nb):
            if occupants[b1] != occupants[0]:
                continue
            t = frac[b1] - rf[0]
            perm, d = [], []
            for b in range(nb):
                x = rf[b] + t
                hit = None
                for b2 in range(nb):
                    if occupants[b2] != occupants[b]:
                        continue
                    diff = x - frac[b2]
                    if np.all(np.abs(diff - np.rint(diff)) < tol):
                        hit = b2
                        break
                if hit is None:
                    break
                perm.append(hit)
                d.append(tuple(int(v) for v in np.rint(x - frac[hit])))
            if len(perm) == nb:
                ops.append(SiteOp(tuple(tuple(int(v) for v in row) for row in R), tuple(perm), tuple(d)))
    return ops


def canonical(ops, sites, labels=None) -> tuple:
    """Canonical form of a (decorated) cluster of integral sites
    [(b, (i, j, k))]: the smallest, over the operations, of the sorted
    (i, j, k, b, label) list translated so that its first site is in cell 0."""
    labs = labels if labels is not None else (0,) * len(sites)
    best = None
    for op in ops:
        m = sorted(op.apply(b, u) + (lab,) for (b, u), lab in zip(sites, labs))
        i0, j0, k0 = m[0][0], m[0][1], m[0][2]
        key = tuple((x[0] - i0, x[1] - j0, x[2] - k0, x[3], x[4]) for x in m)
        if best is None or key < best:
            best = key
    return best


class SublatticeView:
    """The sublattices with an occupation degree of freedom, as the kernel
    tables and the samplers see them (renumbered 0, 1, ...)."""

    def __init__(self, crystal: Crystal):
        self.crystal = crystal
        self.title = crystal.title
        self.occupants = crystal.occupants[crystal.dof[0]]

    @property
    def n_basis(self) -> int:
        return len(self.crystal.dof)

    @property
    def n_occ(self) -> int:
        return len(self.occupants)


class CrystalClusterExpansion(ClusterExpansion):
    """Orbits, occupation-basis functions, flower and owned tables of a
    general crystal, with the attributes of the cubic ``ClusterExpansion``
    (the table builder, the C ABI and the samplers use either).

    ``orbit_order`` optionally gives the prototypes (lists of (b, (i, j, k))
    in prim sublattice numbering) of a reference basis set: the orbits then
    follow that order, and every prototype must match one built orbit."""

    def __init__(self, crystal: Crystal, max_length: dict, eci=None, tol: float = 1e-5,
                 orbit_order=None):
        self.crystal = crystal
        self.prim = SublatticeView(crystal)
        self.ops = crystal.ops
        self.max_length = {int(k): float(v) for k, v in max_length.items()}
        self.tol = tol
        self.n_sf = self.prim.n_occ - 1
        self._kb = {b: i for i, b in enumerate(crystal.dof)}
        self._build_orbits(orbit_order)
        self._build_functions()
        self._build_flowers()
        self.eci = np.zeros(self.n_funcs) if eci is None else np.asarray(eci, float)
        if self.eci.shape != (self.n_funcs,):
            raise ValueError(f"eci must have {self.n_funcs} entries")
        self.param_RT = None

    # ---- neighbourhood of a site with a degree of freedom
    def _neighbours(self, b: int, rmax: float):
        cr = self.crystal
        inv = np.linalg.inv(cr.lattice)
        n = [int(math.ceil(rmax * np.linalg.norm(inv[:, a]))) + 2 for a in range(3)]
        c0 = cr.cart(b, (0, 0, 0))
        out = []
        for u in itertools.product(*[range(-m, m + 1) for m in n]):
            for bb in cr.dof:
                d = float(np.linalg.norm(cr.cart(bb, u) - c0))
                if 0.0 < d <= rmax + self.tol:
                    out.append((bb, tuple(int(x) for x in u)))
        return out

    def _dist(self, s1, s2) -> float:
        cr = self.crystal
        return float(np.linalg.norm(cr.cart(s1[0], s1[1]) - cr.cart(s2[0], s2[1])))

    def _build_orbits(self, orbit_order):
        cr = self.crystal
        found = {}  # canonical key -> (max_l, min_l)
        clusters_at = {b: [] for b in cr.dof}  # (key, [centre] + partners)
        rmax = max([v for k, v in self.max_length.items() if k >= 2] + [0.0])
        for b in cr.dof:
            centre = (b, (0, 0, 0))
            key = canonical(self.ops, [centre])
            found.setdefault(key, (0.0, 0.0))
            clusters_at[b].append((key, [centre]))
            nb = self._neighbours(b, rmax) if rmax > 0 else []
            pos = np.array([cr.cart(s[0], s[1]) for s in nb]).reshape(-1, 3)
            dm = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=2) if len(nb) else None
            d0 = np.linalg.norm(pos - cr.cart(b, (0, 0, 0)), axis=1) if len(nb) else None
            for size in sorted(k for k in self.max_length if k >= 2):
                lim = self.max_length[size] + self.tol
                cand = [i for i in range(len(nb)) if d0[i] <= lim]
                for combo in itertools.combinations(cand, size - 1):
                    if any(dm[i, j] > lim for i, j in itertools.combinations(combo, 2)):
                        continue
                    sites = [centre] + [nb[i] for i in combo]
                    key = canonical(self.ops, sites)
                    if key not in found:
                        ds = [self._dist(s, t) for s, t in itertools.combinations(sites, 2)]
                        found[key] = (max(ds), min(ds))
                    clusters_at[b].append((key, sites))
        keys = sorted(found, key=lambda k: (len(k), round(found[k][0], 5), round(found[k][1], 5), k))
        if orbit_order is not None:
            want = []
            for proto in orbit_order:
                if len(proto) == 0:
                    continue  # the empty cluster is function 0
                k = canonical(self.ops, [(int(b), tuple(int(x) for x in u)) for b, u in proto])
                if k not in found:
                    raise ValueError(f"reference orbit {proto} is not among the built orbits")
                want.append(k)
            if sorted(want) != sorted(found):
                raise ValueError(
                    f"built {len(found)} orbits, the reference basis set has {len(want)}"
                )
            keys = want
        self.orbits = []
        idx = {}
        for i, k in enumerate(keys):
            mx, mn = found[k]
            proto = [(x[3], (x[0], x[1], x[2])) for x in k]
            o = Orbit(i, len(k), np.array([[x[0], x[1], x[2], x[3]] for x in k], dtype=np.int64),
                      proto, mx, mn, 0)
            self.orbits.append(o)
            idx[k] = i
        self._clusters_at = {b: [(idx[k], s) for k, s in clusters_at[b]] for b in clusters_at}
        counts = np.zeros(len(self.orbits), dtype=np.int64)
        for b in cr.dof:
            for oi, _ in self._clusters_at[b]:
                counts[oi] += 1
        for o in self.orbits:
            if counts[o.index] % o.size:
                raise RuntimeError("inconsistent orbit counting")
            o.mult = int(counts[o.index] // o.size)

    def _build_functions(self):
        f = 1
        self.func_orbit = [-1]
        self.func_coeff = [1.0]
        self.func_rep = [()]
        self._func_of_class = {}
        for o in self.orbits:
            o.func_begin = f
            classes = {}
            for assign in itertools.product(range(self.n_sf), repeat=o.size):
                key = canonical(self.ops, o.proto_sites, assign)
                classes.setdefault(key, []).append(assign)
            reps = sorted((min(v), key, len(v)) for key, v in classes.items())
            for rep, key, nterms in reps:
                coeff = round(1.0 / math.sqrt(nterms), 6)
                o.func_reps.append(rep)
                o.func_coeff.append(coeff)
                o.func_nterms.append(nterms)
                self._func_of_class[key] = f
                self.func_orbit.append(o.index)
                self.func_coeff.append(coeff)
                self.func_rep.append(rep)
                f += 1
            o.n_funcs = f - o.func_begin
        self.n_funcs = f
        self.func_orbit = np.array(self.func_orbit, dtype=np.int64)
        self.func_coeff = np.array(self.func_coeff, dtype=np.float64)

    def _build_flowers(self):
        self.flowers = {}
        self.owned = {}
        for b in self.crystal.dof:
            kb = self._kb[b]
            fl, own = [], []
            for oi, sites in self._clusters_at[b]:
                o = self.orbits[oi]
                partners = [(self._kb[s[0]], s[1]) for s in sites[1:]]
                lut = np.full(self.n_sf ** o.size, -1, dtype=np.int16)
                for combo in itertools.product(range(self.n_sf), repeat=o.size):
                    key = canonical(self.ops, sites, combo)
                    code = sum(s * self.n_sf**j for j, s in enumerate(combo))
                    lut[code] = self._func_of_class[key]
                c = FlowerCluster(oi, partners, lut)
                fl.append(c)
                first = min((u[0], u[1], u[2], bb) for bb, u in sites)
                if first == (0, 0, 0, b):
                    own.append(FlowerCluster(oi, partners, lut))
            fl.sort(key=lambda c: c.orbit)
            own.sort(key=lambda c: c.orbit)
            self.flowers[kb] = fl
            self.owned[kb] = own

    def function_signatures(self) -> list:
        raise NotImplementedError("general crystals identify functions by canonical forms")

    def prototype_sites(self, f: int) -> list:
        """Prototype of function f's orbit as [(b, (i, j, k))] in prim
        sublattice numbering."""
        return list(self.orbits[self.func_orbit[f]].proto_sites)
