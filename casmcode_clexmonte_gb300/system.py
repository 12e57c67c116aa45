"""Cluster-expansion system model for the Metropolis hot path.

This module builds, once per system, everything the GPU path needs to
evaluate the energy change of an occupation change:

* the crystal (``Prim``): lattice vectors and basis sites on an integer grid,
  so that all site coordinates and squared distances are exact integers;
* orbits of clusters (points, pairs, triplets, quadruplets) generated by
  per-branch maximum lengths, as CASM's ``periodic_max_length`` cluster specs
  do (reference ``tests/unit/clexmonte/data/FCC_binary_vacancy/
  formation_energy_eci.json`` ``bspecs.cluster_specs``);
* occupation-basis cluster functions, one per symmetry class of site-function
  decorations, with CASM's occupation site functions
  ``phi_k(occ) = [occ == k+1]`` (generated Clexulator
  ``FCC_binary_vacancy_Clexulator_default.cc:306-311``) and CASM's
  symmetrised coefficient ``sqrt(1/n_terms)`` printed to six decimals
  (``0.707107`` at ``:879-903``);
* per-sublattice "flower" tables: every cluster that contains a site, with
  its partner offsets and a decoration -> function look-up table, which is
  the data the generated ``_calc_delta_point_corr`` walks
  (``FCC_binary_vacancy_Clexulator_default.cc:555-580``);
* per-sublattice "owned" cluster lists used for the full energy
  (``per_supercell``), each periodic cluster counted exactly once;
* the site colouring used by the parallel sweep and the canonical pair-move
  geometry, verified on the host before any launch.

Energies follow the reference's normalisation: the extensive correlation of
function f is ``coeff_f * count_f / mult_b`` and
``E = sum_f ECI_f * coeff_f * count_f / mult_b`` (per supercell), where
``count_f`` is the integer number of clusters of the orbit whose decoration is
in class f and ``mult_b`` is the orbit multiplicity per unit cell (the
``mult`` field of the reference ECI files). The integer ``count_f`` changes are
the delta correlations the GPU reproduces exactly.
"""

from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# Boltzmann constant in eV/K (CODATA 2018). CASM::KB lives in libcasm-global,
# which the reference does not vendor.
KB = 8.617333262e-5


def cubic_point_group() -> list[np.ndarray]:
    """The 48 operations of the cubic point group m-3m as signed permutations."""
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            m = np.zeros((3, 3), dtype=np.int64)
            for r in range(3):
                m[r, perm[r]] = signs[r]
            ops.append(m)
    return ops


@dataclass
class Prim:
    """A crystal whose sites are all related by lattice translations of the
    crystal (a Bravais lattice, possibly described with a non-primitive cell).

    Coordinates are on an integer grid of spacing ``grid`` Angstrom:
    ``lattice`` rows are the cell vectors, ``basis`` rows the site positions.
    """

    title: str
    grid: float
    lattice: np.ndarray  # (3,3) int, rows = cell vectors in grid units
    basis: np.ndarray  # (n_basis,3) int, site positions in grid units
    occupants: tuple  # species names; occupant index 0 is the reference species

    @property
    def n_basis(self) -> int:
        return int(self.basis.shape[0])

    @property
    def n_occ(self) -> int:
        return len(self.occupants)

    def cart(self, b: int, u) -> np.ndarray:
        return np.asarray(u, dtype=np.int64) @ self.lattice + self.basis[b]

    def site_of(self, cart) -> tuple[int, tuple]:
        """Inverse of ``cart``: (sublattice, unit cell) of a grid point."""
        inv = np.linalg.inv(self.lattice.astype(float))
        for b in range(self.n_basis):
            f = (np.asarray(cart, dtype=float) - self.basis[b]) @ inv
            r = np.rint(f)
            if np.allclose(f, r, atol=1e-9):
                return b, tuple(int(x) for x in r)
        raise ValueError(f"grid point {cart} is not a site")


def fcc_prim(a: float = 4.0, occupants=("A", "B")) -> Prim:
    """FCC primitive cell with conventional lattice parameter ``a``; same cell
    as reference ``FCC_binary_vacancy/prim.json`` for a = 4.0."""
    return Prim(
        title="FCC",
        grid=a / 2.0,
        lattice=np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], dtype=np.int64),
        basis=np.zeros((1, 3), dtype=np.int64),
        occupants=tuple(occupants),
    )


def bcc_prim(a: float = 3.2, occupants=("A", "B", "C")) -> Prim:
    return Prim(
        title="BCC",
        grid=a / 2.0,
        lattice=np.array([[-1, 1, 1], [1, -1, 1], [1, 1, -1]], dtype=np.int64),
        basis=np.zeros((1, 3), dtype=np.int64),
        occupants=tuple(occupants),
    )


def bcc_conventional(a: float = 3.2, occupants=("A", "B", "C")) -> Prim:
    """Two-site cubic BCC cell: an L x L x L supercell of it has 2 L^3 sites."""
    return Prim(
        title="BCC_conventional",
        grid=a / 2.0,
        lattice=np.array([[2, 0, 0], [0, 2, 0], [0, 0, 2]], dtype=np.int64),
        basis=np.array([[0, 0, 0], [1, 1, 1]], dtype=np.int64),
        occupants=tuple(occupants),
    )


# --------------------------------------------------------------------------
# cluster canonical forms


def _canon_points(pts: np.ndarray, ops) -> tuple:
    best = None
    for op in ops:
        q = pts @ op.T
        o = q[np.lexsort(q.T[::-1])]
        o = o - o[0]
        key = tuple(map(tuple, o.tolist()))
        if best is None or key < best:
            best = key
    return best


def _canon_decorated(pts: np.ndarray, labels, ops) -> tuple:
    best = None
    lab = np.asarray(labels, dtype=np.int64).reshape(-1, 1)
    for op in ops:
        q = pts @ op.T
        mn = q[np.lexsort(q.T[::-1])][0]
        q = np.hstack([q - mn, lab])
        o = q[np.lexsort(q.T[::-1])]
        key = tuple(map(tuple, o.tolist()))
        if best is None or key < best:
            best = key
    return best


def _sq(d) -> int:
    d = np.asarray(d, dtype=np.int64)
    return int((d * d).sum())


def signature(pts: np.ndarray, occs) -> tuple:
    """Translation/rotation invariant of a decorated cluster: sorted edge list
    (squared length, species pair) and sorted species. The oracle identifies
    cluster functions by this invariant instead of by symmetry operations."""
    n = len(pts)
    edges = []
    for i in range(n):
        for j in range(i + 1, n):
            a, b = int(occs[i]), int(occs[j])
            edges.append((_sq(pts[i] - pts[j]), min(a, b), max(a, b)))
    return (n, tuple(sorted(edges)), tuple(sorted(int(o) for o in occs)))


@dataclass
class Orbit:
    index: int
    size: int
    prototype: np.ndarray  # (size,3) grid points, canonical translation
    proto_sites: list  # [(b, u)] sites of the prototype
    max_length: float
    min_length: float
    mult: int  # clusters per unit cell
    func_begin: int = 0
    n_funcs: int = 0
    func_reps: list = field(default_factory=list)  # representative sf tuples
    func_coeff: list = field(default_factory=list)
    func_nterms: list = field(default_factory=list)


@dataclass
class FlowerCluster:
    orbit: int
    partners: list  # [(b', du)] other sites, in prototype-consistent order
    lut: np.ndarray  # int16 [(n_sf)**size] -> global function index


def _lattice_index(vecs) -> int:
    """Index in Z^3 of the lattice spanned by integer 3-vectors (0 if they
    span less than three dimensions): integer row echelon form by Euclid's
    algorithm, index = |product of the pivots|."""
    rows = [list(v) for v in vecs if any(v)]
    det = 1
    for col in range(3):
        piv, rest = None, []
        for r in rows:
            if r[col] == 0:
                rest.append(r)
            elif piv is None:
                piv = r
            else:
                a, b = piv, r
                while b[col] != 0:
                    q = a[col] // b[col]
                    a = [x - q * y for x, y in zip(a, b)]
                    a, b = b, a
                piv = a
                if any(b):
                    rest.append(b)
        if piv is None:
            return 0
        det *= piv[col]
        rows = [r for r in rest if any(r)]
    return abs(det)


def _swaps_connect(subl, edges) -> bool:
    """Whether swaps of site (b, x) with (pb, x + du), for the given edges
    (b, pb, du), connect every site of the sublattices ``subl`` on the
    infinite lattice: the graph over the sublattices is connected and the
    translations of its cycles generate Z^3."""
    adj = {b: [] for b in subl}
    for b, pb, du in edges:
        adj[b].append((pb, du))
        adj[pb].append((b, tuple(-x for x in du)))
    pot = {subl[0]: (0, 0, 0)}
    stack = [subl[0]]
    while stack:
        b = stack.pop()
        for pb, du in adj[b]:
            if pb not in pot:
                pot[pb] = tuple(p + d for p, d in zip(pot[b], du))
                stack.append(pb)
    if len(pot) != len(subl):
        return False
    cycles = [tuple(p + d - q for p, d, q in zip(pot[b], du, pot[pb])) for b, pb, du in edges]
    return _lattice_index(cycles) == 1


class ClusterExpansion:
    """Orbits, occupation-basis functions and ECI for a ``Prim``.

    ``max_length`` maps cluster size (2, 3, 4) to the maximum site-to-site
    distance in Angstrom, as CASM's ``orbit_branch_specs``.
    """

    def __init__(self, prim: Prim, max_length: dict, eci=None, tol: float = 1e-5):
        self.prim = prim
        self.ops = cubic_point_group()
        self._check_symmetry()
        self.max_length = {int(k): float(v) for k, v in max_length.items()}
        self.tol = tol
        self.n_sf = prim.n_occ - 1
        self._build_orbits()
        self._build_functions()
        self._build_flowers()
        self.eci = np.zeros(self.n_funcs) if eci is None else np.asarray(eci, float)
        if self.eci.shape != (self.n_funcs,):
            raise ValueError(f"eci must have {self.n_funcs} entries")
        # R^T of the parametric composition axes; None = the standard axes
        # (origin: every site occupant 0; end member k: every site occupant k)
        self.param_RT = None

    # ---- symmetry
    def _check_symmetry(self):
        p = self.prim
        pts = {tuple(p.cart(b, (0, 0, 0))) for b in range(p.n_basis)}
        for op in self.ops:
            for b in range(p.n_basis):
                q = p.basis[b] @ op.T
                p.site_of(q)  # raises if not a site
            _ = pts

    # ---- neighbourhood of a basis site
    def _neighbours(self, b: int, rmax: float):
        p = self.prim
        r2max = (rmax / p.grid) ** 2 + self.tol
        c0 = p.cart(b, (0, 0, 0))
        n = int(math.ceil(rmax / p.grid / 1.0)) + 2
        out = []
        for u in itertools.product(range(-n, n + 1), repeat=3):
            for bb in range(p.n_basis):
                c = p.cart(bb, u)
                d2 = _sq(c - c0)
                if 0 < d2 <= r2max:
                    out.append(c)
        return out

    def _build_orbits(self):
        p = self.prim
        found = {}  # canon -> (pts, max_l, min_l)
        clusters_at = {b: [] for b in range(p.n_basis)}  # (canon, pts incl centre first)
        for b in range(p.n_basis):
            c0 = p.cart(b, (0, 0, 0))
            # point
            pts = c0.reshape(1, 3)
            key = _canon_points(pts, self.ops)
            found.setdefault(key, (pts, 0.0, 0.0))
            clusters_at[b].append((key, pts))
            for size in sorted(self.max_length):
                rmax = self.max_length[size]
                r2 = (rmax / p.grid) ** 2 + self.tol
                nb = self._neighbours(b, rmax)
                for combo in itertools.combinations(range(len(nb)), size - 1):
                    q = np.vstack([c0] + [nb[i] for i in combo])
                    ok = True
                    d2s = []
                    for i in range(size):
                        for j in range(i + 1, size):
                            d2 = _sq(q[i] - q[j])
                            d2s.append(d2)
                            if d2 > r2:
                                ok = False
                    if not ok:
                        continue
                    key = _canon_points(q, self.ops)
                    if key not in found:
                        found[key] = (
                            np.array(key, dtype=np.int64),
                            math.sqrt(max(d2s)) * p.grid,
                            math.sqrt(min(d2s)) * p.grid,
                        )
                    clusters_at[b].append((key, q))
        order = sorted(
            found.keys(),
            key=lambda k: (len(k), round(found[k][1], 6), round(found[k][2], 6), k),
        )
        self.orbits = []
        idx = {}
        for i, k in enumerate(order):
            pts, mx, mn = found[k]
            sites = [p.site_of(c) for c in np.array(k, dtype=np.int64)]
            self.orbits.append(
                Orbit(i, len(k), np.array(k, dtype=np.int64), sites, mx, mn, 0)
            )
            idx[k] = i
        self._clusters_at = {
            b: [(idx[k], q) for (k, q) in clusters_at[b]] for b in clusters_at
        }
        counts = np.zeros(len(self.orbits), dtype=np.int64)
        for b in range(p.n_basis):
            for oi, _ in self._clusters_at[b]:
                counts[oi] += 1
        for o in self.orbits:
            if counts[o.index] % o.size:
                raise RuntimeError("inconsistent orbit counting")
            o.mult = int(counts[o.index] // o.size)

    def _build_functions(self):
        """One function per symmetry class of site-function assignments."""
        f = 1  # function 0 is the empty cluster
        self.func_orbit = [-1]
        self.func_coeff = [1.0]
        self.func_rep = [()]
        self._func_of_class = {}
        for o in self.orbits:
            o.func_begin = f
            classes = {}
            for assign in itertools.product(range(self.n_sf), repeat=o.size):
                key = _canon_decorated(o.prototype, assign, self.ops)
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
        p = self.prim
        self.flowers = {}
        self.owned = {}
        for b in range(p.n_basis):
            c0 = p.cart(b, (0, 0, 0))
            fl = []
            own = []
            for oi, q in self._clusters_at[b]:
                o = self.orbits[oi]
                partners = [p.site_of(c) for c in q[1:]]
                lut = np.full(self.n_sf ** o.size, -1, dtype=np.int16)
                for combo in itertools.product(range(self.n_sf), repeat=o.size):
                    key = _canon_decorated(q, combo, self.ops)
                    code = 0
                    for j, s in enumerate(combo):
                        code += s * self.n_sf**j
                    lut[code] = self._func_of_class[key]
                fl.append(FlowerCluster(oi, partners, lut))
                # anchor = lexicographically smallest grid point
                o_ = q[np.lexsort(q.T[::-1])]
                if tuple(o_[0]) == tuple(c0):
                    own.append(FlowerCluster(oi, partners, lut))
            fl.sort(key=lambda c: c.orbit)
            own.sort(key=lambda c: c.orbit)
            self.flowers[b] = fl
            self.owned[b] = own

    # ---- derived quantities
    @property
    def func_mult(self) -> np.ndarray:
        m = np.ones(self.n_funcs, dtype=np.float64)
        for f in range(1, self.n_funcs):
            m[f] = self.orbits[self.func_orbit[f]].mult
        return m

    def weights(self) -> np.ndarray:
        """Per-count energy weight W_f = ECI_f * coeff_f / mult_f (f >= 1);
        W_0 = ECI_0 (the empty cluster, multiplied by the number of cells)."""
        w = self.eci * self.func_coeff / self.func_mult
        w[0] = self.eci[0]
        return w

    def flower_reach(self) -> int:
        """Largest |unit-cell offset component| over all flower partners."""
        r = 0
        for b, fl in self.flowers.items():
            for c in fl:
                for bb, du in c.partners:
                    r = max(r, max(abs(x) for x in du))
        return r

    def neighbour_partners(self, b: int) -> list:
        """Displacements (partner sublattice, cell offset) of the canonical
        local swaps of sublattice b: the partners of the shortest pair
        orbits. Orbits are taken in order of length until the swaps connect
        every site of every sublattice with a degree of freedom, i.e. the
        displacement graph over those sublattices is connected and its cycle
        translations generate the whole lattice Z^3. Swaps inside a colour
        class only permute that class, so this connectivity is what makes the
        canonical chain ergodic (the reference's canonical proposal swaps any
        two sites, CanonicalCalculator.cc:78-83). FCC and BCC: the nearest
        neighbours already do; hcp Zr-O: the O-O pairs along c do not (they
        only link the octahedral sites of one column), the in-plane pairs are
        added."""
        return [c.partners[0] for c in self.flowers[b] if c.orbit in self.local_swap_orbits()]

    def local_swap_orbits(self) -> frozenset:
        """Indices of the pair orbits whose partners are the local-swap
        displacements (see neighbour_partners)."""
        cached = getattr(self, "_local_swap_orbits", None)
        if cached is not None:
            return cached
        pairs = sorted((o for o in self.orbits if o.size == 2), key=lambda o: (o.max_length, o.index))
        subl = sorted(self.flowers)
        chosen = set()
        result = frozenset()
        for o in pairs:
            chosen.add(o.index)
            edges = [(b, c.partners[0][0], tuple(int(x) for x in c.partners[0][1]))
                     for b in subl for c in self.flowers[b] if c.orbit in chosen]
            if _swaps_connect(subl, edges):
                result = frozenset(chosen)
                break
        else:
            if pairs:
                raise ValueError("no set of pair orbits connects the sites with a degree of freedom: "
                                 "canonical local swaps would not be ergodic")
        self._local_swap_orbits = result
        return result

    def function_signatures(self) -> list:
        """For each function f >= 1: decorated-cluster invariant of its
        representative (occupants = site-function index + 1), plus its orbit's
        undecorated invariant."""
        out = [None]
        for f in range(1, self.n_funcs):
            o = self.orbits[self.func_orbit[f]]
            rep = self.func_rep[f]
            occs = [s + 1 for s in rep]
            out.append(signature(o.prototype, occs))
        return out

    def describe(self) -> str:
        lines = []
        for o in self.orbits:
            lines.append(
                f"orbit {o.index}: size {o.size} mult {o.mult} "
                f"max_length {o.max_length:.4f} funcs {o.n_funcs} "
                f"coeff {o.func_coeff}"
            )
        return "\n".join(lines)


# --------------------------------------------------------------------------
# supercells, colouring and pair-move geometry


@dataclass
class Supercell:
    """Diagonal supercell ``T = diag(L)`` of a prim; linear site index
    ``l = b * n_uc + (i + Lx * (j + Ly * k))`` (sublattice-major, as the
    reference's ``l = b * N_uc + uc`` in
    ``tests/unit/clexmonte/canonical_metropolis_test.cpp:34-36``)."""

    L: tuple

    @property
    def n_uc(self) -> int:
        return int(self.L[0] * self.L[1] * self.L[2])

    def n_sites(self, prim: Prim) -> int:
        return self.n_uc * prim.n_basis

    def index(self, b, i, j, k):
        Lx, Ly, Lz = self.L
        return b * self.n_uc + (i % Lx) + Lx * ((j % Ly) + Ly * (k % Lz))

    def coords(self, prim: Prim):
        n = self.n_sites(prim)
        l = np.arange(n, dtype=np.int64)
        b = l // self.n_uc
        uc = l % self.n_uc
        Lx, Ly, _ = self.L
        return b, uc % Lx, (uc // Lx) % Ly, uc // (Lx * Ly)


def neighbour_index_table(ce: ClusterExpansion, sc: Supercell, clusters="flowers"):
    """Explicit site indices of every flower (or owned) cluster of every site:
    returns (site_partner[n_sites, n_clusters_max, 3], cluster_orbit...) with
    -1 padding. Used by host-side checks, not by the GPU path."""
    prim = ce.prim
    b, i, j, k = sc.coords(prim)
    tables = ce.flowers if clusters == "flowers" else ce.owned
    nmax = max(len(v) for v in tables.values())
    n = sc.n_sites(prim)
    part = np.full((n, nmax, 3), -1, dtype=np.int64)
    for bb, fl in tables.items():
        sel = np.nonzero(b == bb)[0]
        for ci, c in enumerate(fl):
            for pj, (pb, du) in enumerate(c.partners):
                part[sel, ci, pj] = sc.index(pb, i[sel] + du[0], j[sel] + du[1], k[sel] + du[2])
    return part


def _axis_blocks(L: int, p: int) -> np.ndarray:
    """Colour of each coordinate on a ring of length L, cut into blocks of
    size >= p (block sizes p or p+1...), colour = position within the block."""
    q = L // p
    if q == 0:
        raise ValueError(f"supercell length {L} is shorter than colour block {p}")
    sizes = [p] * q
    for r in range(L - q * p):
        sizes[r % q] += 1
    col = []
    for s in sizes:
        col.extend(range(s))
    return np.array(col, dtype=np.int64)


@dataclass
class Colouring:
    """Site colour classes: sites of one class never share a cluster, so all
    sites of a class can be updated at once. Class = (sublattice, cx, cy, cz).
    ``axis_coords[a][c]`` lists the coordinates of colour c along axis a."""

    p: int
    n_colours: tuple  # per axis
    axis_coords: list  # [axis][colour] -> np.ndarray of coordinates
    n_sublat: int

    @property
    def n_classes(self) -> int:
        return self.n_sublat * int(np.prod(self.n_colours))

    def class_dims(self, c: int):
        b, rest = divmod(c, int(np.prod(self.n_colours)))
        nx, ny, _ = self.n_colours
        cx = rest % nx
        cy = (rest // nx) % ny
        cz = rest // (nx * ny)
        return b, (cx, cy, cz), tuple(len(self.axis_coords[a][(cx, cy, cz)[a]]) for a in range(3))

    def class_of_sites(self, sc: Supercell, prim: Prim) -> np.ndarray:
        b, i, j, k = sc.coords(prim)
        cols = [_axis_blocks(sc.L[a], self.p) for a in range(3)]
        nx, ny, nz = self.n_colours
        return b * (nx * ny * nz) + cols[0][i] + nx * (cols[1][j] + ny * cols[2][k])


def make_colouring(ce: ClusterExpansion, sc: Supercell, p_start: int = 2) -> Colouring:
    """Smallest per-axis block size whose colour classes contain no two
    interacting sites (checked against every flower partner of every site)."""
    prim = ce.prim
    part = neighbour_index_table(ce, sc)
    n = sc.n_sites(prim)
    for p in range(p_start, max(sc.L) + 1):
        try:
            cols = [_axis_blocks(sc.L[a], p) for a in range(3)]
        except ValueError:
            break
        ncol = tuple(int(c.max()) + 1 for c in cols)
        axis_coords = [
            [np.nonzero(cols[a] == c)[0] for c in range(ncol[a])] for a in range(3)
        ]
        col = Colouring(p, ncol, axis_coords, prim.n_basis)
        cls = col.class_of_sites(sc, prim)
        flat = part.reshape(n, -1)
        valid = flat >= 0
        site_rep = np.repeat(np.arange(n)[:, None], flat.shape[1], axis=1)
        if np.any(flat[valid] == site_rep[valid]):
            raise ValueError("supercell too small: a cluster contains a site twice")
        if np.any(cls[flat[valid]] == cls[site_rep[valid]]):
            continue
        return col
    raise ValueError("no valid colouring for this supercell")


def verify_local_pairs(ce: ClusterExpansion, sc: Supercell, col: Colouring) -> bool:
    """Check that every local pair sub-step the parallel kernel can draw is
    made of pairwise non-interacting pairs: class c, every other coordinate of
    the class along each axis (after any rotation), displacement = one
    nearest-neighbour vector. Returns True or raises."""
    prim = ce.prim
    part = neighbour_index_table(ce, sc)
    n = sc.n_sites(prim)
    flat = part.reshape(n, -1)
    for c in range(col.n_classes):
        b, cc, dims = col.class_dims(c)
        for rot in itertools.product(*[range(min(d, 2)) for d in dims]):
            for par in itertools.product((0, 1), repeat=3):
                sel = []
                for a in range(3):
                    d = dims[a]
                    dd = d - (d & 1)
                    idx = [(rot[a] + par[a] + 2 * t) % d for t in range(dd // 2)] if d > 1 else [0]
                    if d > 1 and par[a] >= dd:
                        idx = []
                    sel.append(col.axis_coords[a][cc[a]][idx])
                if any(len(s) == 0 for s in sel):
                    continue
                ii, jj, kk = np.meshgrid(*sel, indexing="ij")
                s = sc.index(b, ii.ravel(), jj.ravel(), kk.ravel())
                for pb, du in ce.neighbour_partners(b):
                    t = sc.index(pb, ii.ravel() + du[0], jj.ravel() + du[1], kk.ravel() + du[2])
                    owner = np.full(n, -1, dtype=np.int64)
                    pid = np.arange(len(s))
                    if np.any(owner[s] >= 0):
                        raise ValueError("pair overlap")
                    owner[s] = pid
                    if np.any(owner[t] >= 0):
                        raise ValueError("pair members collide")
                    owner[t] = pid
                    for members in (s, t):
                        nb = flat[members]
                        ok = nb < 0
                        other = owner[np.where(ok, 0, nb)]
                        bad = (~ok) & (other >= 0) & (other != pid[:, None])
                        if np.any(bad):
                            raise ValueError(
                                f"local pair move interacts: class {c} delta {du}"
                            )
    return True


def composition_RT(n_basis: int, n_occ: int) -> np.ndarray:
    """R^T = dparam_dmol for the standard composition axes (origin: every
    site occupant 0; end member k: every site occupant k): the change of the
    parametric composition per change of the species counts per unit cell
    (reference ``SemiGrandCanonicalCalculator.cc:144``)."""
    Q = np.zeros((n_occ, n_occ - 1))
    for k in range(1, n_occ):
        Q[0, k - 1] = -n_basis
        Q[k, k - 1] = n_basis
    return np.ascontiguousarray(np.linalg.pinv(Q))


def param_RT_of(ce: ClusterExpansion) -> np.ndarray:
    """R^T of the cluster expansion's composition axes (standard axes unless
    set from a CASM system file)."""
    rt = getattr(ce, "param_RT", None)
    if rt is None:
        return composition_RT(ce.prim.n_basis, ce.prim.n_occ)
    return np.ascontiguousarray(rt, dtype=np.float64)


def system_arrays(ce: ClusterExpansion) -> dict:
    """Flat arrays of the C ABI's ``cem_system_desc`` for a cluster expansion."""
    n_sf = ce.n_sf
    stride = n_sf**4
    orbits = ce.orbits
    out = dict(
        n_sublat=ce.prim.n_basis,
        n_occ=ce.prim.n_occ,
        n_funcs=ce.n_funcs,
        n_orbits=len(orbits),
        orbit_size=np.array([o.size for o in orbits], dtype=np.int32),
        orbit_func_begin=np.array([o.func_begin for o in orbits], dtype=np.int32),
        orbit_n_funcs=np.array([o.n_funcs for o in orbits], dtype=np.int32),
        weights=np.ascontiguousarray(ce.weights(), dtype=np.float64),
        param_RT=param_RT_of(ce).reshape(-1),
    )
    for name, table in (("flower", ce.flowers), ("owned", ce.owned)):
        sub, orb, psub, pdu, lut = [], [], [], [], []
        for b in range(ce.prim.n_basis):
            for c in table[b]:
                sub.append(b)
                orb.append(c.orbit)
                ps = [-1, -1, -1]
                pd = [0] * 9
                for j, (pb, du) in enumerate(c.partners):
                    ps[j] = pb
                    pd[3 * j : 3 * j + 3] = list(du)
                psub.append(ps)
                pdu.append(pd)
                row = np.full(stride, -1, dtype=np.int16)
                row[: len(c.lut)] = c.lut
                lut.append(row)
        out[f"n_{name}"] = len(sub)
        out[f"{name}_sublat"] = np.array(sub, dtype=np.int32)
        out[f"{name}_orbit"] = np.array(orb, dtype=np.int32)
        out[f"{name}_partner_sublat"] = np.array(psub, dtype=np.int32).reshape(-1)
        out[f"{name}_partner_du"] = np.array(pdu, dtype=np.int32).reshape(-1)
        out[f"{name}_lut"] = np.array(lut, dtype=np.int16).reshape(-1)
    nb_n = np.zeros(ce.prim.n_basis, dtype=np.int32)
    nb_s = np.zeros((ce.prim.n_basis, 16), dtype=np.int32)
    nb_d = np.zeros((ce.prim.n_basis, 16, 3), dtype=np.int32)
    for b in range(ce.prim.n_basis):
        nbs = ce.neighbour_partners(b)[:16]
        nb_n[b] = len(nbs)
        for k, (pb, du) in enumerate(nbs):
            nb_s[b, k] = pb
            nb_d[b, k] = du
    out["n_neighbour"] = nb_n
    out["neighbour_sublat"] = nb_s.reshape(-1)
    out["neighbour_du"] = nb_d.reshape(-1)
    return out
