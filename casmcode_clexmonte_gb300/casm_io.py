"""Reference-format input and results output.

* ``read_system``: a CASM ``system.json`` (prim, composition axes, the
  formation-energy basis set and its coefficients).
* ``read_prim`` / ``read_cluster_expansion``: CASM ``prim.json`` and the basis
  set / ECI JSON (``formation_energy_eci.json``: ``bspecs`` with
  ``orbit_branch_specs`` max lengths, ``orbits`` with ``mult`` and
  ``cluster_functions`` / ``eci``), or a sparse ECI list ``[[index, value]]``
  (reference ``tests/unit/clexmonte/data/FCC_binary_vacancy/``). Supported:
  crystals whose sites are all related by lattice translations and whose point
  group is cubic (FCC, BCC); the orbit structure built here is checked against
  the file's orbits (sizes, multiplicities, function counts) before its ECI are
  used.
* ``write_eci_json``: the same schema, for a cluster expansion built here.
* ``SummaryWriter``: results of a series of runs in the layout of the
  reference's ``summary.json`` (``analysis``, ``completion_check_results``,
  ``conditions``, ``statistics``; one list entry per run), the file the
  reference's tests read back (``python/tests/conftest.py:141-259``).
"""

from __future__ import annotations

import json
import os

import numpy as np

from .crystal import Crystal, CrystalClusterExpansion
from .system import KB, ClusterExpansion, Prim, cubic_point_group


def _integer_grid(lattice: np.ndarray, basis_cart: np.ndarray, tol: float = 1e-6):
    vals = np.abs(np.concatenate([lattice.ravel(), basis_cart.ravel()]))
    vals = vals[vals > tol]
    best = None
    for v in sorted(set(np.round(vals, 9))):
        for k in range(1, 13):
            g = v / k
            ok = np.all(np.abs(lattice / g - np.rint(lattice / g)) < tol) and np.all(
                np.abs(basis_cart / g - np.rint(basis_cart / g)) < tol)
            if ok and (best is None or g > best):
                best = g
    if best is None:
        raise ValueError("prim coordinates do not lie on an integer grid")
    return best


def read_prim(src) -> Prim:
    d = json.load(open(src)) if isinstance(src, (str, os.PathLike)) else src
    lat = np.array(d["lattice_vectors"], dtype=float)
    mode = d.get("coordinate_mode", "Fractional").lower()
    coords = np.array([b["coordinate"] for b in d["basis"]], dtype=float)
    cart = coords @ lat if mode.startswith("frac") else coords
    occs = [tuple(b["occupants"]) for b in d["basis"]]
    if any(o != occs[0] for o in occs):
        raise ValueError("every basis site must allow the same occupants")
    g = _integer_grid(lat, cart)
    return Prim(
        title=d.get("title", "prim"),
        grid=g,
        lattice=np.rint(lat / g).astype(np.int64),
        basis=np.rint(cart / g).astype(np.int64),
        occupants=occs[0],
    )


def read_crystal(src) -> Crystal:
    """Any CASM ``prim.json``: lattice, basis (fractional or Cartesian) and
    the occupants of every basis site."""
    d = json.load(open(src)) if isinstance(src, (str, os.PathLike)) else src
    lat = np.array(d["lattice_vectors"], dtype=float)
    mode = d.get("coordinate_mode", "Fractional").lower()
    coords = np.array([b["coordinate"] for b in d["basis"]], dtype=float)
    frac = coords if mode.startswith("frac") else coords @ np.linalg.inv(lat)
    return Crystal(d.get("title", "prim"), lat, frac, [tuple(b["occupants"]) for b in d["basis"]])


def _cubic_prim(d: dict):
    """The cubic builder's ``Prim`` when every site allows the same (two or
    more) occupants, the sites lie on an integer grid and the cubic point
    group maps the crystal onto itself; None otherwise."""
    occs = [tuple(b["occupants"]) for b in d["basis"]]
    if len(occs[0]) < 2 or any(o != occs[0] for o in occs):
        return None
    try:
        prim = read_prim(d)
        for op in cubic_point_group():
            for b in range(prim.n_basis):
                prim.site_of(prim.basis[b] @ op.T)
    except ValueError:
        return None
    return prim


def _max_lengths(bspecs: dict) -> dict:
    br = bspecs["cluster_specs"]["params"]["orbit_branch_specs"]
    return {int(k): float(v["max_length"]) for k, v in br.items() if int(k) >= 2}


def read_cluster_expansion(prim_src, eci_src, sparse_eci=None) -> ClusterExpansion:
    """Cluster expansion from CASM files; ECI from ``eci_src`` (its
    ``cluster_functions[*].eci``) or from a sparse list ``[[index, value]]``."""
    pd = json.load(open(prim_src)) if isinstance(prim_src, (str, os.PathLike)) else prim_src
    d = json.load(open(eci_src)) if isinstance(eci_src, (str, os.PathLike)) else eci_src
    basis = d.get("bspecs", {}).get("basis_function_specs", {})
    site_bf = basis.get("dof_specs", {}).get("occ", {}).get("site_basis_functions", "OCCUPATION")
    if str(site_bf).upper() != "OCCUPATION":
        raise ValueError(f"site basis functions '{site_bf}' are not supported (occupation only)")
    orbits = d["orbits"]
    prim = _cubic_prim(pd)
    if prim is not None:
        ce = ClusterExpansion(prim, _max_lengths(d["bspecs"]))
    else:
        protos = None
        if all("prototype" in o and "sites" in o["prototype"] for o in orbits):
            protos = [[(int(x[0]), tuple(int(v) for v in x[1:])) for x in o["prototype"]["sites"]]
                      for o in orbits]
        ce = CrystalClusterExpansion(read_crystal(pd), _max_lengths(d["bspecs"]), orbit_order=protos)
    if len(orbits) != len(ce.orbits) + 1:
        raise ValueError(f"file has {len(orbits)} orbits, built {len(ce.orbits) + 1}")
    eci = np.zeros(ce.n_funcs)
    for k, o in enumerate(orbits):
        funcs = o["cluster_functions"]
        if k == 0:
            if len(funcs) != 1:
                raise ValueError("orbit 0 must be the empty cluster")
        else:
            mine = ce.orbits[k - 1]
            n_sites = len(o["prototype"]["sites"]) if "prototype" in o else mine.size
            if n_sites != mine.size or o["mult"] != mine.mult or len(funcs) != mine.n_funcs:
                raise ValueError(
                    f"orbit {k}: file (size {n_sites}, mult {o['mult']}, {len(funcs)} functions)"
                    f" != built (size {mine.size}, mult {mine.mult}, {mine.n_funcs} functions)")
        for f in funcs:
            if "eci" in f:
                eci[int(f["linear_function_index"])] = float(f["eci"])
    if sparse_eci is not None:
        sp = json.load(open(sparse_eci)) if isinstance(sparse_eci, (str, os.PathLike)) else sparse_eci
        eci[:] = 0.0
        for idx, val in sp:
            eci[int(idx)] = float(val)
    ce.eci = eci
    return ce


def composition_axes_RT(axes: dict, occupants, fixed=None) -> np.ndarray:
    """R^T (independent axes x occupants, in the prim's occupant order) of
    CASM composition axes (``origin`` and one end member per axis, species
    per unit cell, over ``components``). ``occupants`` are the species of the
    sublattices with a degree of freedom; ``fixed`` maps the species of the
    single-occupant sublattices to their count per unit cell. The samplers
    count the composition from the state where every site with a degree of
    freedom holds occupant 0, so the origin must be that state, and no axis
    may change a species that only the fixed sublattices hold."""
    fixed = dict(fixed or {})
    comps = list(axes["components"])
    species = list(occupants) + [c for c in fixed if c not in occupants]
    if sorted(comps) != sorted(species):
        raise ValueError(f"composition components {comps} differ from the species {species}")
    origin = np.asarray(axes["origin"], dtype=np.float64).reshape(-1)
    names = [k for k in "abcdefghijklmnopqrstuvwxyz" if k in axes]
    if len(names) != len(occupants) - 1:
        raise ValueError(f"expected {len(occupants) - 1} independent composition axes, found {len(names)}")
    Q = np.stack([np.asarray(axes[k], dtype=np.float64).reshape(-1) - origin for k in names], axis=1)
    n_dof = origin[[comps.index(o) for o in occupants]].sum() - sum(
        fixed.get(o, 0) for o in occupants)
    expect = np.zeros(len(comps))
    for c, n in fixed.items():
        expect[comps.index(c)] += n
    expect[comps.index(occupants[0])] += n_dof
    if not np.allclose(origin, expect):
        raise ValueError("composition axes whose origin is not 'every site occupant 0' are not supported")
    for c in comps:
        if c not in occupants and np.any(np.abs(Q[comps.index(c)]) > 1e-12):
            raise ValueError(f"a composition axis changes {c}, which no site can take or lose")
    RT = np.linalg.pinv(Q)
    return np.ascontiguousarray(RT[:, [comps.index(o) for o in occupants]])


def read_system(path: str) -> ClusterExpansion:
    """Formation-energy cluster expansion of a CASM ``system.json``
    (``System_json_io.cc:491-538``): ``prim``, ``composition_axes``,
    ``clex.formation_energy`` = (basis set, coefficients). The basis set's
    functions are rebuilt from its ``bspecs`` (the generated Clexulator
    source is not compiled) and checked orbit by orbit against the
    coefficients file, or against the basis set's ``basis.json`` when the
    coefficients are a sparse ``[[index, value]]`` list."""
    base = os.path.dirname(os.path.abspath(path))
    d = json.load(open(path))
    clex = d["clex"]["formation_energy"]
    bset = d["basis_sets"][clex["basis_set"]]
    bdir = os.path.dirname(os.path.join(base, bset["source"]))
    coef = json.load(open(os.path.join(base, clex["coefficients"])))
    if isinstance(coef, dict):
        doc = dict(coef)
        if "bspecs" not in doc:
            doc["bspecs"] = json.load(open(os.path.join(bdir, "bspecs.json")))
        ce = read_cluster_expansion(d["prim"], doc)
    else:
        basis = json.load(open(os.path.join(bdir, "basis.json")))
        if "bspecs" not in basis:
            basis["bspecs"] = json.load(open(os.path.join(bdir, "bspecs.json")))
        ce = read_cluster_expansion(d["prim"], basis, sparse_eci=coef)
    if "composition_axes" in d:
        cr = getattr(ce, "crystal", None)
        ce.param_RT = composition_axes_RT(d["composition_axes"], ce.prim.occupants,
                                          cr.fixed_counts() if cr is not None else None)
    return ce


def _prim_doc(ce) -> dict:
    cr = getattr(ce, "crystal", None)
    if cr is not None:
        return {
            "title": cr.title,
            "coordinate_mode": "Fractional",
            "lattice_vectors": cr.lattice.tolist(),
            "basis": [{"coordinate": cr.frac[b].tolist(), "occupants": list(cr.occupants[b])}
                      for b in range(cr.n_basis)],
        }
    p = ce.prim
    return {
        "title": p.title,
        "coordinate_mode": "Cartesian",
        "lattice_vectors": (p.lattice * p.grid).tolist(),
        "basis": [{"coordinate": (b * p.grid).tolist(), "occupants": list(p.occupants)}
                  for b in p.basis],
    }


def write_eci_json(ce: ClusterExpansion, path: str):
    orbits = [{
        "linear_orbit_index": 0, "mult": 1,
        "cluster_functions": [{"linear_function_index": 0, "eci": float(ce.eci[0])}],
        "prototype": {"sites": [], "max_length": 0.0, "min_length": 0.0},
    }]
    for o in ce.orbits:
        orbits.append({
            "linear_orbit_index": o.index + 1,
            "mult": int(o.mult),
            "cluster_functions": [
                {"linear_function_index": int(o.func_begin + j), "eci": float(ce.eci[o.func_begin + j])}
                for j in range(o.n_funcs)
            ],
            "prototype": {
                "sites": [[int(b)] + [int(x) for x in u] for b, u in o.proto_sites],
                "max_length": float(o.max_length), "min_length": float(o.min_length),
            },
        })
    branch = {"0": {"max_length": 0.0}, "1": {"max_length": 0.0}}
    for k, v in ce.max_length.items():
        branch[str(k)] = {"max_length": float(v)}
    doc = {
        "bspecs": {
            "basis_function_specs": {"dof_specs": {"occ": {"site_basis_functions": "OCCUPATION"}},
                                     "dofs": ["occ"]},
            "cluster_specs": {"method": "periodic_max_length",
                              "params": {"orbit_branch_specs": branch}},
        },
        "orbits": orbits,
        "prim": _prim_doc(ce),
    }
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


def equilibration_index(x, precision: float, n_blocks: int = 20):
    """First sample after which the series counts as equilibrated, or None.

    The series is split at its midpoint; the start of the first half is moved
    forward one block (N / ``n_blocks`` samples) at a time until the mean of
    [start, N/2) and the mean of [N/2, N) agree within ``precision``. This is
    the two-partition equilibration test described for CASM's Monte Carlo
    completion checks (``monte::default_equilibration_check``, used at
    ``CanonicalCalculator.cc:264``; that function lives in libcasm-monte,
    which is not part of this project's sources)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    if n < 2 * n_blocks:
        return None
    half = n // 2
    second = x[half:].mean()
    step = max(1, n // n_blocks)
    for start in range(0, half - step + 1, step):
        if abs(x[start:half].mean() - second) <= precision:
            return start
    return None


def _z(confidence: float) -> float:
    from statistics import NormalDist

    return NormalDist().inv_cdf(0.5 + 0.5 * confidence)


class SummaryWriter:
    """Series of run results in the layout of the reference's summary.json.

    One call of ``append`` per run (one temperature / chemical potential /
    composition); each quantity keeps one list entry per run. Analysis
    functions follow ``monte_calculator/analysis_functions.cc:17-173``
    (heat capacity = var(E) N / (k T^2); susceptibilities = covariances
    N / (k T); matrices flattened column-major with component names
    "row,col"; "S" names the energy). Statistics carry the mean and the
    calculated precision = z(confidence) x the standard error corrected by the
    integrated autocorrelation time; with requested precisions, completion
    results add the convergence and equilibration fields. Mol compositions
    follow CASM composition axes when given (``composition_axes``: the
    system.json entry, e.g. Zr(2)Va(2-2a)O(2a) with a fixed Zr sublattice),
    else the standard axes (origin every site occupant 0, end member k every
    site occupant k).
    """

    def __init__(self, path: str, method: str, component_names, n_sites_per_uc: int,
                 comp_var_names=None, confidence: float = 0.95, requested_precision=None,
                 composition_axes=None):
        if method not in ("canonical", "semigrand_canonical"):
            raise ValueError(f"unknown method '{method}'")
        self.path = path
        self.method = method
        self.components = list(component_names)
        self.n_basis = int(n_sites_per_uc)
        self.comp_vars = list(comp_var_names or "abcdefgh"[: len(self.components) - 1])
        self.axes = None
        if composition_axes is not None:
            ax = composition_axes
            names = [k for k in "abcdefghijklmnopqrstuvwxyz" if k in ax]
            origin = np.asarray(ax["origin"], dtype=np.float64).reshape(-1)
            Q = np.stack([np.asarray(ax[k], dtype=np.float64).reshape(-1) - origin for k in names],
                         axis=1)
            self.components = list(ax["components"])
            self.comp_vars = names
            self.axes = (origin, Q)
        self.z = _z(confidence)
        self.requested = dict(requested_precision or {})
        self.data = {"analysis": {}, "completion_check_results": {}, "conditions": {},
                     "statistics": {}}

    # composition axes: origin = every site occupant 0, end member k = every
    # site occupant k (mol = origin + Q x)
    def _Q(self):
        if self.axes is not None:
            return self.axes[1]
        nc = len(self.comp_vars)
        Q = np.zeros((nc + 1, nc))
        for k in range(nc):
            Q[0, k] = -self.n_basis
            Q[k + 1, k] = self.n_basis
        return Q

    def _mol(self, x):
        if self.axes is not None:
            return self.axes[0] + self.axes[1] @ np.asarray(x, dtype=np.float64)
        origin = np.zeros(len(self.components))
        origin[0] = self.n_basis
        return origin + self._Q() @ np.asarray(x, dtype=np.float64)

    @staticmethod
    def _scalar(d, key, v):
        e = d.setdefault(key, {"shape": [], "value": []})
        e["value"].append(float(v))

    @staticmethod
    def _vector(d, key, names, vals, shape=None):
        e = d.setdefault(key, {"component_names": list(names),
                               "shape": list(shape or [len(names)])})
        for n, v in zip(names, np.asarray(vals, dtype=np.float64).ravel(order="F")):
            e.setdefault(n, []).append(float(v))

    @staticmethod
    def _matrix_names(rows, cols):
        return [f"{r},{c}" for c in cols for r in rows]

    def _stat(self, d, key, names, means, precs, converged):
        if names is None:
            e = d.setdefault(key, {"shape": [], "value": {"mean": [], "calculated_precision": []}})
            slots = [e["value"]]
        else:
            e = d.setdefault(key, {"component_names": list(names), "shape": [len(names)]})
            slots = [e.setdefault(n, {"mean": [], "calculated_precision": []}) for n in names]
        for k, c in enumerate(slots):
            c["mean"].append(float(np.atleast_1d(means)[k]))
            c["calculated_precision"].append(float(np.atleast_1d(precs)[k]))
            if converged is not None:
                c.setdefault("is_converged", []).append(bool(np.atleast_1d(converged)[k]))

    def append(self, *, temperature, n_unitcells, stats: dict, samples=None,
               param_chem_pot=None, elapsed_s=0.0, count=0):
        """Add one run. ``stats`` is ``ReplicaBatch.stats(i)`` (moments of the
        sampled tail); ``samples`` = (potential energy per unit cell, param
        composition) series of that tail, from ``ReplicaBatch.samples``."""
        from .stats import mean_error

        d = self.data
        nc = len(self.comp_vars)
        x = np.atleast_1d(np.asarray(stats["mean_comp"], dtype=np.float64))[:nc]
        mol = self._mol(x)
        Q = self._Q()
        norm = n_unitcells / (KB * temperature)

        self._scalar(d["conditions"], "temperature", temperature)
        if self.method == "semigrand_canonical":
            self._vector(d["conditions"], "param_chem_pot", self.comp_vars,
                         np.atleast_1d(param_chem_pot)[:nc])
        else:
            self._vector(d["conditions"], "param_composition", self.comp_vars, x)
            self._vector(d["conditions"], "mol_composition", self.components, mol)

        self._scalar(d["analysis"], "heat_capacity", stats["var_potential"] * norm / temperature)
        if self.method == "semigrand_canonical":
            cov = np.atleast_2d(stats["cov_comp"])[:nc, :nc]
            cex = np.atleast_1d(stats["cov_e_comp"])[:nc]
            self._vector(d["analysis"], "mol_susc",
                         self._matrix_names(self.components, self.components),
                         Q @ cov @ Q.T * norm, [len(self.components)] * 2)
            self._vector(d["analysis"], "param_susc",
                         self._matrix_names(self.comp_vars, self.comp_vars), cov * norm, [nc, nc])
            self._vector(d["analysis"], "mol_thermochem_susc",
                         self._matrix_names(["S"], self.components),
                         (Q @ cex * norm).reshape(1, -1), [1, len(self.components)])
            self._vector(d["analysis"], "param_thermochem_susc",
                         self._matrix_names(["S"], self.comp_vars),
                         (cex * norm).reshape(1, -1), [1, nc])

        prec_e, prec_x = 0.0, np.zeros(nc)
        eq_at = 0
        if samples is not None:
            pot, comp = samples
            prec_e = self.z * mean_error(pot)[1]
            comp = np.asarray(comp, dtype=np.float64).reshape(len(pot), -1)
            if self.method == "semigrand_canonical":
                prec_x = np.array([self.z * mean_error(comp[:, k])[1] for k in range(nc)])
        prec_mol = np.abs(Q) @ prec_x
        conv = {}
        if self.requested:
            req_e = self.requested.get("potential_energy")
            req_x = self.requested.get("param_composition")
            conv["potential_energy"] = None if req_e is None else prec_e <= req_e
            conv["param_composition"] = None if req_x is None else prec_x <= req_x
            if samples is not None:
                checks = []
                if req_e is not None:
                    checks.append(equilibration_index(samples[0], req_e))
                if req_x is not None:
                    comp = np.asarray(samples[1], dtype=np.float64).reshape(len(samples[0]), -1)
                    checks += [equilibration_index(comp[:, k], req_x) for k in range(nc)]
                eq_at = None if any(c is None for c in checks) else max(checks, default=0)
        self._stat(d["statistics"], "potential_energy", None, stats["mean_potential"], prec_e,
                   conv.get("potential_energy"))
        self._stat(d["statistics"], "clex.formation_energy", None, stats["mean_formation"], prec_e,
                   None)
        self._stat(d["statistics"], "param_composition", self.comp_vars, x, prec_x,
                   conv.get("param_composition"))
        self._stat(d["statistics"], "mol_composition", self.components, mol, prec_mol, None)

        cc = d["completion_check_results"]
        rows = [("N_samples", int(stats["n_samples"])),
                ("N_samples_for_statistics", int(stats["n_samples"])),
                ("acceptance_rate", stats["n_accepted"] / max(1, stats["n_proposed"])),
                ("count", int(count)), ("elapsed_clocktime", float(elapsed_s))]
        if self.requested:
            flags = [v for v in conv.values() if v is not None]
            rows += [("N_samples_for_all_to_equilibrate", -1 if eq_at is None else int(eq_at)),
                     ("all_converged", bool(all(np.all(v) for v in flags))),
                     ("all_equilibrated", eq_at is not None)]
        for k, v in rows:
            cc.setdefault(k, []).append(v)

    def write(self):
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        with open(self.path, "w") as f:
            json.dump(self.data, f, indent=1)
