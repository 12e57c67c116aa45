"""Host-side mirror of the ``libcasm.clexmonte`` calculator interface for the
Metropolis hot path, driving the CUDA library through its C ABI.

Reference interface (paths relative to the CASMcode_clexmonte tree):

* ``MonteCalculator(method, system, params)`` with
  ``method in {"canonical", "semigrand_canonical"}``
  (``python/libcasm/clexmonte/_MonteCalculator.py:24-95``);
* ``MonteCalculator.set_state_and_potential``, ``.potential``,
  ``.run_fixture`` (``python/src/clexmonte_monte_calculator.cpp:2106-2145``);
* ``MontePotential(calculator, state)`` with ``per_supercell``,
  ``per_unitcell`` and ``occ_delta_per_supercell(linear_site_index, new_occ)``
  (``python/src/clexmonte_monte_calculator.cpp:694-750``);
* ``MonteCarloState(configuration, conditions)`` with conditions
  ``temperature`` and ``param_chem_pot`` (SGC) or ``param_composition``
  (canonical) (``python/tests/semigrand_canonical/
  test_SemiGrandCanonicalCalculator.py:23-31``);
* analyses ``heat_capacity``, ``param_susc`` and ``param_thermochem_susc``
  (``src/casm/clexmonte/monte_calculator/analysis_functions.cc:17-173``).

Errors are raised as exceptions with the library's message, as the
reference's calculators throw ``std::runtime_error``
(``CanonicalCalculator.cc:380-390``).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import CEM_CANONICAL, CEM_SEMIGRAND_CANONICAL, check, ptr
from .system import KB, ClusterExpansion, param_RT_of, system_arrays

METHODS = {"semigrand_canonical": CEM_SEMIGRAND_CANONICAL, "canonical": CEM_CANONICAL}


class System:
    """A cluster expansion uploaded to the GPU (the role of
    ``libcasm.clexmonte.System`` for the formation-energy clex)."""

    def __init__(self, ce: ClusterExpansion):
        self.ce = ce
        self.lib = _lib.load()
        self.arrays = system_arrays(ce)
        desc, self._keep = _lib.make_desc(self.arrays)
        h = C.c_void_p()
        check(self.lib.cem_system_create(C.byref(desc), C.byref(h)))
        self.handle = h
        self.n_occ = ce.prim.n_occ
        self.n_funcs = ce.n_funcs
        self.RT = param_RT_of(ce)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.cem_system_destroy(h)
            self.handle = None


class ReplicaBatch:
    """Replicas of one ensemble resident on the GPU (occupations in HBM)."""

    def __init__(self, system: System, ensemble: str, L):
        """``L``: per replica, the three edge lengths of a diagonal supercell
        or a 3 x 3 ``transformation_matrix_to_super`` (columns = supercell
        lattice vectors in prim cell coordinates). Non-diagonal supercells
        number their unit cells on the matrix's lower-triangular Hermite normal
        form H (cell i + H00 (j + H11 k)) and support the exact paths (energy,
        delta, replay, n-fold way, enforce_composition, state transfer) and
        semi-grand canonical runs; canonical runs need a diagonal supercell."""
        self.system = system
        self.lib = system.lib
        self.ensemble = ensemble
        h = C.c_void_p()
        if any(np.ndim(l) == 2 for l in L):
            self.L = [tuple(tuple(int(x) for x in row) for row in np.asarray(l))
                      if np.ndim(l) == 2 else tuple(int(x) for x in l) for l in L]
            T = np.zeros((len(L), 3, 3), dtype=np.int64)
            for r, l in enumerate(self.L):
                T[r] = np.asarray(l) if np.ndim(l) == 2 else np.diag(l)
            T = np.ascontiguousarray(T.reshape(-1))
            check(self.lib.cem_replicas_create_supercells(system.handle, len(self.L), ptr(T),
                                                          METHODS[ensemble], C.byref(h)))
        else:
            self.L = [tuple(int(x) for x in l) for l in L]
            Ls = np.ascontiguousarray(np.array(self.L, dtype=np.int32).reshape(-1))
            check(self.lib.cem_replicas_create(system.handle, len(self.L), _lib.iptr(Ls),
                                               METHODS[ensemble], C.byref(h)))
        self.handle = h
        self.n = len(self.L)
        ns = C.c_int64()
        sizes = []
        for i in range(self.n):
            check(self.lib.cem_n_sites(h, i, C.byref(ns)))
            sizes.append(ns.value)
        self.n_sites = np.array(sizes, dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.n_sites)])

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.cem_replicas_destroy(h)
            self.handle = None
        for hp in getattr(self, "_pinned", []):
            self.lib.cem_host_free(hp)
        self._pinned = []

    def set_conditions(self, i: int, temperature: float, param_chem_pot=None):
        mu = None
        if param_chem_pot is not None:
            mu = np.ascontiguousarray(param_chem_pot, dtype=np.float64)
        check(self.lib.cem_set_conditions(self.handle, i, float(temperature),
                                          None if mu is None else _lib.dptr(mu)))

    def set_seed(self, i: int, seed: int):
        check(self.lib.cem_set_seed(self.handle, i, int(seed) & (2**64 - 1)))

    def set_occupation(self, i: int, occ):
        occ = np.ascontiguousarray(occ, dtype=np.int8)
        if occ.size != self.n_sites[i]:
            raise ValueError(f"occupation has {occ.size} sites, expected {self.n_sites[i]}")
        check(self.lib.cem_set_occupation(self.handle, i, ptr(occ)))

    def get_occupation(self, i: int) -> np.ndarray:
        out = np.zeros(self.n_sites[i], dtype=np.int8)
        check(self.lib.cem_get_occupation(self.handle, i, ptr(out)))
        return out

    def set_occupation_all(self, packed: np.ndarray):
        assert packed.dtype == np.int8 and packed.size == self.offsets[-1]
        check(self.lib.cem_set_occupation_all(self.handle, ptr(packed)))

    def get_occupation_all(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros(self.offsets[-1], dtype=np.int8)
        check(self.lib.cem_get_occupation_all(self.handle, ptr(out)))
        return out

    def energy(self, i: int):
        e = C.c_double()
        counts = np.zeros(self.system.n_funcs, dtype=np.int64)
        check(self.lib.cem_energy(self.handle, i, C.byref(e), ptr(counts)))
        return e.value, counts

    def delta(self, i: int, sites, new_occ, potential: bool = False):
        sites = np.ascontiguousarray(np.atleast_2d(sites), dtype=np.int64)
        new_occ = np.ascontiguousarray(np.atleast_2d(new_occ), dtype=np.int32)
        if sites.shape != new_occ.shape:
            raise ValueError("sites and new_occ must have the same shape")
        n_events, k = sites.shape
        dE = np.zeros(n_events)
        dc = np.zeros((n_events, self.system.n_funcs), dtype=np.int64)
        check(self.lib.cem_delta_energy(self.handle, i, n_events, k, ptr(sites), ptr(new_occ),
                                        int(bool(potential)), ptr(dE), ptr(dc)))
        return dE, dc

    def replay(self, i: int, mt_seed: int, n_steps: int, record: bool = True):
        acc = np.zeros(n_steps, dtype=np.uint8) if record else None
        de = np.zeros(n_steps) if record else None
        sites = np.zeros((n_steps, 2), dtype=np.int64) if record else None
        n_acc = C.c_int64()
        draws = C.c_uint64()
        check(self.lib.cem_replay(self.handle, i, int(mt_seed), int(n_steps), ptr(acc), ptr(de),
                                  ptr(sites), C.byref(n_acc), C.byref(draws)))
        return dict(accept=acc, dE=de, sites=sites, n_accept=n_acc.value, draws=draws.value)

    def enforce_composition(self, target_mol, mt_seed: int) -> np.ndarray:
        """Greedy flips toward ``target_mol`` (species per unit cell; one row
        per replica, or one row for all); replica i draws from
        std::mt19937_64(mt_seed + i). Returns the flips per replica."""
        t = np.asarray(target_mol, dtype=np.float64)
        n = len(self.L)
        if t.ndim == 1:
            t = np.tile(t, (n, 1))
        if t.shape != (n, self.system.n_occ):
            raise ValueError(f"target_mol must have {self.system.n_occ} components per replica")
        t = np.ascontiguousarray(t)
        flips = np.zeros(n, dtype=np.int64)
        check(self.lib.cem_enforce_composition(self.handle, t.ctypes.data_as(_lib._dp),
                                               int(mt_seed), flips.ctypes.data_as(C.POINTER(C.c_int64))))
        return flips

    def nfold_run(self, n_events: int, n_equil: int = 0, record: int = 0):
        """n-fold way (rejection-free) events on every replica (semi-grand
        canonical). Statistics become residence-time weighted. With
        ``record`` > 0 returns the first ``record`` events of each replica:
        site, new occupant and residence weight arrays of shape (n, record)."""
        n = len(self.L)
        site = np.zeros((n, record), dtype=np.int64) if record else None
        occ = np.zeros((n, record), dtype=np.int32) if record else None
        dt = np.zeros((n, record)) if record else None
        check(self.lib.cem_nfold_run(self.handle, int(n_events), int(n_equil), int(record),
                                     ptr(site), ptr(occ), ptr(dt)))
        return dict(site=site, occ=occ, dt=dt) if record else None

    def run(self, n_passes: int, n_equil: int = 0, record_samples: bool = False):
        check(self.lib.cem_run(self.handle, int(n_passes), int(n_equil), int(bool(record_samples))))

    def step_async(self, host_in: np.ndarray, host_out: np.ndarray, n_passes: int = 1):
        """Copy the packed occupations in, run ``n_passes`` passes, copy them
        out, as one CUDA graph on the batch's stream (page-locked int8
        buffers of all sites, e.g. from ``pinned_buffer``)."""
        check(self.lib.cem_step_async(self.handle, ptr(host_in), ptr(host_out), int(n_passes)))

    def pinned_buffer(self) -> np.ndarray:
        """Page-locked int8 buffer of all replicas' sites (freed with the batch)."""
        nbytes = int(self.offsets[-1])
        hp = C.c_void_p()
        check(self.lib.cem_host_alloc(nbytes, C.byref(hp)))
        self._pinned = getattr(self, "_pinned", []) + [hp]
        return np.ctypeslib.as_array((C.c_int8 * nbytes).from_address(hp.value))

    def autotune(self, trial_passes: int = 20) -> dict:
        """Pick the fastest launch schedule (threads per replica, replica
        order) by timing trial passes from the current state; the state is
        restored afterwards."""
        ms = C.c_double()
        check(self.lib.cem_autotune(self.handle, int(trial_passes), C.byref(ms)))
        return dict(threads=self.get_option("threads"), cta_order=self.get_option("cta_order"),
                    trial_ms=ms.value)

    def set_option(self, key: str, value: int):
        check(self.lib.cem_set_option(self.handle, key.encode(), int(value)))

    def get_option(self, key: str) -> int:
        v = C.c_int64()
        check(self.lib.cem_get_option(self.handle, key.encode(), C.byref(v)))
        return v.value

    def synchronize(self) -> bool:
        """Wait for the batch's work; True when the last run was stopped early
        by ``request_stop``."""
        rc = self.lib.cem_synchronize(self.handle)
        if rc == _lib.CEM_STOPPED:
            return True
        check(rc)
        return False

    def request_stop(self):
        """Ask the run in flight to stop at its next pass boundary (may be
        called from another thread while ``synchronize`` waits)."""
        check(self.lib.cem_request_stop(self.handle))

    def get_state(self, i: int):
        """(occupation, state bytes) checkpoint of replica i."""
        nb = C.c_int64()
        check(self.lib.cem_state_bytes(self.handle, C.byref(nb)))
        occ = np.zeros(self.n_sites[i], dtype=np.int8)
        st = np.zeros(nb.value, dtype=np.uint8)
        check(self.lib.cem_get_state(self.handle, i, ptr(occ), ptr(st)))
        return occ, st

    def set_state(self, i: int, occ, state):
        occ = np.ascontiguousarray(occ, dtype=np.int8)
        state = np.ascontiguousarray(state, dtype=np.uint8)
        check(self.lib.cem_set_state(self.handle, i, ptr(occ), ptr(state)))

    def order_samples(self, i: int, capacity: int) -> np.ndarray:
        op = np.zeros(capacity)
        n = C.c_int64()
        check(self.lib.cem_get_order_samples(self.handle, i, ptr(op), int(capacity), C.byref(n)))
        return op[: n.value]

    # ---- learned proposal
    def learned_features(self, i: int):
        n = int(self.n_sites[i])
        X = np.zeros((n, LearnedProposal.N_IN), dtype=np.int8)
        t = np.zeros(n, dtype=np.float32)
        check(self.lib.cem_learned_features(self.handle, i, ptr(X), ptr(t)))
        return X, t

    def learned_run(self, proposal, n_passes: int, n_equil: int = 0, record_samples: bool = False):
        h = None if proposal is None else proposal.handle
        check(self.lib.cem_learned_run(self.handle, h, int(n_passes), int(n_equil),
                                       int(bool(record_samples))))

    GROUP_WEIGHTS = {"uniform": 0, "network": 1, "exact": 2}

    def learned_group_run(self, proposal, n_passes: int, n_equil: int = 0,
                          record_samples: bool = False, weights: str | None = None,
                          rounds: int = 2, local_substeps: int = 4):
        """Learned group sweep (cem_learned_group_run): ``weights`` is
        "network" (default when ``proposal`` is given), "uniform" or "exact"
        (the locally balanced weights the network is trained toward). The
        defaults (2 swap rounds per group, 4 nearest-neighbour sub-steps per
        pass) are the fastest measured on the L1_2 workload: more rounds or
        sub-steps left tau_int unchanged and cost time."""
        if weights is None:
            weights = "uniform" if proposal is None else "network"
        mode = self.GROUP_WEIGHTS[weights]
        h = None if proposal is None else proposal.handle
        check(self.lib.cem_learned_group_run(self.handle, h, mode, int(rounds), int(local_substeps),
                                             int(n_passes), int(n_equil), int(bool(record_samples))))

    def learned_samples(self, i: int, capacity: int):
        e = np.zeros(capacity)
        op = np.zeros(capacity)
        n = C.c_int64()
        check(self.lib.cem_learned_samples(self.handle, i, ptr(e), ptr(op), int(capacity),
                                           C.byref(n)))
        return e[: n.value], op[: n.value]

    def kernel_ms(self) -> float:
        ms = C.c_double()
        check(self.lib.cem_last_kernel_ms(self.handle, C.byref(ms)))
        return ms.value

    def reset_stats(self):
        check(self.lib.cem_reset_stats(self.handle))

    def stats(self, i: int) -> dict:
        s = _lib.Stats()
        check(self.lib.cem_get_stats(self.handle, i, C.byref(s)))
        nc = self.system.n_occ - 1
        return dict(
            n_samples=s.n_samples, mean_potential=s.mean_potential,
            var_potential=s.var_potential, mean_formation=s.mean_formation,
            mean_comp=np.array(s.mean_comp[:nc]),
            cov_comp=np.array(s.cov_comp[:]).reshape(3, 3)[:nc, :nc],
            cov_e_comp=np.array(s.cov_e_comp[:nc]), energy=s.energy,
            n_proposed=s.n_proposed, n_accepted=s.n_accepted, passes=s.passes,
        )

    def samples(self, i: int, capacity: int):
        nc = self.system.n_occ - 1
        pot = np.zeros(capacity)
        comp = np.zeros((capacity, nc))
        n = C.c_int64()
        check(self.lib.cem_get_samples(self.handle, i, ptr(pot), ptr(comp), int(capacity),
                                       C.byref(n)))
        return pot[: n.value], comp[: n.value]


def mol_composition(system: "System", param_composition) -> np.ndarray:
    """Species per unit cell for a parametric composition on the system's
    composition axes (origin: every site occupant 0; mol = origin + Q x with
    Q the pseudo-inverse of the axes' R^T)."""
    nb = system.ce.prim.n_basis
    x = np.atleast_1d(np.asarray(param_composition, dtype=np.float64))
    if x.size != system.n_occ - 1:
        raise ValueError(f"param_composition must have {system.n_occ - 1} components")
    origin = np.zeros(system.n_occ)
    origin[0] = nb
    return origin + np.linalg.pinv(system.RT) @ x


def enforce_composition(state: "MonteCarloState", target_mol_composition, system: "System",
                        seed: int = 0) -> int:
    """Apply semi-grand canonical flips to ``state.occupation`` until no flip
    brings its composition closer to ``target_mol_composition`` (species per
    unit cell), on the GPU; the draws follow std::mt19937_64(seed) as the
    reference's ``enforce_composition`` (python/src/clexmonte_functions.cpp:
    71-140) does with its engine. Returns the number of flips."""
    t = np.asarray(target_mol_composition, dtype=np.float64)
    if t.shape != (system.n_occ,):
        raise ValueError(
            f"Error in enforce_composition: mismatch target_mol_composition={t.tolist()}, "
            f"expected {system.n_occ} components")
    b = ReplicaBatch(system, "canonical", [_supercell_key(state.L)])
    b.set_occupation(0, state.occupation)
    n = int(b.enforce_composition(t, seed)[0])
    state.occupation[:] = b.get_occupation(0)
    return n


def supercell_hnf(transformation_matrix_to_super) -> np.ndarray:
    """Lower-triangular Hermite normal form the library numbers a supercell's
    unit cells on (cell (i, j, k), 0 <= i < H00, 0 <= j < H11, 0 <= k < H22, is
    unit cell i + H00 (j + H11 k)); no device needed."""
    t = np.ascontiguousarray(np.asarray(transformation_matrix_to_super, dtype=np.int64).reshape(9))
    h = np.zeros(9, dtype=np.int64)
    check(_lib.load().cem_supercell_hnf(ptr(t), ptr(h)))
    return h.reshape(3, 3)


def _cell_index(H, i, j, k):
    """Unit cells (i, j, k) (arrays) reduced into the Hermite-normal-form box of H."""
    L0, L1, L2 = int(H[0, 0]), int(H[1, 1]), int(H[2, 2])
    q = np.floor_divide(i, L0)
    i, j, k = i - q * L0, j - q * int(H[1, 0]), k - q * int(H[2, 0])
    q = np.floor_divide(j, L1)
    j, k = j - q * L1, k - q * int(H[2, 1])
    return i + L0 * (j + L1 * np.mod(k, L2))


def scale_supercell(transformation_matrix_to_super, dirs: str = "abc",
                    min_volume: int = 1000) -> np.ndarray:
    """T M with M diagonal: every axis named in ``dirs`` grows by one cell per
    step until det(T M) >= min_volume (the reference's scale_supercell,
    python/libcasm/clexmonte/_auto_configuration.py:19-58)."""
    T = np.asarray(transformation_matrix_to_super, dtype=np.int64).reshape(3, 3)
    if not any(c in dirs for c in "abc"):
        raise ValueError("dirs must name at least one of 'a', 'b', 'c'")
    M = np.eye(3, dtype=np.int64)
    while int(round(np.linalg.det(T @ M))) < min_volume:
        for a, c in enumerate("abc"):
            if c in dirs:
                M[a, a] += 1
    return T @ M


def tile_motif(motif_occupation, motif_T, T, n_sublat: int) -> np.ndarray:
    """Occupation of supercell T filled with a motif (its occupation on
    supercell motif_T, both in this library's site order); T must be a
    supercell of motif_T."""
    motif_T = np.asarray(motif_T, dtype=np.int64).reshape(3, 3)
    T = np.asarray(T, dtype=np.int64).reshape(3, 3)
    N = np.linalg.solve(motif_T.astype(float), T.astype(float))
    if not np.allclose(N, np.round(N), atol=1e-9):
        raise ValueError("Failed to tile motif into supercell")
    H, Hm = supercell_hnf(T), supercell_hnf(motif_T)
    k, j, i = np.meshgrid(np.arange(H[2, 2]), np.arange(H[1, 1]), np.arange(H[0, 0]), indexing="ij")
    cell = _cell_index(Hm, i.ravel(), j.ravel(), k.ravel())  # motif cell of each cell of T
    m_uc, n_uc = int(np.prod(np.diag(Hm))), int(np.prod(np.diag(H)))
    occ = np.asarray(motif_occupation, dtype=np.int8).reshape(n_sublat, m_uc)
    return np.ascontiguousarray(occ[:, cell].reshape(n_sublat * n_uc))


def match_composition(state: "MonteCarloState", system: "System") -> None:
    """Set the state's ``mol_composition`` (species per unit cell) and
    ``param_composition`` conditions to its occupation's composition (the
    reference calculators' "match.composition" modifier)."""
    occ = np.asarray(state.occupation)
    n_uc = _n_unitcells(state.L)
    counts = np.bincount(occ, minlength=system.n_occ).astype(np.float64)
    dn = counts.copy()
    dn[0] -= occ.size
    state.conditions["mol_composition"] = counts / n_uc
    state.conditions["param_composition"] = system.RT @ dn / n_uc


def make_canonical_initial_state(calculator: "MonteCalculator", conditions: dict,
                                 dirs: str = "abc", min_volume: int = 1000,
                                 transformation_matrix_to_super=None, motif=None,
                                 seed: int = 0):
    """Initial state for canonical Monte Carlo (the reference's
    make_canonical_initial_state, _auto_configuration.py:496-640): the motif
    (``None``: every site occupant 0 in the prim cell; else a pair
    (occupation, transformation_matrix_to_super) in this library's site order)
    is tiled into scale_supercell(transformation_matrix_to_super or the
    motif's supercell, dirs, min_volume); the composition of ``conditions``
    (``mol_composition`` or ``param_composition``; neither: the motif's) is
    enforced by greedy flips drawn from std::mt19937_64(seed); the composition
    conditions are then matched to the result. The reference also searches the
    motif's orientations under the prim factor group for the lowest potential;
    here the motif is tiled as given. Returns (state, motif)."""
    system = calculator.system
    nb = system.ce.prim.n_basis
    if motif is None:
        motif = (np.zeros(nb, dtype=np.int8), np.eye(3, dtype=np.int64))
    m_occ, m_T = np.asarray(motif[0], dtype=np.int8), np.asarray(motif[1], dtype=np.int64)
    conditions = dict(conditions)
    if "mol_composition" in conditions:
        target = np.asarray(conditions["mol_composition"], dtype=np.float64)
    elif "param_composition" in conditions:
        target = mol_composition(system, conditions["param_composition"])
    else:
        counts = np.bincount(m_occ, minlength=system.n_occ).astype(np.float64)
        target = counts / (m_occ.size // nb)
    T0 = m_T if transformation_matrix_to_super is None else transformation_matrix_to_super
    T = scale_supercell(T0, dirs, min_volume)
    occ = tile_motif(m_occ, m_T, T, nb)
    L = tuple(int(T[a, a]) for a in range(3)) if np.count_nonzero(T - np.diag(np.diag(T))) == 0 \
        and np.all(np.diag(T) > 0) else T
    state = MonteCarloState(occupation=occ, L=L, conditions=conditions)
    enforce_composition(state, target, system, seed)
    match_composition(state, system)
    return state, motif


class LearnedProposal:
    """The proposal network (42 neighbour occupants -> 64 -> 64 -> 1 logit,
    bf16 parameters) on the GPU. A site holding A is weighted exp(z), one
    holding B exp(-z)."""

    N_IN = 42
    N_HIDDEN = 64

    def __init__(self, seed: int = 0):
        self.lib = _lib.load()
        ni, nh, npar = C.c_int(), C.c_int(), C.c_int()
        check(self.lib.cem_mlp_info(C.byref(ni), C.byref(nh), C.byref(npar)))
        self.n_params = npar.value
        h = C.c_void_p()
        check(self.lib.cem_mlp_create(int(seed), C.byref(h)))
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.cem_mlp_destroy(h)
            self.handle = None

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        check(self.lib.cem_mlp_get_params(self.handle, ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        check(self.lib.cem_mlp_set_params(self.handle, ptr(p)))

    def forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.int8)
        z = np.zeros(len(X), dtype=np.float32)
        check(self.lib.cem_mlp_forward(self.handle, len(X), ptr(X), ptr(z)))
        return z

    def forward_tc(self, X) -> np.ndarray:
        """Logits on the tensor-core (tcgen05) path of the group sweep."""
        X = np.ascontiguousarray(X, dtype=np.int8)
        z = np.zeros(len(X), dtype=np.float32)
        check(self.lib.cem_mlp_forward_tc(self.handle, len(X), ptr(X), ptr(z)))
        return z

    def gradient(self, X, t):
        X = np.ascontiguousarray(X, dtype=np.int8)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double()
        check(self.lib.cem_mlp_gradient(self.handle, len(X), ptr(X), ptr(t), ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, X, t, epochs=5, batch=4096, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.int8)
        t = np.ascontiguousarray(t, dtype=np.float32)
        losses = np.zeros(epochs)
        check(self.lib.cem_mlp_train(self.handle, len(X), ptr(X), ptr(t), int(epochs), int(batch),
                                     float(lr), int(seed), ptr(losses)))
        return losses


def _supercell_key(L):
    """A supercell as given: three edge lengths, or a 3 x 3
    ``transformation_matrix_to_super`` (tuple of rows)."""
    if np.ndim(L) == 2:
        return tuple(tuple(int(x) for x in row) for row in np.asarray(L))
    return tuple(int(x) for x in L)


def _n_unitcells(L) -> int:
    if np.ndim(L) == 2:
        return abs(int(round(np.linalg.det(np.asarray(L, dtype=float)))))
    return int(L[0] * L[1] * L[2])


@dataclass
class MonteCarloState:
    """Occupation of a supercell plus thermodynamic conditions. ``L``: three
    edge lengths of a diagonal supercell, or a 3 x 3
    ``transformation_matrix_to_super`` (non-diagonal supercells support the
    potential, the replay, composition enforcement and semi-grand canonical
    runs; canonical runs need a diagonal supercell)."""

    occupation: np.ndarray
    L: tuple
    conditions: dict = field(default_factory=dict)


@dataclass
class SamplingFixtureParams:
    """Sampling fixture: one sample per pass (a sampling period of one pass
    in the reference's fixtures) after ``n_equil`` unsampled passes.

    Without ``requested_precision`` the run has a fixed length of
    ``n_passes`` passes. With it (absolute precisions, e.g.
    ``{"potential_energy": 0.001}`` as the reference's default canonical
    fixture, CanonicalCalculator.cc:261-270, or also "param_composition"),
    the run stops at the first completion check, every ``check_period``
    sampled passes, at which every requested quantity is equilibrated (the
    two-partition test of ``casm_io.equilibration_index``) and its calculated
    precision over the equilibrated tail, z(confidence) x the standard error
    corrected by the integrated autocorrelation time, is within the request;
    ``n_passes`` is then the cutoff (maximum passes) and ``min_samples`` the
    fewest samples checked."""

    n_passes: int = 1000
    n_equil: int = 200
    record_samples: bool = True
    requested_precision: dict | None = None
    check_period: int = 100
    min_samples: int = 100
    confidence: float = 0.95


def _tail_moments(e, x) -> dict:
    """The moments ``ReplicaBatch.stats`` reports, over given samples of the
    potential energy per unit cell and param composition."""
    e = np.asarray(e, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64).reshape(e.size, -1)
    de = e - e.mean()
    dx = x - x.mean(axis=0)
    return dict(n_samples=float(e.size), mean_potential=float(e.mean()),
                var_potential=float(np.mean(de * de)), mean_comp=x.mean(axis=0),
                cov_comp=(dx.T @ dx) / e.size, cov_e_comp=(dx.T @ de) / e.size)


def analyses(stats: dict, temperature: float, n_unitcells: int) -> dict:
    """Heat capacity and susceptibilities per unit cell from the sampled
    moments (analysis_functions.cc:17-173; variances and covariances are
    population moments of the sampled tail)."""
    beta_norm = KB * temperature
    return dict(
        heat_capacity=stats["var_potential"] * n_unitcells / (KB * temperature * temperature),
        param_susc=stats["cov_comp"] * n_unitcells / beta_norm,
        param_thermochem_susc=stats["cov_e_comp"] * n_unitcells / beta_norm,
    )


class MontePotential:
    """Potential of one state: canonical (formation energy) or semi-grand
    canonical (formation energy - n_unitcells * param_chem_pot . x)."""

    def __init__(self, calculator: "MonteCalculator", state: MonteCarloState):
        self.calculator = calculator
        self.state = state
        calculator._bind(state)

    @property
    def _batch(self) -> ReplicaBatch:
        return self.calculator._batch

    def _n_uc(self) -> int:
        return _n_unitcells(self.state.L)

    def per_supercell(self) -> float:
        e, _ = self._batch.energy(0)
        if self.calculator.method == "semigrand_canonical":
            occ = np.asarray(self.state.occupation)
            n_sites = occ.size
            counts = np.bincount(occ, minlength=self.calculator.system.n_occ).astype(float)
            dn = counts.copy()
            dn[0] -= n_sites
            x = self.calculator.system.RT @ dn / self._n_uc()
            mu = np.asarray(self.state.conditions["param_chem_pot"], dtype=float)
            e -= self._n_uc() * float(mu @ x)
        return e

    def per_unitcell(self) -> float:
        return self.per_supercell() / self._n_uc()

    def occ_delta_per_supercell(self, linear_site_index, new_occ) -> float:
        dE, _ = self._batch.delta(
            0, np.asarray(linear_site_index).reshape(1, -1), np.asarray(new_occ).reshape(1, -1),
            potential=self.calculator.method == "semigrand_canonical",
        )
        return float(dE[0])


class MonteCalculator:
    """GPU Metropolis calculator for ``method`` in {"canonical",
    "semigrand_canonical"}. ``params`` may hold ``seed`` (counter-based
    stream of the parallel sweep)."""

    def __init__(self, method: str, system: System, params: dict | None = None):
        if method not in METHODS:
            raise ValueError(f"Unknown method: '{method}'. Options are: {list(METHODS)}")
        self.method = method
        self.system = system
        self.params = dict(params or {})
        self._batch: ReplicaBatch | None = None
        self._state: MonteCarloState | None = None
        self.potential: MontePotential | None = None

    def _check_conditions(self, state: MonteCarloState):
        c = state.conditions
        if "temperature" not in c:
            raise ValueError("state conditions need 'temperature'")
        if self.method == "semigrand_canonical" and "param_chem_pot" not in c:
            raise ValueError("semi-grand canonical states need 'param_chem_pot'")

    def _bind(self, state: MonteCarloState):
        self._check_conditions(state)
        L = _supercell_key(state.L)
        if self._batch is None or self._batch.L[0] != L:
            self._batch = ReplicaBatch(self.system, self.method, [L])
        b = self._batch
        mu = state.conditions.get("param_chem_pot") if self.method == "semigrand_canonical" else None
        b.set_conditions(0, state.conditions["temperature"], mu)
        b.set_seed(0, int(self.params.get("seed", 0x5EED)))
        b.set_occupation(0, state.occupation)
        self._state = state

    def set_state_and_potential(self, state: MonteCarloState):
        self.potential = MontePotential(self, state)
        return self.potential

    def replay(self, state: MonteCarloState, mt_seed: int, n_steps: int, record: bool = True):
        """Sequential reference-order Metropolis steps on the GPU; updates
        ``state.occupation``."""
        self._bind(state)
        out = self._batch.replay(0, mt_seed, n_steps, record)
        state.occupation[:] = self._batch.get_occupation(0)
        return out

    def run_fixture(self, state: MonteCarloState, sampling_fixture_params: SamplingFixtureParams):
        """Parallel Metropolis run; updates ``state.occupation`` and returns
        the sampled statistics and analyses (with requested precisions, also
        the completion-check results: ``count``, ``is_converged`` per
        quantity, ``N_samples_for_equilibration``)."""
        p = sampling_fixture_params
        self._bind(state)
        b = self._batch
        n_uc = _n_unitcells(state.L)
        T = state.conditions["temperature"]
        if not p.requested_precision:
            b.run(p.n_passes, p.n_equil, p.record_samples)
            st = b.stats(0)
            state.occupation[:] = b.get_occupation(0)
            res = dict(st)
            res.update(analyses(st, T, n_uc))
            if p.record_samples:
                res["samples_potential"], res["samples_comp"] = b.samples(0, p.n_passes)
            return res
        return self._run_to_precision(state, p, n_uc, T)

    def _run_to_precision(self, state, p, n_uc, T):
        """Completion-checked run (CanonicalCalculator.cc:261-270): chunks of
        ``check_period`` sampled passes until every requested quantity is
        equilibrated and within its requested absolute precision, or the
        cutoff of ``n_passes`` passes."""
        from . import casm_io
        from .stats import mean_error

        b = self._batch
        z = casm_io._z(p.confidence)
        req = dict(p.requested_precision)
        unknown = set(req) - {"potential_energy", "param_composition"}
        if unknown:
            raise ValueError(f"requested precision for unknown quantities: {sorted(unknown)}")
        if p.n_equil > 0:
            b.run(p.n_equil, p.n_equil)  # unsampled passes
        b.reset_stats()
        pots, comps = [], []
        count = p.n_equil
        max_count = max(p.n_passes, p.n_equil + 1)
        done = False
        conv = {}
        eq_at = None
        while not done and count < max_count:
            chunk = min(p.check_period, max_count - count)
            b.run(chunk, 0, record_samples=True)
            pot, comp = b.samples(0, chunk)
            pots.append(pot)
            comps.append(comp)
            count += chunk
            e = np.concatenate(pots)
            x = np.concatenate(comps).reshape(e.size, -1)
            if e.size < p.min_samples:
                continue
            series = []
            if "potential_energy" in req:
                series.append(("potential_energy", e, req["potential_energy"]))
            if "param_composition" in req:
                series += [("param_composition", x[:, k], req["param_composition"])
                           for k in range(x.shape[1])]
            starts = [casm_io.equilibration_index(v, r) for _, v, r in series]
            if any(s0 is None for s0 in starts):
                continue
            eq_at = max(starts)
            conv = {}
            for (name, v, r) in series:
                prec = z * mean_error(v[eq_at:])[1]
                conv[name] = conv.get(name, True) and bool(prec <= r)
            done = all(conv.values())
        state.occupation[:] = b.get_occupation(0)
        e = np.concatenate(pots)
        x = np.concatenate(comps).reshape(e.size, -1)
        s0 = eq_at if eq_at is not None else 0
        st = dict(b.stats(0))
        st.update(_tail_moments(e[s0:], x[s0:]))
        st["mean_formation"] = st["mean_potential"]
        if self.method == "semigrand_canonical":  # E_f = E_pot + mu . x per unit cell
            mu = np.atleast_1d(np.asarray(state.conditions["param_chem_pot"], dtype=float))
            st["mean_formation"] = st["mean_potential"] + float(mu @ st["mean_comp"])
        res = dict(st)
        res.update(analyses(st, T, n_uc))
        res.update(count=count, is_converged=conv, all_converged=bool(done),
                   N_samples_for_equilibration=None if eq_at is None else int(eq_at),
                   requested_precision=req)
        res["samples_potential"], res["samples_comp"] = e[s0:], x[s0:]
        return res
