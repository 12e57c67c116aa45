"""ctypes wrapper around the CPU FP64 oracle (``oracle/cem_oracle.cc``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the comparison. The product library
never imports this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcem_oracle.so")


def build_oracle(force: bool = False) -> str:
    """Compile the oracle with g++ (no cmake). Returns the library path."""
    src = os.path.join(HERE, "cem_oracle.cc")
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        cmd = [
            "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
            "-o", LIB, src, "-lpthread",
        ]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB)
        P = C.c_void_p
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
        i8p = np.ctypeslib.ndpointer(np.int8, flags="C")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
        L.ora_last_error.restype = C.c_char_p
        L.ora_system_create.restype = P
        L.ora_system_create.argtypes = [
            C.c_int, i64p, i64p, C.c_double, C.c_int, f64p, C.c_int, i32p, i64p, i32p,
            f64p, f64p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
        ]
        L.ora_system_create_xtal.restype = P
        L.ora_system_create_xtal.argtypes = [
            C.c_int, f64p, f64p, i32p, i32p, C.c_int, f64p, C.c_int, i32p, i64p, i32p,
            f64p, f64p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
        ]
        L.ora_system_destroy.argtypes = [P]
        L.ora_n_sites.argtypes = [P]
        L.ora_n_clusters.argtypes = [P]
        L.ora_multiplicities.argtypes = [P, f64p]
        L.ora_counts.argtypes = [P, i8p, i64p]
        L.ora_energy.argtypes = [P, i8p]
        L.ora_energy.restype = C.c_double
        L.ora_corr.argtypes = [P, i8p, f64p]
        L.ora_delta.argtypes = [P, i8p, C.c_int, i64p, i32p, i64p]
        L.ora_delta.restype = C.c_double
        L.ora_delta_sgc.argtypes = [P, i8p, C.c_int, i64p, i32p, f64p, i64p]
        L.ora_delta_sgc.restype = C.c_double
        L.ora_run.restype = C.c_int
        L.ora_run.argtypes = [
            P, i8p, C.c_int, C.c_double, f64p, C.c_uint64, C.c_int64, C.c_int64,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
            C.c_void_p, C.c_void_p, C.c_void_p,
        ]
        L.ora_run_threads.restype = C.c_double
        L.ora_run_threads.argtypes = [
            P, i8p, C.c_int, C.c_int, f64p, f64p, C.c_uint64, C.c_int64, C.c_int,
            C.POINTER(C.c_int64),
        ]
        L.ora_time_delta.restype = C.c_double
        L.ora_time_delta.argtypes = [P, i8p, C.c_int64, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_double)]
        L.ora_run_chains.restype = C.c_double
        L.ora_run_chains.argtypes = [
            P, i8p, C.c_int, C.c_int, f64p, f64p, C.c_uint64, C.c_int64, C.c_int,
            C.c_void_p, C.c_void_p,
        ]
        L.ora_enforce_composition.restype = C.c_int64
        L.ora_enforce_composition.argtypes = [P, i8p, f64p, C.c_uint64, u64p]
        L.ora_exp_neg.restype = C.c_double
        L.ora_exp_neg.argtypes = [C.c_double]
        L.ora_nfold.restype = C.c_int64
        L.ora_nfold.argtypes = [P, i8p, C.c_double, f64p, f64p, C.c_uint64, C.c_int64, C.c_int64,
                                C.c_int64, i64p, i32p, f64p, f64p]
        L.ora_mt19937_64.argtypes = [C.c_uint64, C.c_int64, u64p]
        L.ora_std_uniform_int.argtypes = [C.c_uint64, C.c_int64, i64p, i64p, u64p]
        L.ora_std_uniform_real.argtypes = [C.c_uint64, C.c_int64, f64p]
        L.ora_philox4x32_10.argtypes = [u32p, u32p, u32p]
        _ = (u8p,)
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def composition_RT(n_basis: int, n_occ: int) -> np.ndarray:
    """R^T (param composition per change of species counts) for the standard
    axes: origin = all sites of species 0, end member k = all of species k."""
    Q = np.zeros((n_occ, n_occ - 1))
    for k in range(1, n_occ):
        Q[0, k - 1] = -n_basis
        Q[k, k - 1] = n_basis
    return np.ascontiguousarray(np.linalg.pinv(Q))


def _in_lattice(T, adj, det, v) -> bool:
    """v in T Z^3: T^-1 v = adj(T) v / det(T) is integral."""
    w = adj @ np.asarray(v, dtype=np.int64)
    return bool(np.all(w % det == 0))


def hermite_lower(T) -> np.ndarray:
    """Lower-triangular Hermite normal form of the superlattice T Z^3 (columns
    of T = supercell lattice vectors in prim cell coordinates), found from its
    definition rather than by column operations: H22 is the smallest positive
    z with (0, 0, z) in the lattice; (0, H11, H21) the lattice vector with the
    smallest positive y among those with x = 0 (0 <= z < H22); (H00, H10, H20)
    one with the smallest positive x (the gcd of the first row of T, reached by
    the extended Euclid algorithm) with y and z reduced by the two others."""
    T = np.asarray(T, dtype=np.int64).reshape(3, 3)
    det = int(round(np.linalg.det(T)))
    if det == 0:
        raise ValueError("singular supercell matrix")
    adj = np.array([[int(round(x)) for x in row] for row in np.linalg.inv(T) * det], dtype=np.int64)
    n = abs(det)
    h22 = next(z for z in range(1, n + 1) if _in_lattice(T, adj, det, (0, 0, z)))
    h11, h21 = next((y, z) for y in range(1, n + 1) for z in range(h22)
                    if _in_lattice(T, adj, det, (0, y, z)))

    def egcd(a, b):
        if b == 0:
            return (abs(a), (1 if a >= 0 else -1), 0)
        g, x, y = egcd(b, a % b)
        return g, y, x - (a // b) * y

    a0, a1, a2 = (int(x) for x in T[0])
    g01, x0, x1 = egcd(a0, a1)
    g, y01, y2 = egcd(g01, a2)
    coef = np.array([y01 * x0, y01 * x1, y2], dtype=np.int64)
    v = T @ coef  # a lattice vector with first coordinate g
    assert v[0] == g
    q = v[1] // h11
    v = v - q * np.array([0, h11, h21])
    v[2] %= h22
    return np.array([[g, 0, 0], [v[1], h11, 0], [v[2], h21, h22]], dtype=np.int64)


class OracleSystem:
    """A cluster expansion on one supercell, evaluated by the oracle. ``L``:
    three edge lengths of a diagonal supercell, or a 3 x 3 supercell matrix
    (columns = supercell lattice vectors in prim cell coordinates), indexed on
    its lower-triangular Hermite normal form H: cell (i, j, k) with
    0 <= i < H00, 0 <= j < H11, 0 <= k < H22 is unit cell i + H00 (j + H11 k)."""

    def __init__(self, ce, L):
        self.ce = ce
        prim = ce.prim
        if np.ndim(L) == 2:
            H = hermite_lower(L)
            self.L = (int(H[0, 0]), int(H[1, 1]), int(H[2, 2]))
            self.twist = (int(H[1, 0]), int(H[2, 0]), int(H[2, 1]))
        else:
            self.L = tuple(int(x) for x in L)
            self.twist = (0, 0, 0)
        nf = ce.n_funcs
        size = np.zeros(nf, dtype=np.int32)
        occ = np.zeros((nf, 4), dtype=np.int32)
        for f in range(1, nf):
            o = ce.orbits[ce.func_orbit[f]]
            size[f] = o.size
            occ[f, : o.size] = np.array(ce.func_rep[f]) + 1
        ml = np.zeros(5)
        for k, v in ce.max_length.items():
            ml[k] = v
        rt = getattr(ce, "param_RT", None)
        self.RT = composition_RT(prim.n_basis, prim.n_occ) if rt is None else np.asarray(rt, dtype=np.float64)
        common = (
            np.ascontiguousarray(ce.eci, dtype=np.float64),
            np.ascontiguousarray(ce.func_coeff, dtype=np.float64),
            np.ascontiguousarray(self.RT.reshape(-1)),
            *self.L,
            *self.twist,
        )
        cr = getattr(ce, "crystal", None)
        if cr is not None:
            # general crystal: prototypes as integral sites (prim sublattice, cell)
            sites = np.zeros((nf, 4, 4), dtype=np.int64)
            for f in range(1, nf):
                for q, (b, u) in enumerate(ce.orbits[ce.func_orbit[f]].proto_sites):
                    sites[f, q] = (b, *u)
            kinds = {o: k for k, o in enumerate(dict.fromkeys(cr.occupants))}
            h = lib().ora_system_create_xtal(
                cr.n_basis,
                np.ascontiguousarray(cr.lattice.reshape(-1)),
                np.ascontiguousarray(cr.frac.reshape(-1)),
                np.array([kinds[o] for o in cr.occupants], dtype=np.int32),
                np.array([1 if len(o) > 1 else 0 for o in cr.occupants], dtype=np.int32),
                prim.n_occ, ml, nf, size, np.ascontiguousarray(sites.reshape(-1)),
                np.ascontiguousarray(occ.reshape(-1)), *common,
            )
        else:
            pts = np.zeros((nf, 4, 3), dtype=np.int64)
            for f in range(1, nf):
                o = ce.orbits[ce.func_orbit[f]]
                pts[f, : o.size] = o.prototype
            h = lib().ora_system_create(
                prim.n_basis,
                np.ascontiguousarray(prim.lattice.reshape(-1), dtype=np.int64),
                np.ascontiguousarray(prim.basis.reshape(-1), dtype=np.int64),
                float(prim.grid), prim.n_occ, ml, nf, size,
                np.ascontiguousarray(pts.reshape(-1)), np.ascontiguousarray(occ.reshape(-1)),
                *common,
            )
        if not h:
            raise RuntimeError(lib().ora_last_error().decode())
        self.h = h
        self.n_sites = lib().ora_n_sites(h)
        self.n_uc = self.L[0] * self.L[1] * self.L[2]

    def __del__(self):
        if getattr(self, "h", None):
            lib().ora_system_destroy(self.h)
            self.h = None

    def multiplicities(self):
        out = np.zeros(self.ce.n_funcs)
        lib().ora_multiplicities(self.h, out)
        return out

    def counts(self, occ):
        out = np.zeros(self.ce.n_funcs, dtype=np.int64)
        lib().ora_counts(self.h, np.ascontiguousarray(occ, dtype=np.int8), out)
        return out

    def energy(self, occ) -> float:
        return lib().ora_energy(self.h, np.ascontiguousarray(occ, dtype=np.int8))

    def corr(self, occ):
        out = np.zeros(self.ce.n_funcs)
        lib().ora_corr(self.h, np.ascontiguousarray(occ, dtype=np.int8), out)
        return out

    def delta(self, occ, sites, new_occ, mu=None):
        sites = np.ascontiguousarray(sites, dtype=np.int64)
        new_occ = np.ascontiguousarray(new_occ, dtype=np.int32)
        dc = np.zeros(self.ce.n_funcs, dtype=np.int64)
        o = np.ascontiguousarray(occ, dtype=np.int8)
        if mu is None:
            de = lib().ora_delta(self.h, o, len(sites), sites, new_occ, dc)
        else:
            de = lib().ora_delta_sgc(
                self.h, o, len(sites), sites, new_occ,
                np.ascontiguousarray(mu, dtype=np.float64), dc,
            )
        return de, dc

    def run(self, occ, ensemble, temperature, mu, seed, n_passes, record_steps=0):
        """Sequential Metropolis chain. ``occ`` is updated in place."""
        n = self.n_sites
        nc = self.ce.prim.n_occ - 1
        rs0 = np.zeros(record_steps, dtype=np.int64)
        rs1 = np.zeros(record_steps, dtype=np.int64)
        rde = np.zeros(record_steps, dtype=np.float64)
        racc = np.zeros(record_steps, dtype=np.uint8)
        se = np.zeros(n_passes)
        sp = np.zeros(n_passes)
        scomp = np.zeros((n_passes, nc))
        nacc = np.zeros(1, dtype=np.int64)
        draws = np.zeros(1, dtype=np.uint64)
        mu = np.zeros(nc) if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        assert occ.dtype == np.int8 and occ.flags.c_contiguous and occ.size == n
        rc = lib().ora_run(
            self.h, occ, int(ensemble), float(temperature), mu, int(seed), int(n_passes),
            int(record_steps), _ptr(rs0), _ptr(rs1), _ptr(rde), _ptr(racc), _ptr(se),
            _ptr(sp), _ptr(scomp), _ptr(nacc), _ptr(draws),
        )
        if rc:
            raise RuntimeError(lib().ora_last_error().decode())
        return dict(
            site0=rs0, site1=rs1, dE=rde, accept=racc, energy=se, potential=sp,
            comp=scomp, n_accept=int(nacc[0]), draws=int(draws[0]),
        )

    def enforce_composition(self, occ, target_mol, seed):
        """Greedy composition enforcement; ``occ`` is updated in place.
        Returns (flips, engine draws)."""
        assert occ.dtype == np.int8 and occ.flags.c_contiguous and occ.size == self.n_sites
        draws = np.zeros(1, dtype=np.uint64)
        n = lib().ora_enforce_composition(
            self.h, occ, np.ascontiguousarray(target_mol, dtype=np.float64), int(seed), draws)
        if n < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return int(n), int(draws[0])

    def nfold(self, occ, temperature, mu, w, seed, n_events, n_equil=0, record=0):
        """n-fold way restated sequentially; ``occ`` is updated in place.
        ``w`` are the per-function weights the GPU uses."""
        assert occ.dtype == np.int8 and occ.flags.c_contiguous and occ.size == self.n_sites
        rec_site = np.zeros(max(record, 1), dtype=np.int64)
        rec_occ = np.zeros(max(record, 1), dtype=np.int32)
        rec_dt = np.zeros(max(record, 1))
        st = np.zeros(19)
        n = lib().ora_nfold(self.h, occ, float(temperature), np.ascontiguousarray(mu, dtype=np.float64),
                            np.ascontiguousarray(w, dtype=np.float64), int(seed), int(n_events),
                            int(n_equil), int(record), rec_site, rec_occ, rec_dt, st)
        if n < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return dict(n=int(n), site=rec_site[:record], occ=rec_occ[:record], dt=rec_dt[:record],
                    stats=st)

    def time_delta(self, occ, sites, new_occ):
        """(seconds, checksum) of independent one-site energy changes on one
        thread (the state is left unchanged)."""
        sites = np.ascontiguousarray(sites, dtype=np.int64)
        new_occ = np.ascontiguousarray(new_occ, dtype=np.int32)
        o = np.ascontiguousarray(occ, dtype=np.int8)
        cs = C.c_double()
        secs = lib().ora_time_delta(self.h, o, len(sites), sites.ctypes.data, new_occ.ctypes.data,
                                    C.byref(cs))
        return secs, cs.value

    def run_chains(self, occ, ensemble, temps, mus, seed, n_passes, n_threads):
        """Independent sequential chains (chain r: block r of ``occ``, updated
        in place, engine seed + r), spread over ``n_threads`` host threads.
        Returns (potential [n_rep, n_passes], comp [n_rep, n_passes, n_occ-1],
        wall seconds) with the per-unit-cell samples after every pass."""
        nrep = len(temps)
        nc = self.ce.prim.n_occ - 1
        assert occ.dtype == np.int8 and occ.flags.c_contiguous and occ.size == nrep * self.n_sites
        pot = np.zeros((nrep, n_passes))
        comp = np.zeros((nrep, n_passes, nc))
        secs = lib().ora_run_chains(
            self.h, occ, nrep, int(ensemble), np.ascontiguousarray(temps, dtype=np.float64),
            np.ascontiguousarray(mus, dtype=np.float64).reshape(-1), int(seed), int(n_passes),
            int(n_threads), _ptr(pot), _ptr(comp))
        if secs < 0:
            raise RuntimeError(lib().ora_last_error().decode())
        return pot, comp, secs

    def run_threads(self, occ, ensemble, temps, mus, seed, n_passes, n_threads):
        nrep = len(temps)
        nsteps = C.c_int64(0)
        secs = lib().ora_run_threads(
            self.h, occ, nrep, int(ensemble), np.ascontiguousarray(temps, dtype=np.float64),
            np.ascontiguousarray(mus, dtype=np.float64).reshape(-1), int(seed), int(n_passes),
            int(n_threads), C.byref(nsteps),
        )
        return secs, nsteps.value


def mt19937_64(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint64)
    lib().ora_mt19937_64(seed, n, out)
    return out


def std_uniform_int(seed: int, maxv) -> tuple:
    maxv = np.ascontiguousarray(maxv, dtype=np.int64)
    out = np.zeros(len(maxv), dtype=np.int64)
    draws = np.zeros(1, dtype=np.uint64)
    lib().ora_std_uniform_int(seed, len(maxv), maxv, out, draws)
    return out, int(draws[0])


def std_uniform_real(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    lib().ora_std_uniform_real(seed, n, out)
    return out


def philox4x32_10(ctr, key) -> np.ndarray:
    out = np.zeros(4, dtype=np.uint32)
    lib().ora_philox4x32_10(
        np.ascontiguousarray(ctr, dtype=np.uint32), np.ascontiguousarray(key, dtype=np.uint32), out
    )
    return out
