"""The compiled C++ calculator plugin: GpuCanonicalCalculator and
GpuSemiGrandCanonicalCalculator behind the reference's BaseMonteCalculator /
BaseMontePotential interface (include/casm/clexmonte/monte_calculator/
BaseMonteCalculator.hh:26-264), created by their make_<Name> factories
(CanonicalCalculator.cc:580-586, SemiGrandCanonicalCalculator.cc:517-523)
and driven through the plugin's C entry points. occ_delta_per_supercell,
per_supercell and run() are checked against the oracle."""

import ctypes as C
import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from casmcode_clexmonte_gb300.stats import jackknife_chains

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plugin():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    lib = C.CDLL(build.PLUGIN)
    vp, i64 = C.c_void_p, C.c_int64
    lib.cem_plugin_last_error.restype = C.c_char_p
    lib.cem_plugin_create.restype = vp
    lib.cem_plugin_create.argtypes = [C.c_char_p, vp, C.c_int, vp]
    lib.cem_plugin_destroy.argtypes = [vp]
    lib.cem_plugin_set_state.argtypes = [vp, vp, vp, i64, C.c_double, vp]
    lib.cem_plugin_occ_delta.argtypes = [vp, C.c_int, vp, vp, C.POINTER(C.c_double)]
    lib.cem_plugin_per_supercell.argtypes = [vp, C.POINTER(C.c_double)]
    lib.cem_plugin_run.argtypes = [vp, C.c_longlong, C.c_longlong, C.c_longlong, C.c_longlong,
                                   C.c_double, C.c_double, vp, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                   C.POINTER(C.c_int)]
    lib.cem_plugin_n_mol.argtypes = [vp, C.c_int, C.POINTER(C.c_int64)]
    return lib, calculator


class Calc:
    def __init__(self, lib, cm, method, ce):
        self.lib = lib
        self.system = cm.System(ce)  # keeps the device tables alive
        RT = np.ascontiguousarray(self.system.RT, dtype=np.float64)
        self.h = lib.cem_plugin_create(method.encode(), self.system.handle, ce.prim.n_occ,
                                       RT.ctypes.data)
        assert self.h, lib.cem_plugin_last_error().decode()

    def check(self, rc):
        assert rc == 0, self.lib.cem_plugin_last_error().decode()

    def set_state(self, T_mat, occ, temperature, mu=None):
        T_mat = np.ascontiguousarray(T_mat, dtype=np.int64)
        occ = np.ascontiguousarray(occ, dtype=np.int32)
        m = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        return self.lib.cem_plugin_set_state(self.h, T_mat.ctypes.data, occ.ctypes.data, occ.size,
                                             temperature, None if m is None else m.ctypes.data)

    def delta(self, sites, new_occ):
        s = np.ascontiguousarray(sites, dtype=np.int64)
        o = np.ascontiguousarray(new_occ, dtype=np.int32)
        d = C.c_double()
        self.check(self.lib.cem_plugin_occ_delta(self.h, s.size, s.ctypes.data, o.ctypes.data,
                                                 C.byref(d)))
        return d.value

    def per_supercell(self):
        v = C.c_double()
        self.check(self.lib.cem_plugin_per_supercell(self.h, C.byref(v)))
        return v.value

    def run(self, n_sites, seed, max_count, n_equil, period, req_e, req_x=0.0):
        occ = np.zeros(n_sites, dtype=np.int32)
        m, p, cnt, conv = C.c_double(), C.c_double(), C.c_longlong(), C.c_int()
        rc = self.lib.cem_plugin_run(self.h, seed, max_count, n_equil, period, req_e, req_x,
                                     occ.ctypes.data, C.byref(m), C.byref(p), C.byref(cnt),
                                     C.byref(conv))
        return rc, occ, m.value, p.value, cnt.value, bool(conv.value)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.cem_plugin_destroy(self.h)


@pytest.mark.parametrize("method", ["canonical", "semigrand_canonical"])
def test_plugin_potential_and_run_against_oracle(method, plugin, oracle_mod):
    lib, cm = plugin
    ce = workloads.config(0).ce
    L = (12, 12, 12)
    n = int(np.prod(L))
    sgc = method == "semigrand_canonical"
    mu = np.array([0.04]) if sgc else None
    calc = Calc(lib, cm, method, ce)
    o = oracle_mod.OracleSystem(ce, L)
    rng = np.random.default_rng(23)
    occ = workloads.fixed_composition(rng, n, 0.35)
    calc.check(calc.set_state(np.diag(L), occ, 900.0, mu))
    # occ_delta_per_supercell: one- and two-site events, sequential semantics
    for k in (1, 2):
        for _ in range(64):
            sites = rng.integers(0, n, k)
            new = 1 - occ[sites]
            de_o, _ = o.delta(occ, sites, new, mu=mu) if sgc else o.delta(occ, sites, new)
            de = calc.delta(sites, new)
            assert abs(de - de_o) <= 1e-10 * abs(de_o) + 1e-12, (sites, de, de_o)
    # per_supercell: the formation energy (canonical) or the semi-grand potential
    e_o = o.energy(occ)
    if sgc:
        e_o -= mu[0] * (occ.sum() - 0.0)  # x = N_B / n_uc for the binary axes; n_uc mu x = mu N_B
    assert abs(calc.per_supercell() - e_o) <= 1e-10 * abs(e_o) + 1e-12
    # run(): a completion-checked run that evolves the state
    rc, occ2, mean_e, prec_e, count, conv = calc.run(n, 99, 100000, 100, 200, 2e-4,
                                                     2e-3 if sgc else 0.0)
    assert rc == 0, lib.cem_plugin_last_error().decode()
    assert conv and 0 < prec_e <= 2e-4 and count < 100000
    if not sgc:
        assert occ2.sum() == occ.sum()
    nb = C.c_int64()
    calc.check(lib.cem_plugin_n_mol(calc.h, 1, C.byref(nb)))
    assert nb.value == occ2.sum()  # the occupant lists follow the evolved state
    e_after = o.energy(occ2.astype(np.int8))
    if sgc:
        e_after -= mu[0] * occ2.sum()
    assert abs(calc.per_supercell() - e_after) <= 1e-10 * abs(e_after) + 1e-12
    # the run's mean against 16 oracle chains (2 combined standard errors)
    occ_o = np.ascontiguousarray(np.concatenate([occ] * 16), dtype=np.int8)
    pot, _, _ = o.run_chains(occ_o, 0 if sgc else 1, np.full(16, 900.0),
                             np.full((16, 1), mu[0] if sgc else 0.0), 5, 700, os.cpu_count() or 1)
    e_ref, se_ref = jackknife_chains(lambda a: a[:, 0].mean(), [pot[i, 200:, None] for i in range(16)])
    assert abs(mean_e - e_ref) <= 2.0 * np.hypot(prec_e / 1.959963984540054, se_ref), \
        (mean_e, e_ref, prec_e, se_ref)


def test_plugin_rejects_what_the_reference_rejects(plugin, oracle_mod):
    lib, cm = plugin
    ce = workloads.config(0).ce
    calc = Calc(lib, cm, "canonical", ce)
    occ = np.zeros(8 ** 3, dtype=np.int32)
    occ[::3] = 1
    # a run manager without an engine (CanonicalCalculator.cc:418-422)
    calc.check(calc.set_state(np.diag((8, 8, 8)), occ, 500.0))
    rc, *_ = calc.run(occ.size, -1, 100, 0, 50, 0.0)
    assert rc == -1 and "engine" in lib.cem_plugin_last_error().decode()
    # non-diagonal supercells: the potential works, run() needs a diagonal one
    T = np.array([[8, 1, 0], [0, 8, 0], [0, 0, 8]])
    calc.check(calc.set_state(T, occ, 500.0))
    o_t = oracle_mod.OracleSystem(ce, T)
    for site in (0, 5, 100, 511):
        de_o, _ = o_t.delta(occ.astype(np.int8), [site], [1 - occ[site]])
        assert abs(calc.delta([site], [1 - occ[site]]) - de_o) <= 1e-10 * abs(de_o) + 1e-12
    rc, *_ = calc.run(occ.size, 7, 100, 0, 50, 0.0)
    assert rc == -1 and "diagonal supercells" in lib.cem_plugin_last_error().decode()
    # missing semi-grand conditions
    sg = Calc(lib, cm, "semigrand_canonical", ce)
    assert sg.set_state(np.diag((8, 8, 8)), occ, 500.0, None) == -1
    assert "param_chem_pot" in lib.cem_plugin_last_error().decode()
