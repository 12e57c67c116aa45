"""Completion-checked runs (the reference's default canonical fixture stops
when potential_energy reaches an absolute precision of 0.001,
CanonicalCalculator.cc:261-270) and summary.json written from real GPU
statistics, checked against the reference validator's keys
(python/tests/conftest.py:180-259, restated in tests/test_casm_io.py) and
against the oracle's sequential chains."""

import json
import os

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads
from casmcode_clexmonte_gb300.casm_io import SummaryWriter
from casmcode_clexmonte_gb300.stats import jackknife_chains
from tests.test_casm_io import _validate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cm():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import calculator

    return calculator


@pytest.mark.parametrize("method", ["canonical", "semigrand_canonical"])
def test_run_to_requested_precision_and_summary(method, cm, oracle_mod, tmp_path):
    ce = workloads.config(0).ce
    L = (12, 12, 12)
    n = int(np.prod(L))
    sysd = cm.System(ce)
    calc = cm.MonteCalculator(method, sysd, {"seed": 4242})
    sgc = method == "semigrand_canonical"
    req = {"potential_energy": 2e-4}
    if sgc:
        req["param_composition"] = 2e-3
    path = str(tmp_path / "summary.json")
    w = SummaryWriter(path, method, ["A", "B"], n_sites_per_uc=1, requested_precision=req)
    o = oracle_mod.OracleSystem(ce, L)
    rng = np.random.default_rng(3)
    conds = [(600.0, 0.05, 0.3), (1100.0, -0.05, 0.5)]
    for T, mu, x in conds:
        occ = workloads.fixed_composition(rng, n, x)
        c = {"temperature": T}
        if sgc:
            c["param_chem_pot"] = np.array([mu])
        state = cm.MonteCarloState(occupation=occ.copy(), L=L, conditions=c)
        p = cm.SamplingFixtureParams(n_passes=200000, n_equil=100, requested_precision=req,
                                     check_period=200)
        res = calc.run_fixture(state, p)
        # stopped by the completion check, well before the cutoff
        assert res["all_converged"], res["is_converged"]
        assert res["count"] < p.n_passes
        assert all(res["is_converged"].values())
        # the state is the final state of the run, with its exact energy
        assert np.array_equal(state.occupation, calc._batch.get_occupation(0))
        if not sgc:
            assert state.occupation.sum() == occ.sum()
        w.append(temperature=T, n_unitcells=n, stats=res,
                 samples=(res["samples_potential"], res["samples_comp"]),
                 param_chem_pot=np.array([mu]), elapsed_s=0.0, count=res["count"])
        # the mean against 16 oracle chains: within 2 combined standard errors
        # (the run's standard error is its calculated precision / z(0.95))
        occ_o = np.ascontiguousarray(np.concatenate([occ] * 16), dtype=np.int8)
        pot, comp, _ = o.run_chains(occ_o, 0 if sgc else 1, np.full(16, T),
                                    np.full((16, 1), mu if sgc else 0.0), 17, 700,
                                    os.cpu_count() or 1)
        chains = [pot[i, 200:, None] for i in range(16)]
        e_o, se_o = jackknife_chains(lambda a: a[:, 0].mean(), chains)
        se_g = req["potential_energy"] / 1.959963984540054
        assert abs(res["mean_potential"] - e_o) <= 2.0 * np.hypot(se_g, se_o), \
            (res["mean_potential"], e_o, se_g, se_o)
    w.write()
    data = json.load(open(path))
    _validate(data, len(conds), method == "canonical", True)
    cc = data["completion_check_results"]
    assert cc["all_converged"] == [True, True]
    assert all(v >= 0 for v in cc["N_samples_for_all_to_equilibrate"])
    prec = data["statistics"]["potential_energy"]["value"]["calculated_precision"]
    assert all(0.0 < v <= req["potential_energy"] for v in prec)
