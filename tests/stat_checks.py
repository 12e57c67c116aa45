"""Checks shared by the statistical GPU tests: chain-length guard and the
2-sigma comparison of pooled independent chains (jackknife errors, 1 %
family-wise contract stated in tests/test_gpu_equilibrium.py)."""

import numpy as np

from casmcode_clexmonte_gb300.stats import family_2sigma, jackknife_chains, tau_int

MIN_TAUS = 50.0
KB = 8.617333262e-5  # eV/K


def check_chain_lengths(chains, sgc, label, min_taus=MIN_TAUS):
    """Every chain (samples x [E, x...]) holds at least ``min_taus``
    integrated autocorrelation times of E, of (E - <E>)^2 and, in the
    semi-grand canonical ensemble, of each composition."""
    for c in chains:
        series = [c[:, 0], (c[:, 0] - c[:, 0].mean()) ** 2]
        if sgc:
            series += [c[:, 1 + k] for k in range(c.shape[1] - 1)]
        for s in series:
            t = tau_int(s)
            assert s.size >= min_taus * t, f"{label}: {s.size} samples < {min_taus} tau_int ({t:.2f})"


def observables(T, n_uc, nc, sgc):
    """[(name, estimator over pooled [n, 1 + nc] samples of (E, x...))]:
    <E>, heat capacity C = var(E) N_uc / (k_B T^2) and, semi-grand canonical,
    <x_k>, cov(E, x_k) N_uc / (k_B T) and the susceptibilities
    cov(x_k, x_l) N_uc / (k_B T)
    (monte_calculator/analysis_functions.cc:43-173,
    run/io/convariance_functions.cc:29-146)."""
    out = [("<E>", lambda a: a[:, 0].mean()),
           ("C", lambda a: a[:, 0].var() * n_uc / (KB * T * T))]
    if sgc:
        for k in range(nc):
            out.append((f"<x{k}>", lambda a, k=k: a[:, 1 + k].mean()))
            out.append((f"chi_E{k}", lambda a, k=k: np.cov(a[:, 0], a[:, 1 + k], bias=True)[0, 1]
                        * n_uc / (KB * T)))
            for k2 in range(k, nc):
                out.append((f"chi_{k}{k2}",
                            lambda a, k=k, k2=k2: np.cov(a[:, 1 + k], a[:, 1 + k2], bias=True)[0, 1]
                            * n_uc / (KB * T)))
    return out


def compare(conditions, gpu_chains, ora_chains, n_uc, sgc):
    """conditions: [(label, T)]; per condition a list of chains (arrays
    [samples, 1 + nc]) on each side. Asserts the family-wise 2-sigma contract
    and returns the report."""
    rows, zs = [], []
    for (label, T), g, o in zip(conditions, gpu_chains, ora_chains):
        check_chain_lengths(g, sgc, f"GPU {label}")
        check_chain_lengths(o, sgc, f"oracle {label}")
        for name, f in observables(T, n_uc, g[0].shape[1] - 1, sgc):
            eg, sg = jackknife_chains(f, g)
            eo, so = jackknife_chains(f, o)
            z = (eg - eo) / np.hypot(sg, so)
            zs.append(z)
            rows.append(f"{label:>24s} {name:>8s} gpu {eg:+.6e} +- {sg:.1e}  oracle {eo:+.6e} "
                        f"+- {so:.1e}  z {z:+.2f}")
    ok, k, bound, n2 = family_2sigma(zs)
    msg = "\n".join(rows) + f"\n{n2} of {len(zs)} beyond 2 sigma (allowed {k}); bound {bound:.2f}"
    assert ok, msg
    return msg
