"""Checks shared by the statistical GPU tests."""

from casmcode_clexmonte_gb300.stats import tau_int

MIN_TAUS = 50.0


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
