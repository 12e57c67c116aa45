"""GB300-native cluster-expansion Metropolis hot path (canonical and
semi-grand canonical), a drop-in for the per-event potential change and the
Metropolis loop of libcasm-clexmonte, built on hand-written CUDA kernels for
sm_103a behind the C ABI in ``include/cem.h``."""

from .system import (  # noqa: F401
    KB,
    ClusterExpansion,
    Prim,
    Supercell,
    bcc_conventional,
    bcc_prim,
    composition_RT,
    fcc_prim,
    make_colouring,
    system_arrays,
    verify_local_pairs,
)
from .casm_io import (  # noqa: F401
    SummaryWriter,
    read_cluster_expansion,
    read_prim,
    read_system,
    write_eci_json,
)


def __getattr__(name):
    # the CUDA-backed classes load the shared library on first use
    if name in (
        "System", "ReplicaBatch", "MonteCarloState", "MontePotential", "MonteCalculator",
        "SamplingFixtureParams", "analyses", "enforce_composition", "mol_composition",
    ):
        from . import calculator

        return getattr(calculator, name)
    raise AttributeError(name)
