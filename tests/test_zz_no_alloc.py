"""The allocation-free delta entry point against the allocating one.

cem_delta_energy_noalloc is for callers that cannot allocate device memory
(a host program whose device memory belongs to another framework's pool, or
a per-event loop that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree). It stages events in a fixed array in the library's own
device memory. Two calls in a row must give the results of
cem_delta_energy (integer delta correlations exactly, dE within 1e-10
relative), and calls above the stated maximum are rejected.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_EVENTS = 4096


@pytest.fixture(scope="module")
def env():
    from casmcode_clexmonte_gb300 import build

    build.build()
    from casmcode_clexmonte_gb300 import _lib
    from casmcode_clexmonte_gb300 import calculator as cm
    from casmcode_clexmonte_gb300 import workloads

    lib = _lib.load()
    f = lib.cem_delta_energy_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return lib, cm, workloads, _lib


def _noalloc(lib, batch, sites, new_occ, potential, n_funcs, with_dcount=True):
    n_events, k = sites.shape
    dE = np.zeros(n_events)
    dc = np.zeros((n_events, n_funcs), dtype=np.int64) if with_dcount else None
    rc = lib.cem_delta_energy_noalloc(batch.handle, 0, n_events, k, sites.ctypes.data,
                                      new_occ.ctypes.data, int(potential), dE.ctypes.data,
                                      dc.ctypes.data if with_dcount else None)
    return rc, dE, dc


@pytest.mark.parametrize("kind", ["fcc_binary_sgc", "bcc_ternary_sgc", "zro_sgc", "fcc_twisted_sgc"])
def test_noalloc_delta_matches_allocating_entry_point(kind, env):
    lib, cm, workloads, _lib = env
    rng = np.random.default_rng(99)
    if kind == "fcc_binary_sgc":
        ce, L, mu = workloads.fcc_binary_ce(1), (10, 10, 10), np.array([0.03])
    elif kind == "bcc_ternary_sgc":
        ce, L, mu = workloads.bcc_ternary_ce(2), (6, 6, 6), np.array([0.1, -0.05])
    elif kind == "fcc_twisted_sgc":
        # a non-diagonal supercell (Hermite normal form with all three twists)
        L = np.array([[6, 0, 0], [3, 6, 0], [3, 3, 6]]) @ np.array([[1, 1, 0], [0, 1, 1], [1, 1, 1]])
        ce, mu = workloads.fcc_binary_ce(1), np.array([0.03])
    else:
        # the reference's Zr-O basis set: 74 functions, so every event's
        # delta-correlation row in the scratch array is 74 entries wide
        from tests.zro_fixture import zro_ce

        ce, L, mu = zro_ce(), (8, 8, 8), np.array([-0.4])
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "semigrand_canonical", [L])
    b.set_conditions(0, 900.0, mu)
    n = int(b.n_sites[0])
    nocc = ce.prim.n_occ
    occ = rng.integers(0, nocc, n).astype(np.int8)
    b.set_occupation(0, occ)
    for call in range(2):  # two calls in a row share the scratch array
        k = 1 if call == 0 else 2
        n_events = MAX_EVENTS if call == 0 else 1500
        sites = np.ascontiguousarray(rng.integers(0, n, (n_events, k)), dtype=np.int64)
        new_occ = np.ascontiguousarray((occ[sites] + rng.integers(1, nocc, (n_events, k))) % nocc,
                                       dtype=np.int32)
        potential = call == 0
        ref_dE, ref_dc = b.delta(0, sites, new_occ, potential=potential)
        rc, dE, dc = _noalloc(lib, b, sites, new_occ, potential, ce.n_funcs)
        assert rc == 0, lib.cem_last_error().decode()
        np.testing.assert_array_equal(dc, ref_dc)
        assert np.all(np.abs(dE - ref_dE) <= 1e-10 * np.abs(ref_dE) + 1e-12)
    # without a delta-correlation output the kernel skips that section
    sites = np.ascontiguousarray(rng.integers(0, n, (700, 2)), dtype=np.int64)
    new_occ = np.ascontiguousarray((occ[sites] + rng.integers(1, nocc, (700, 2))) % nocc,
                                   dtype=np.int32)
    ref_dE, _ = b.delta(0, sites, new_occ, potential=True)
    rc, dE, _ = _noalloc(lib, b, sites, new_occ, True, ce.n_funcs, with_dcount=False)
    assert rc == 0, lib.cem_last_error().decode()
    assert np.all(np.abs(dE - ref_dE) <= 1e-10 * np.abs(ref_dE) + 1e-12)


def test_noalloc_rejects_calls_above_the_limit(env):
    lib, cm, workloads, _lib = env
    ce = workloads.fcc_binary_ce(1)
    sysd = cm.System(ce)
    b = cm.ReplicaBatch(sysd, "canonical", [(8, 8, 8)])
    b.set_occupation(0, np.zeros(512, dtype=np.int8))
    sites = np.zeros((MAX_EVENTS + 1, 1), dtype=np.int64)
    new_occ = np.ones((MAX_EVENTS + 1, 1), dtype=np.int32)
    rc, _, _ = _noalloc(lib, b, sites, new_occ, False, ce.n_funcs)
    assert rc == 3  # CEM_ERR_UNSUPPORTED
    assert "at most 4096 events" in lib.cem_last_error().decode()
