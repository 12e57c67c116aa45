"""Non-diagonal supercells (the reference state's transformation_matrix_to_super,
include/casm/clexmonte/state/Configuration.hh:29-50) on the CPU: the library's
Hermite normal form against the oracle's definition-based one, and the
oracle's twisted cell reduction against a diagonal supercell that tiles it
(the diagonal path is pinned to the reference's own Clexulator)."""

import ctypes

import numpy as np
import pytest

from casmcode_clexmonte_gb300 import workloads

FCC_CONV = np.array([[-1, 1, 1], [1, -1, 1], [1, 1, -1]])  # conventional FCC cell, prim coords

# (name, supercell matrix); columns are the supercell lattice vectors
SUPERCELLS = [
    ("fcc_conventional_2", 2 * FCC_CONV),
    ("fcc_conventional_5", 5 * FCC_CONV),
    ("sheared", np.array([[6, 0, 0], [3, 6, 0], [0, 0, 6]])),
    # H U: H = [[6, 0, 0], [3, 6, 0], [3, 3, 6]] (both twists) times a unimodular U
    ("general", np.array([[6, 0, 0], [3, 6, 0], [3, 3, 6]]) @ np.array([[1, 1, 0], [0, 1, 1], [1, 1, 1]])),
]


def cell_index(H, i, j, k):
    """Unit cell (i, j, k) reduced into the Hermite-normal-form box of H."""
    L0, L1, L2 = int(H[0, 0]), int(H[1, 1]), int(H[2, 2])
    q = i // L0
    i, j, k = i - q * L0, j - q * int(H[1, 0]), k - q * int(H[2, 0])
    q = j // L1
    j, k = j - q * L1, k - q * int(H[2, 1])
    return i + L0 * (j + L1 * (k % L2))


def product_hnf(T):
    from casmcode_clexmonte_gb300 import _lib, build

    build.build()
    lib = _lib.load()
    t = np.ascontiguousarray(np.asarray(T, dtype=np.int64).reshape(-1))
    h = np.zeros(9, dtype=np.int64)
    if lib.cem_supercell_hnf(t.ctypes.data_as(ctypes.c_void_p), h.ctypes.data_as(ctypes.c_void_p)):
        raise RuntimeError(lib.cem_last_error().decode())
    return h.reshape(3, 3)


def test_library_hnf_matches_the_definition(oracle_mod):
    rng = np.random.default_rng(21)
    mats = [T for _, T in SUPERCELLS] + [np.diag([4, 5, 6]), np.diag([-3, 2, -5])]
    while len(mats) < 60:
        T = rng.integers(-6, 7, (3, 3))
        if 0 < abs(round(np.linalg.det(T))) <= 400:
            mats.append(T)
    for T in mats:
        H = product_hnf(T)
        np.testing.assert_array_equal(H, oracle_mod.hermite_lower(T), err_msg=str(T))
        if T is SUPERCELLS[3][1]:
            np.testing.assert_array_equal(H, [[6, 0, 0], [3, 6, 0], [3, 3, 6]])
        assert H[0, 1] == H[0, 2] == H[1, 2] == 0
        assert np.all(np.diag(H) > 0)
        assert 0 <= H[1, 0] < H[1, 1] and 0 <= H[2, 0] < H[2, 2] and 0 <= H[2, 1] < H[2, 2]
        assert np.prod(np.diag(H)) == abs(round(np.linalg.det(T)))
        # H's columns generate the lattice of T's columns: T = H V with V integral
        V = np.linalg.solve(H, T)
        np.testing.assert_allclose(V, np.round(V), atol=1e-9)
        for c in range(3):  # every supercell lattice vector is a period of the reduction
            assert cell_index(H, *T[:, c]) == 0
    with pytest.raises(RuntimeError, match="singular"):
        product_hnf(np.array([[1, 2, 3], [2, 4, 6], [0, 0, 1]]))


def _tiling(H):
    """Smallest diagonal supercell D inside the lattice of H, and for every
    cell of D (in D's order) the cell of H it is an image of."""
    d = [next(x for x in range(1, 10_000) if cell_index(H, *(x * e)) == 0) for e in np.eye(3, dtype=int)]
    k, j, i = np.meshgrid(np.arange(d[2]), np.arange(d[1]), np.arange(d[0]), indexing="ij")
    img = cell_index(H, i.ravel(), j.ravel(), k.ravel())
    return tuple(d), img


@pytest.mark.parametrize("name,T", SUPERCELLS)
@pytest.mark.parametrize("system", ["fcc_binary", "bcc_ternary"])
def test_oracle_supercell_matches_a_diagonal_tiling(name, T, system, oracle_mod):
    """A configuration on T tiled onto a diagonal supercell D: every cluster
    count is m times T's (m = cells of D per cell of T), and changing one site
    of T changes D's counts by m times T's change when all m images change."""
    ce = workloads.fcc_binary_ce(3) if system == "fcc_binary" else workloads.bcc_ternary_ce(4)
    nocc = ce.prim.n_occ
    H = oracle_mod.hermite_lower(T)
    o_t = oracle_mod.OracleSystem(ce, T)
    assert o_t.L == (H[0, 0], H[1, 1], H[2, 2])
    d, img = _tiling(H)
    o_d = oracle_mod.OracleSystem(ce, d)
    n_uc_t, n_uc_d = o_t.n_uc, o_d.n_uc
    m = n_uc_d // n_uc_t
    assert m * n_uc_t == n_uc_d and np.bincount(img, minlength=n_uc_t).min() == m
    nb = o_t.n_sites // n_uc_t
    site_map = (np.arange(nb)[:, None] * n_uc_t + img[None, :]).ravel()  # D site -> T site
    rng = np.random.default_rng(31)
    for _ in range(2):
        occ_t = rng.integers(0, nocc, o_t.n_sites).astype(np.int8)
        occ_d = occ_t[site_map]
        np.testing.assert_array_equal(o_d.counts(occ_d)[1:], m * o_t.counts(occ_t)[1:])
        assert o_d.energy(occ_d) == pytest.approx(m * o_t.energy(occ_t), rel=1e-12, abs=1e-9)
        for s in rng.integers(0, o_t.n_sites, 25):
            f = (occ_t[s] + rng.integers(1, nocc)) % nocc
            _, dc_t = o_t.delta(occ_t, [s], [f])
            images = np.nonzero(site_map == s)[0]
            assert images.size == m
            _, dc_d = o_d.delta(occ_d, images, [f] * m)
            np.testing.assert_array_equal(dc_d[1:], m * dc_t[1:])


def test_oracle_refuses_a_supercell_with_a_cluster_on_two_images(oracle_mod):
    """The conventional FCC cell itself: its lattice vector (-1, 1, 1) is the
    second-neighbour distance a, so a second-neighbour pair joins a site and
    its own image."""
    with pytest.raises(RuntimeError, match="supercell too small"):
        oracle_mod.OracleSystem(workloads.fcc_binary_ce(3), FCC_CONV)


def test_scale_supercell_grows_every_named_axis():
    from casmcode_clexmonte_gb300 import calculator as c

    np.testing.assert_array_equal(c.scale_supercell(np.eye(3, dtype=int), "abc", 1000), 10 * np.eye(3))
    np.testing.assert_array_equal(c.scale_supercell(FCC_CONV, "abc", 1000), 7 * FCC_CONV)  # 1372 >= 1000 > 864
    np.testing.assert_array_equal(c.scale_supercell(np.eye(3, dtype=int), "c", 50), np.diag([1, 1, 50]))
    np.testing.assert_array_equal(c.scale_supercell(np.diag([2, 3, 4]), "ab", 24), np.diag([2, 3, 4]))
    np.testing.assert_array_equal(c.scale_supercell(np.diag([2, 3, 4]), "ab", 25), np.diag([4, 6, 4]))


def test_tiled_l12_motif(oracle_mod):
    """The L1_2 motif on the conventional FCC cell (B on one of its four
    simple-cubic sublattices: prim cells with i = j = k mod 2) tiled into a
    diagonal supercell holds B exactly there, and tiled into a non-diagonal
    one it has the same energy per unit cell."""
    from casmcode_clexmonte_gb300 import build
    from casmcode_clexmonte_gb300 import calculator as c

    build.build()
    H = c.supercell_hnf(FCC_CONV)
    k, j, i = np.meshgrid(np.arange(H[2, 2]), np.arange(H[1, 1]), np.arange(H[0, 0]), indexing="ij")
    motif = ((i % 2 == j % 2) & (j % 2 == k % 2)).ravel().astype(np.int8)
    assert motif.sum() == 1 and motif.size == 4
    diag = c.tile_motif(motif, FCC_CONV, 6 * np.eye(3, dtype=int), 1)
    k, j, i = np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij")
    np.testing.assert_array_equal(diag, ((i % 2 == j % 2) & (j % 2 == k % 2)).ravel())
    twisted = c.tile_motif(motif, FCC_CONV, 3 * FCC_CONV, 1)
    ce = workloads.fcc_binary_ce(3, nn1=0.08)
    e_d = oracle_mod.OracleSystem(ce, (6, 6, 6)).energy(diag) / 216
    e_t = oracle_mod.OracleSystem(ce, 3 * FCC_CONV).energy(twisted) / 108
    assert e_t == pytest.approx(e_d, rel=1e-12, abs=1e-12)
    with pytest.raises(ValueError, match="Failed to tile"):
        c.tile_motif(motif, FCC_CONV, np.diag([3, 3, 3]), 1)


def test_match_composition_and_unit_cell_count():
    """The "match.composition" modifier on a ternary system (standard axes:
    param x_k = N_k / n_uc for one sublattice) and the unit-cell count of a
    supercell given as a matrix."""
    from types import SimpleNamespace

    from casmcode_clexmonte_gb300 import calculator as c
    from casmcode_clexmonte_gb300.system import composition_RT

    system = SimpleNamespace(n_occ=3, RT=composition_RT(1, 3))
    occ = np.array([0] * 50 + [1] * 30 + [2] * 28, dtype=np.int8)
    T = np.array([[6, 0, 0], [3, 6, 0], [0, 0, 3]])  # 108 unit cells
    state = c.MonteCarloState(occupation=occ, L=T, conditions={"temperature": 300.0})
    assert c._n_unitcells(T) == 108 and c._n_unitcells((4, 5, 6)) == 120
    c.match_composition(state, system)
    np.testing.assert_allclose(state.conditions["mol_composition"], [50 / 108, 30 / 108, 28 / 108])
    np.testing.assert_allclose(state.conditions["param_composition"], [30 / 108, 28 / 108], atol=1e-12)
    assert c._supercell_key(T) == ((6, 0, 0), (3, 6, 0), (0, 0, 3))
    assert c._supercell_key(np.array([4, 5, 6])) == (4, 5, 6)
