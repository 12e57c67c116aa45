"""Generate a specialised site evaluator ("flower" of one site with
compile-time neighbour offsets) for a binary single-sublattice cluster
expansion, the GPU counterpart of CASM's generated Clexulator
``_calc_delta_point_corr`` (reference
``FCC_binary_vacancy_Clexulator_default.cc:555-580``).

The evaluator reads the Z distinct neighbours of a site once, from a
shared-memory block with x pitch P and y pitch P (P a template parameter),
and returns, for every non-empty orbit g, the number of flower clusters of g
whose partners are all occupant 1 (the product of the partners' occupation
site functions). The energy change of a flip is then
dE = (o_f - o_i) * sum_g W_g * count_g.

Run ``python -m casmcode_clexmonte_gb300.codegen`` to rewrite
``csrc/gen_fcc_binary.cuh``; a test checks that the committed header is what
this script produces.
"""

from __future__ import annotations

import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "gen_fcc_binary.cuh")


def topology(ce):
    """(neighbours [(du)], orbits [(size, [(partner neighbour indices)])])
    of sublattice 0, neighbours in order of first appearance."""
    assert ce.prim.n_basis == 1 and ce.prim.n_occ == 2
    nbs = []
    index = {}
    orbits = []
    for g, o in enumerate(ce.orbits):
        cl = [c for c in ce.flowers[0] if c.orbit == g]
        lst = []
        for c in cl:
            idx = []
            for pb, du in c.partners:
                assert pb == 0
                if du not in index:
                    index[du] = len(nbs)
                    nbs.append(du)
                idx.append(index[du])
            lst.append(tuple(idx))
        orbits.append((o.size, lst))
    return nbs, orbits


def render(ce, name="gen_fcc") -> str:
    nbs, orbits = topology(ce)
    L = []
    L.append("// GENERATED by casmcode_clexmonte_gb300/codegen.py -- do not edit.")
    L.append("// Site evaluator of the binary FCC cluster expansion: point, pairs to the")
    L.append("// third neighbour shell, triplets with all edges up to the second shell.")
    L.append("#pragma once")
    L.append("#include <cstdint>")
    L.append("namespace cem {")
    L.append(f"namespace {name} {{")
    L.append(f"constexpr int N_NB = {len(nbs)};")
    L.append(f"constexpr int N_ORBITS = {len(orbits)};")
    L.append("constexpr int ORBIT_SIZE[N_ORBITS] = {" + ", ".join(str(s) for s, _ in orbits) + "};")
    L.append("constexpr int ORBIT_CLUSTERS[N_ORBITS] = {" + ", ".join(str(len(c)) for _, c in orbits) + "};")
    L.append("// neighbour cell offsets (dx, dy, dz)")
    L.append("constexpr int NB[N_NB][3] = {")
    L.append("    " + ", ".join("{%d, %d, %d}" % tuple(d) for d in nbs) + "};")
    L.append("// per orbit: partner neighbour indices of every flower cluster")
    flat = []
    for g, (size, cl) in enumerate(orbits):
        for c in cl:
            flat.append((g, c))
    L.append(f"constexpr int N_CL = {len(flat)};")
    L.append("constexpr int CL_ORBIT[N_CL] = {" + ", ".join(str(g) for g, _ in flat) + "};")
    L.append("constexpr int CL_P[N_CL][3] = {" + ", ".join(
        "{%s}" % ", ".join(str(x) for x in (list(c) + [-1] * (3 - len(c)))) for _, c in flat) + "};")
    L.append("// copies in constant memory for run-time indexing on the device")
    L.append("static __constant__ int NB_D[N_NB][3] = {")
    L.append("    " + ", ".join("{%d, %d, %d}" % tuple(d) for d in nbs) + "};")
    L.append("static __constant__ int CL_ORBIT_D[N_CL] = {" + ", ".join(str(g) for g, _ in flat) + "};")
    L.append("static __constant__ int CL_P_D[N_CL][3] = {" + ", ".join(
        "{%s}" % ", ".join(str(x) for x in (list(c) + [-1] * (3 - len(c)))) for _, c in flat) + "};")
    L.append("")
    L.append("// counts[g] = number of clusters of orbit g whose partners are all 1")
    L.append("template <int P>")
    L.append("__device__ __forceinline__ void counts(const int8_t *__restrict__ c, int (&n)[N_ORBITS]) {")
    for k, d in enumerate(nbs):
        L.append(f"  const int v{k} = c[({d[0]}) + P * ({d[1]}) + P * P * ({d[2]})];")
    for g, (size, cl) in enumerate(orbits):
        if size == 1:
            L.append(f"  n[{g}] = 1;")
            continue
        terms = []
        for c in cl:
            terms.append(" & ".join(f"v{k}" for k in c) if len(c) > 1 else f"v{c[0]}")
        expr = " + ".join(f"({t})" if "&" in t else t for t in terms)
        L.append(f"  n[{g}] = {expr};")
    L.append("}")
    L.append("")
    L.append("// the same counts, and the neighbour occupants packed into env (bit k =")
    L.append("// neighbour k), the input of the proposal network")
    L.append("template <int P>")
    L.append("__device__ __forceinline__ void counts_env(const int8_t *__restrict__ c, int (&n)[N_ORBITS],")
    L.append("                                           unsigned long long &env) {")
    for k, d in enumerate(nbs):
        L.append(f"  const int v{k} = c[({d[0]}) + P * ({d[1]}) + P * P * ({d[2]})];")
    for g, (size, cl) in enumerate(orbits):
        if size == 1:
            L.append(f"  n[{g}] = 1;")
            continue
        terms = []
        for c in cl:
            terms.append(" & ".join(f"v{k}" for k in c) if len(c) > 1 else f"v{c[0]}")
        expr = " + ".join(f"({t})" if "&" in t else t for t in terms)
        L.append(f"  n[{g}] = {expr};")
    lo = " | ".join(f"((unsigned)v{k} << {k})" for k in range(min(32, len(nbs))))
    hi = " | ".join(f"((unsigned)v{k} << {k - 32})" for k in range(32, len(nbs))) or "0u"
    L.append(f"  const unsigned lo = {lo};")
    L.append(f"  const unsigned hi = {hi};")
    L.append("  env = ((unsigned long long)hi << 32) | lo;")
    L.append("}")
    L.append("")
    # owned clusters: anchored at the site (its lexicographically smallest
    # point), so every periodic cluster is counted once over all sites
    index = {tuple(d): k for k, d in enumerate(nbs)}
    owned = [[] for _ in orbits]
    for c in ce.owned[0]:
        owned[c.orbit].append(tuple(index[tuple(du)] for _, du in c.partners))
    used = sorted({k for cl in owned for c in cl for k in c})
    L.append("// owned[g] = number of clusters of orbit g anchored at this site (its")
    L.append("// lexicographically smallest point) whose other sites are all 1")
    L.append("template <int P>")
    L.append("__device__ __forceinline__ void owned_counts(const int8_t *__restrict__ c,")
    L.append("                                             int (&n)[N_ORBITS]) {")
    for k in used:
        d = nbs[k]
        L.append(f"  const int v{k} = c[({d[0]}) + P * ({d[1]}) + P * P * ({d[2]})];")
    for g, cl in enumerate(owned):
        if orbits[g][0] == 1:
            L.append(f"  n[{g}] = 1;")
            continue
        terms = []
        for c in cl:
            terms.append(" & ".join(f"v{k}" for k in c) if len(c) > 1 else f"v{c[0]}")
        expr = " + ".join(f"({t})" if "&" in t else t for t in terms) if terms else "0"
        L.append(f"  n[{g}] = {expr};")
    L.append("}")
    L.append("")
    L.append(f"}}  // namespace {name}")
    L.append("}  // namespace cem")
    return "\n".join(L) + "\n"


def fcc_binary_header() -> str:
    from .workloads import fcc_binary_ce

    return render(fcc_binary_ce(0))


if __name__ == "__main__":
    with open(OUT, "w") as f:
        f.write(fcc_binary_header())
    print(OUT)
