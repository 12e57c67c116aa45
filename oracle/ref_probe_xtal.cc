// Golden-vector probe for a generated Clexulator whose occupation degree of
// freedom lives on several sublattices (the reference's
// tests/unit/clexmonte/data/Clex_ZrO_Occ/basis_sets/bset.formation_energy/
// ZrO_Clexulator_formation_energy.cc, compiled where it lies against the shim
// in oracle/ref_shim; the factory is named by -DPROBE_FACTORY).
//
// Neighbour list: every unit cell r with r^T W r at most the largest weight
// in the Clexulator's neighbourhood (W = its weight matrix), sorted by weight
// then lexicographically; nlist index = cell position * n_sub + position of
// the site's sublattice among the Clexulator's sublattice indices. Sites of
// an L0 x L1 x L2 supercell are numbered l = s * n_uc + i + L0 * (j + L1 * k)
// over those sublattices (s = position), and occupants 0 .. n_occ-1 index each
// sublattice's occupant list.
//
// Prints JSON: the sublattice indices, the neighbour-list cells, then per
// seeded random configuration the occupations, the global correlations per
// unit cell (sum of _calc_global_corr_contribution over cells / n_uc) and the
// delta point correlations (_calc_delta_point_corr) of random changes.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "casm/clexulator/BaseClexulator.hh"

#ifndef PROBE_FACTORY
#error "define PROBE_FACTORY as the Clexulator's factory function"
#endif

extern "C" CASM::clexulator::BaseClexulator *PROBE_FACTORY();

int main(int argc, char **argv) {
  const int L0 = argc > 1 ? atoi(argv[1]) : 8;
  const int L1 = argc > 2 ? atoi(argv[2]) : 8;
  const int L2 = argc > 3 ? atoi(argv[3]) : 6;
  const int n_cfg = argc > 4 ? atoi(argv[4]) : 3;
  const int n_delta = argc > 5 ? atoi(argv[5]) : 40;
  const unsigned long seed = argc > 6 ? strtoul(argv[6], nullptr, 10) : 12345;
  const int n_occ = argc > 7 ? atoi(argv[7]) : 2;
  auto *clex = PROBE_FACTORY();
  std::vector<int> sub(clex->sublat_indices().begin(), clex->sublat_indices().end());
  const int n_sub = (int)sub.size();
  auto w = [&](long i, long j, long k) {
    long r[3] = {i, j, k};
    long s = 0;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) s += r[a] * clex->weight(a, b) * r[b];
    return s;
  };
  long wmax = 0, rmax = 0;
  for (auto &u : clex->neighborhood()) {
    wmax = std::max(wmax, w(u.i, u.j, u.k));
    rmax = std::max({rmax, std::labs(u.i), std::labs(u.j), std::labs(u.k)});
  }
  struct Cell {
    long w, i, j, k;
  };
  std::vector<Cell> cells;
  const long box = rmax + 6;
  for (long i = -box; i <= box; ++i)
    for (long j = -box; j <= box; ++j)
      for (long k = -box; k <= box; ++k)
        if (w(i, j, k) <= wmax) cells.push_back({w(i, j, k), i, j, k});
  std::sort(cells.begin(), cells.end(), [](const Cell &a, const Cell &b) {
    if (a.w != b.w) return a.w < b.w;
    if (a.i != b.i) return a.i < b.i;
    if (a.j != b.j) return a.j < b.j;
    return a.k < b.k;
  });
  const int nn = (int)cells.size() * n_sub;
  if (nn < (int)clex->nlist_size()) {
    std::fprintf(stderr, "neighbour list shorter than the Clexulator's nlist_size\n");
    return 1;
  }
  const int n_uc = L0 * L1 * L2, n = n_uc * n_sub, ncorr = (int)clex->corr_size();
  auto idx = [&](int s, long i, long j, long k) {
    auto m = [](long a, int L) { return (long)(((a % L) + L) % L); };
    return (long)s * n_uc + m(i, L0) + L0 * (m(j, L1) + L1 * m(k, L2));
  };
  std::vector<long> nlist(nn);
  auto set_cell = [&](long i, long j, long k) {
    for (int c = 0; c < (int)cells.size(); ++c)
      for (int s = 0; s < n_sub; ++s)
        nlist[c * n_sub + s] = idx(s, i + cells[c].i, j + cells[c].j, k + cells[c].k);
  };
  std::mt19937_64 eng(seed);
  std::printf("{\"L\": [%d, %d, %d], \"sublat\": [", L0, L1, L2);
  for (int s = 0; s < n_sub; ++s) std::printf("%s%d", s ? ", " : "", sub[s]);
  std::printf("], \"n_cells\": %d, \"nlist_size\": %u, \"cases\": [", (int)cells.size(),
              clex->nlist_size());
  std::vector<int> occ(n);
  std::vector<double> c(ncorr), tot(ncorr);
  for (int cfg = 0; cfg < n_cfg; ++cfg) {
    for (int l = 0; l < n; ++l) occ[l] = (int)(eng() % (unsigned)n_occ);
    std::fill(tot.begin(), tot.end(), 0.0);
    for (int k = 0; k < L2; ++k)
      for (int j = 0; j < L1; ++j)
        for (int i = 0; i < L0; ++i) {
          set_cell(i, j, k);
          clex->set_pointers(occ.data(), nlist.data());
          clex->global_corr(c.data());
          for (int f = 0; f < ncorr; ++f) tot[f] += c[f];
        }
    std::printf("%s{\"occ\": [", cfg ? ", " : "");
    for (int l = 0; l < n; ++l) std::printf("%s%d", l ? ", " : "", occ[l]);
    std::printf("], \"corr\": [");
    for (int f = 0; f < ncorr; ++f) std::printf("%s%.17g", f ? ", " : "", tot[f] / n_uc);
    std::printf("], \"deltas\": [");
    for (int d = 0; d < n_delta; ++d) {
      const int l = (int)(eng() % (unsigned)n);
      int occ_f = (int)(eng() % (unsigned)n_occ);
      if (occ_f == occ[l]) occ_f = (occ_f + 1) % n_occ;
      const int s = l / n_uc, uc = l % n_uc;
      const int i = uc % L0, j = (uc / L0) % L1, k = uc / (L0 * L1);
      set_cell(i, j, k);
      clex->set_pointers(occ.data(), nlist.data());
      clex->delta_point_corr(s, occ[l], occ_f, c.data());
      std::printf("%s{\"site\": %d, \"occ_f\": %d, \"dcorr\": [", d ? ", " : "", l, occ_f);
      for (int f = 0; f < ncorr; ++f) std::printf("%s%.17g", f ? ", " : "", c[f]);
      std::printf("]}");
    }
    std::printf("]}");
  }
  std::printf("]}\n");
  delete clex;
  return 0;
}
