// Golden-vector probe: drives the reference's generated FCC Clexulator
// (tests/unit/clexmonte/data/FCC_binary_vacancy/basis_sets/bset.default/
// FCC_binary_vacancy_Clexulator_default.cc, compiled where it lies against the
// shim in oracle/ref_shim) on seeded random configurations of an L x L x L
// supercell of the FCC primitive cell, and prints JSON with:
//  * the neighbour-list order used (unit cells sorted by r^T W r, then
//    lexicographically, W = the Clexulator's weight matrix);
//  * global correlations per unit cell (sum of _calc_global_corr_contribution
//    over unit cells / n_uc);
//  * delta point correlations (_calc_delta_point_corr) for random changes.
// Site index l = i + L*(j + L*k).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "casm/clexulator/BaseClexulator.hh"

extern "C" CASM::clexulator::BaseClexulator *make_FCC_binary_vacancy_Clexulator_default();

int main(int argc, char **argv) {
  int L = argc > 1 ? atoi(argv[1]) : 6;
  int n_cfg = argc > 2 ? atoi(argv[2]) : 4;
  int n_delta = argc > 3 ? atoi(argv[3]) : 32;
  unsigned long seed = argc > 4 ? strtoul(argv[4], nullptr, 10) : 12345;
  auto *clex = make_FCC_binary_vacancy_Clexulator_default();
  std::vector<CASM::xtal::UnitCell> nb(clex->neighborhood().begin(), clex->neighborhood().end());
  auto w = [&](const CASM::xtal::UnitCell &u) {
    long r[3] = {u.i, u.j, u.k};
    long s = 0;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) s += r[a] * clex->weight(a, b) * r[b];
    return s;
  };
  std::stable_sort(nb.begin(), nb.end(), [&](auto &a, auto &b) {
    long wa = w(a), wb = w(b);
    if (wa != wb) return wa < wb;
    return a < b;
  });
  int n = L * L * L, ncorr = (int)clex->corr_size(), nn = (int)nb.size();
  auto idx = [&](long i, long j, long k) {
    auto m = [&](long a) { return (int)(((a % L) + L) % L); };
    return m(i) + L * (m(j) + L * m(k));
  };
  std::mt19937_64 eng(seed);
  std::printf("{\"L\": %d, \"nlist\": [", L);
  for (int q = 0; q < nn; ++q) std::printf("%s[%ld, %ld, %ld]", q ? ", " : "", nb[q].i, nb[q].j, nb[q].k);
  std::printf("], \"cases\": [");
  std::vector<int> occ(n);
  std::vector<long> nlist(nn);
  std::vector<double> c(ncorr), tot(ncorr);
  for (int cfg = 0; cfg < n_cfg; ++cfg) {
    for (int l = 0; l < n; ++l) occ[l] = (int)(eng() % 3);
    std::fill(tot.begin(), tot.end(), 0.0);
    for (int k = 0; k < L; ++k)
      for (int j = 0; j < L; ++j)
        for (int i = 0; i < L; ++i) {
          for (int q = 0; q < nn; ++q) nlist[q] = idx(i + nb[q].i, j + nb[q].j, k + nb[q].k);
          clex->set_pointers(occ.data(), nlist.data());
          clex->global_corr(c.data());
          for (int f = 0; f < ncorr; ++f) tot[f] += c[f];
        }
    std::printf("%s{\"occ\": [", cfg ? ", " : "");
    for (int l = 0; l < n; ++l) std::printf("%s%d", l ? ", " : "", occ[l]);
    std::printf("], \"corr\": [");
    for (int f = 0; f < ncorr; ++f) std::printf("%s%.17g", f ? ", " : "", tot[f] / n);
    std::printf("], \"deltas\": [");
    for (int d = 0; d < n_delta; ++d) {
      int l = (int)(eng() % n);
      int occ_f = (int)(eng() % 3);
      if (occ_f == occ[l]) occ_f = (occ_f + 1) % 3;
      int i = l % L, j = (l / L) % L, k = l / (L * L);
      for (int q = 0; q < nn; ++q) nlist[q] = idx(i + nb[q].i, j + nb[q].j, k + nb[q].k);
      clex->set_pointers(occ.data(), nlist.data());
      clex->delta_point_corr(0, occ[l], occ_f, c.data());
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
