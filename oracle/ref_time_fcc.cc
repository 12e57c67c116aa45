// Timing probe: single-core rate of the reference's generated FCC Clexulator
// (tests/unit/clexmonte/data/FCC_binary_vacancy/basis_sets/bset.default/
// FCC_binary_vacancy_Clexulator_default.cc, compiled where it lies against the
// shim in oracle/ref_shim) evaluating the energy change of single-site
// occupation changes: delta_point_corr (its _calc_delta_point_corr) followed
// by the ECI dot, the work occ_delta_value does per changed site
// (CanonicalCalculator.cc:137-140). Neighbour lists are precomputed per site
// (the role of the reference's SuperNeighborList), so only the evaluation is
// timed. Prints JSON: evaluations per second on one thread.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "casm/clexulator/BaseClexulator.hh"

extern "C" CASM::clexulator::BaseClexulator *make_FCC_binary_vacancy_Clexulator_default();

int main(int argc, char **argv) {
  const int L = argc > 1 ? atoi(argv[1]) : 24;
  const long n_eval = argc > 2 ? atol(argv[2]) : 2000000;
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
  const int n = L * L * L, nn = (int)nb.size(), ncorr = (int)clex->corr_size();
  auto idx = [&](long i, long j, long k) {
    auto m = [&](long a) { return (long)(((a % L) + L) % L); };
    return m(i) + L * (m(j) + L * m(k));
  };
  std::vector<long> nlist((size_t)n * nn);
  for (int l = 0; l < n; ++l) {
    const int i = l % L, j = (l / L) % L, k = l / (L * L);
    for (int q = 0; q < nn; ++q) nlist[(size_t)l * nn + q] = idx(i + nb[q].i, j + nb[q].j, k + nb[q].k);
  }
  std::mt19937_64 eng(7);
  std::vector<int> occ(n);
  for (int l = 0; l < n; ++l) occ[l] = (int)(eng() % 3);
  std::vector<double> eci(ncorr), c(ncorr);
  for (int f = 0; f < ncorr; ++f) eci[f] = 0.01 * ((double)(long)(eng() % 200) - 100.0) / 100.0;
  std::vector<int> sites(n_eval), newocc(n_eval);
  for (long e = 0; e < n_eval; ++e) {
    sites[e] = (int)(eng() % n);
    int f = (int)(eng() % 3);
    if (f == occ[sites[e]]) f = (f + 1) % 3;
    newocc[e] = f;
  }
  double sink = 0.0;
  const auto t0 = std::chrono::steady_clock::now();
  for (long e = 0; e < n_eval; ++e) {
    const int l = sites[e];
    clex->set_pointers(occ.data(), nlist.data() + (size_t)l * nn);
    clex->delta_point_corr(0, occ[l], newocc[e], c.data());
    double de = 0.0;
    for (int f = 0; f < ncorr; ++f) de += eci[f] * c[f];
    sink += de;
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("{\"L\": %d, \"evaluations\": %ld, \"seconds\": %.6f, \"evaluations_per_s\": %.6e, "
              "\"checksum\": %.17g}\n", L, n_eval, secs, (double)n_eval / secs, sink);
  delete clex;
  return 0;
}
