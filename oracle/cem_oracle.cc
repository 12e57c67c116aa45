// CPU FP64 oracle for the cluster-expansion Metropolis hot path.
//
// TEST INFRASTRUCTURE ONLY. The GPU results are compared against this file:
// it is linked and called by tests/, by __graft_entry__.smoke() and by
// bench.py's CPU-baseline leg,
// never by the product library. It restates, independently of the product's
// table builder, the arithmetic of the reference's hot path:
//
//  * cluster-expansion energy and delta correlations of the occupation basis
//    (libcasm-clexulator, not vendored; semantics as in the generated
//    Clexulator tests/unit/clexmonte/data/FCC_binary_vacancy/basis_sets/
//    bset.default/FCC_binary_vacancy_Clexulator_default.cc:306-311 (site
//    functions), :555-580 (delta point correlations), :1054-1060 (per-orbit
//    division by the multiplicity));
//  * the canonical and semi-grand canonical potentials
//    (src/casm/clexmonte/monte_calculator/CanonicalCalculator.cc:137-140,
//    SemiGrandCanonicalCalculator.cc:186-213);
//  * the Metropolis loop occupation_metropolis_v2
//    (include/casm/clexmonte/methods/occupation_metropolis.hh:72-123) with a
//    std::mt19937_64 engine (canonical/canonical.hh:139) and the event
//    proposal / acceptance / occupant-location steps of libcasm-monte, which
//    is not vendored and is restated here (see propose_* and accept_metropolis
//    below);
//  * variance / covariance analyses (src/casm/clexmonte/monte_calculator/
//    analysis_functions.cc:17-173, run/io/convariance_functions.cc:29-146).
//
// Clusters are enumerated here from the lattice and the per-size maximum
// lengths, and each decorated cluster is identified by a geometric invariant
// (sorted edge list with squared lengths and species pairs), not by the
// product's symmetry tables. Orbit multiplicities are counted here. Crystals
// whose orbits such invariants do not separate (several sublattices, e.g.
// the reference's Clex_ZrO_Occ prim) go through ora_system_create_xtal: the
// factor group is searched here and clusters are keyed by canonical forms.

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

using i64 = long long;
using u64 = unsigned long long;

std::string g_err;

struct Vec3 {
  i64 x, y, z;
};

inline i64 sq(const Vec3 &a, const Vec3 &b) {
  i64 dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + dy * dy + dz * dz;
}

bool lex_less(const Vec3 &a, const Vec3 &b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}

// Decorated-cluster invariant: (size, sorted edges (d2, min occ, max occ),
// sorted occupants) flattened into a vector key.
std::vector<i64> invariant(const std::vector<Vec3> &p, const std::vector<int> &occ) {
  int n = (int)p.size();
  std::vector<std::array<i64, 3>> e;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      e.push_back({sq(p[i], p[j]), (i64)std::min(occ[i], occ[j]),
                   (i64)std::max(occ[i], occ[j])});
  std::sort(e.begin(), e.end());
  std::vector<int> o(occ.begin(), occ.end());
  std::sort(o.begin(), o.end());
  std::vector<i64> key;
  key.push_back(n);
  for (auto &x : e) key.insert(key.end(), x.begin(), x.end());
  for (int v : o) key.push_back(v);
  return key;
}

struct AnchorType {  // cluster shape anchored at basis site b, uc (0,0,0)
  int size;
  int orbit;               // oracle orbit id (undecorated invariant)
  int b[4];                // sublattice of each site (site 0 = anchor)
  i64 du[4][3];            // unit cell offset of each site
  std::vector<int> lut;    // n_occ^size decoration code -> function (-1: none)
};

struct System {
  int n_basis = 1, n_occ = 2;
  i64 lat[3][3];
  std::vector<Vec3> basis;
  double grid = 1.0;
  int L[3] = {1, 1, 1};
  // supercell in lower-triangular Hermite normal form: lattice columns
  // (L0, tw0, tw1), (0, L1, tw2), (0, 0, L2); zeros for a diagonal supercell
  int tw[3] = {0, 0, 0};
  int n_uc = 1, n_sites = 1;
  int n_funcs = 1;
  std::vector<double> eci, coeff, mult, weight;  // weight = eci*coeff/mult
  std::vector<int> func_orbit;
  std::vector<std::vector<AnchorType>> types;  // per basis site
  // supercell clusters
  std::vector<int> cl_type_b, cl_type_i;  // (anchor b, type index)
  std::vector<int> cl_sites;              // 4 per cluster
  std::vector<int> inc_off, inc_cl, inc_pos;  // incidence CSR over sites
  std::vector<double> RT;  // (n_occ-1) x n_occ, param composition per mol change
  double n_orbits = 0;
  struct Cl {
    const int *lut;
    int size;
    int sites[4];
  };
  std::vector<Cl> cls;  // flattened view of the supercell clusters
  struct Inc {            // a cluster seen from one of its sites (CSR by site)
    const int *lut;
    int size, pos;
    int sites[4];
  };
  std::vector<Inc> inc;
};

Vec3 cart(const System &s, int b, i64 u0, i64 u1, i64 u2) {
  Vec3 v;
  v.x = u0 * s.lat[0][0] + u1 * s.lat[1][0] + u2 * s.lat[2][0] + s.basis[b].x;
  v.y = u0 * s.lat[0][1] + u1 * s.lat[1][1] + u2 * s.lat[2][1] + s.basis[b].y;
  v.z = u0 * s.lat[0][2] + u1 * s.lat[1][2] + u2 * s.lat[2][2] + s.basis[b].z;
  return v;
}

// Cell (i, j, k) reduced into the Hermite-normal-form box: subtract the
// first lattice column until 0 <= i < L0, then the second until
// 0 <= j < L1, then the third; cells are numbered i + L0 (j + L1 k).
inline int site_index(const System &s, int b, i64 i, i64 j, i64 k) {
  auto fdiv = [](i64 a, i64 n) { return (a - (((a % n) + n) % n)) / n; };
  i64 q = fdiv(i, s.L[0]);
  i -= q * s.L[0];
  j -= q * s.tw[0];
  k -= q * s.tw[1];
  q = fdiv(j, s.L[1]);
  j -= q * s.L[1];
  k -= q * s.tw[2];
  k -= fdiv(k, s.L[2]) * s.L[2];
  return b * s.n_uc + (int)(i + s.L[0] * (j + s.L[1] * k));
}

void finish_build(System &s, const std::vector<double> &orbit_count);

void build(System &s, const double *max_length /*[5], index = size*/,
           const int *func_size, const i64 *func_pts /*n_funcs*4*3*/,
           const int *func_occ /*n_funcs*4*/) {
  // 1. function invariants -> function index; undecorated orbit invariants
  std::map<std::vector<i64>, int> fmap, omap;
  s.func_orbit.assign(s.n_funcs, -1);
  for (int f = 1; f < s.n_funcs; ++f) {
    int n = func_size[f];
    std::vector<Vec3> p(n);
    std::vector<int> o(n), z(n, 0);
    for (int i = 0; i < n; ++i) {
      p[i] = {func_pts[(f * 4 + i) * 3 + 0], func_pts[(f * 4 + i) * 3 + 1],
              func_pts[(f * 4 + i) * 3 + 2]};
      o[i] = func_occ[f * 4 + i];
    }
    auto key = invariant(p, o);
    if (fmap.count(key)) throw std::runtime_error("two functions share an invariant");
    fmap[key] = f;
    auto okey = invariant(p, z);
    if (!omap.count(okey)) {
      int id = (int)omap.size();
      omap[okey] = id;
    }
    s.func_orbit[f] = omap[okey];
  }
  int n_orbit = (int)omap.size();
  // 2. anchored cluster shapes per basis site, by enumeration
  double rmax = 0;
  for (int n = 2; n <= 4; ++n) rmax = std::max(rmax, max_length[n]);
  const double tol = 1e-5;
  s.types.assign(s.n_basis, {});
  std::vector<double> orbit_count(n_orbit, 0.0);
  // inverse of lattice for site lookup not needed: enumerate (b,u) directly
  int R = (int)std::ceil(rmax / s.grid) + 2;
  for (int b = 0; b < s.n_basis; ++b) {
    Vec3 c0 = cart(s, b, 0, 0, 0);
    struct Nb {
      Vec3 c;
      int b;
      i64 u[3];
    };
    std::vector<Nb> nb;
    for (i64 u0 = -R; u0 <= R; ++u0)
      for (i64 u1 = -R; u1 <= R; ++u1)
        for (i64 u2 = -R; u2 <= R; ++u2)
          for (int bb = 0; bb < s.n_basis; ++bb) {
            Vec3 c = cart(s, bb, u0, u1, u2);
            i64 d2 = sq(c, c0);
            if (d2 > 0 && d2 * s.grid * s.grid <= rmax * rmax + tol) nb.push_back({c, bb, {u0, u1, u2}});
          }
    auto add_type = [&](std::vector<int> idx) {
      int n = (int)idx.size() + 1;
      std::vector<Vec3> p(n);
      p[0] = c0;
      for (int i = 1; i < n; ++i) p[i] = nb[idx[i - 1]].c;
      double lim = max_length[n];
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
          if (sq(p[i], p[j]) * s.grid * s.grid > lim * lim + tol) return;
      for (int i = 1; i < n; ++i)
        if (lex_less(p[i], p[0])) return;  // anchor must be the smallest point
      std::vector<int> z(n, 0);
      auto okey = invariant(p, z);
      auto it = omap.find(okey);
      if (it == omap.end()) return;
      AnchorType t;
      t.size = n;
      t.orbit = it->second;
      t.b[0] = b;
      t.du[0][0] = t.du[0][1] = t.du[0][2] = 0;
      for (int i = 1; i < n; ++i) {
        t.b[i] = nb[idx[i - 1]].b;
        for (int a = 0; a < 3; ++a) t.du[i][a] = nb[idx[i - 1]].u[a];
      }
      int ncode = 1;
      for (int i = 0; i < n; ++i) ncode *= s.n_occ;
      t.lut.assign(ncode, -1);
      std::vector<int> occ(n);
      for (int code = 0; code < ncode; ++code) {
        int c = code;
        bool all_nonref = true;
        for (int i = 0; i < n; ++i) {
          occ[i] = c % s.n_occ;
          c /= s.n_occ;
          if (occ[i] == 0) all_nonref = false;
        }
        if (!all_nonref) continue;
        auto key = invariant(p, occ);
        auto f = fmap.find(key);
        if (f == fmap.end()) throw std::runtime_error("decorated cluster has no function");
        t.lut[code] = f->second;
      }
      orbit_count[t.orbit] += 1.0;
      s.types[b].push_back(t);
    };
    // point
    {
      std::vector<Vec3> p{c0};
      std::vector<int> z{0};
      auto it = omap.find(invariant(p, z));
      if (it != omap.end()) {
        AnchorType t;
        t.size = 1;
        t.orbit = it->second;
        t.b[0] = b;
        t.du[0][0] = t.du[0][1] = t.du[0][2] = 0;
        t.lut.assign(s.n_occ, -1);
        for (int o = 1; o < s.n_occ; ++o) {
          std::vector<int> oo{o};
          auto f = fmap.find(invariant(p, oo));
          if (f == fmap.end()) throw std::runtime_error("point function missing");
          t.lut[o] = f->second;
        }
        orbit_count[t.orbit] += 1.0;
        s.types[b].push_back(t);
      }
    }
    int m = (int)nb.size();
    for (int i = 0; i < m; ++i) {
      if (max_length[2] > 0) add_type({i});
      for (int j = i + 1; j < m; ++j) {
        if (max_length[3] > 0) add_type({i, j});
        if (max_length[4] > 0)
          for (int k = j + 1; k < m; ++k) add_type({i, j, k});
      }
    }
  }
  finish_build(s, orbit_count);
}

// Multiplicities, weights, supercell clusters and their incidence lists, from
// the anchored cluster types of every basis site.
void finish_build(System &s, const std::vector<double> &orbit_count) {
  // 3. multiplicities, weights
  s.mult.assign(s.n_funcs, 1.0);
  s.weight.assign(s.n_funcs, 0.0);
  for (int f = 1; f < s.n_funcs; ++f) {
    s.mult[f] = orbit_count[s.func_orbit[f]];
    if (s.mult[f] <= 0) throw std::runtime_error("orbit with no cluster in the crystal");
    s.weight[f] = s.eci[f] * s.coeff[f] / s.mult[f];
  }
  s.weight[0] = s.eci[0];
  // 4. supercell clusters and incidence
  s.n_uc = s.L[0] * s.L[1] * s.L[2];
  s.n_sites = s.n_uc * s.n_basis;
  s.cl_sites.clear();
  s.cl_type_b.clear();
  s.cl_type_i.clear();
  for (int b = 0; b < s.n_basis; ++b)
    for (int k = 0; k < s.L[2]; ++k)
      for (int j = 0; j < s.L[1]; ++j)
        for (int i = 0; i < s.L[0]; ++i)
          for (int ti = 0; ti < (int)s.types[b].size(); ++ti) {
            const AnchorType &t = s.types[b][ti];
            for (int q = 0; q < 4; ++q) {
              if (q < t.size)
                s.cl_sites.push_back(site_index(s, t.b[q], i + t.du[q][0],
                                                j + t.du[q][1], k + t.du[q][2]));
              else
                s.cl_sites.push_back(-1);
            }
            s.cl_type_b.push_back(b);
            s.cl_type_i.push_back(ti);
          }
  int ncl = (int)s.cl_type_b.size();
  std::vector<int> cnt(s.n_sites + 1, 0);
  for (int c = 0; c < ncl; ++c)
    for (int q = 0; q < 4; ++q) {
      int site = s.cl_sites[c * 4 + q];
      if (site >= 0) cnt[site + 1]++;
    }
  for (int i = 0; i < s.n_sites; ++i) cnt[i + 1] += cnt[i];
  s.inc_off = cnt;
  s.inc_cl.assign(cnt.back(), 0);
  s.inc_pos.assign(cnt.back(), 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int c = 0; c < ncl; ++c)
    for (int q = 0; q < 4; ++q) {
      int site = s.cl_sites[c * 4 + q];
      if (site < 0) continue;
      for (int q2 = 0; q2 < q; ++q2)
        if (s.cl_sites[c * 4 + q2] == site)
          throw std::runtime_error("supercell too small: a cluster contains a site twice");
      s.inc_cl[fill[site]] = c;
      s.inc_pos[fill[site]] = q;
      fill[site]++;
    }
  s.cls.resize(ncl);
  for (int c = 0; c < ncl; ++c) {
    const AnchorType &t = s.types[s.cl_type_b[c]][s.cl_type_i[c]];
    s.cls[c].lut = t.lut.data();
    s.cls[c].size = t.size;
    for (int q = 0; q < 4; ++q) s.cls[c].sites[q] = s.cl_sites[c * 4 + q];
  }
  s.inc.resize(s.inc_cl.size());
  for (size_t e = 0; e < s.inc_cl.size(); ++e) {
    const System::Cl &k = s.cls[s.inc_cl[e]];
    s.inc[e].lut = k.lut;
    s.inc[e].size = k.size;
    s.inc[e].pos = s.inc_pos[e];
    for (int q = 0; q < 4; ++q) s.inc[e].sites[q] = k.sites[q];
  }
}

// ---- general crystals (any lattice; several sublattices, each with its own
// occupant list). Written independently of the product's table builder:
// the factor group is searched here from the lattice and the basis, and
// clusters are identified by their canonical form under it (the smallest,
// over the operations, of the sorted integral sites (i, j, k, b, label)
// translated so that the first site is in cell 0), since distance lists do
// not separate the orbits of such crystals.
struct XOp {
  int R[3][3];
  std::vector<int> perm;
  std::vector<std::array<i64, 3>> d;
};

std::vector<XOp> xtal_factor_group(const double *lat, int nb, const double *frac, const int *kind,
                                   double tol) {
  double G[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      G[a][b] = 0;
      for (int c = 0; c < 3; ++c) G[a][b] += lat[a * 3 + c] * lat[b * 3 + c];
    }
  double scale = 1.0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) scale = std::max(scale, std::fabs(G[a][b]));
  std::vector<XOp> ops;
  for (int code = 0; code < 19683; ++code) {
    int R[3][3], c = code;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        R[a][b] = c % 3 - 1;
        c /= 3;
      }
    const int det = R[0][0] * (R[1][1] * R[2][2] - R[1][2] * R[2][1]) -
                    R[0][1] * (R[1][0] * R[2][2] - R[1][2] * R[2][0]) +
                    R[0][2] * (R[1][0] * R[2][1] - R[1][1] * R[2][0]);
    if (det != 1 && det != -1) continue;
    bool metric = true;  // R^T G R == G
    for (int a = 0; a < 3 && metric; ++a)
      for (int b = 0; b < 3 && metric; ++b) {
        double v = 0;
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q) v += R[p][a] * G[p][q] * R[q][b];
        if (std::fabs(v - G[a][b]) > tol * scale) metric = false;
      }
    if (!metric) continue;
    std::vector<std::array<double, 3>> rf(nb);
    for (int b = 0; b < nb; ++b)
      for (int a = 0; a < 3; ++a)
        rf[b][a] = R[a][0] * frac[b * 3] + R[a][1] * frac[b * 3 + 1] + R[a][2] * frac[b * 3 + 2];
    for (int b1 = 0; b1 < nb; ++b1) {
      if (kind[b1] != kind[0]) continue;
      double t[3];
      for (int a = 0; a < 3; ++a) t[a] = frac[b1 * 3 + a] - rf[0][a];
      XOp op;
      std::memcpy(op.R, R, sizeof(R));
      bool ok = true;
      for (int b = 0; b < nb && ok; ++b) {
        int hit = -1;
        std::array<i64, 3> dd{};
        for (int b2 = 0; b2 < nb && hit < 0; ++b2) {
          if (kind[b2] != kind[b]) continue;
          bool same = true;
          for (int a = 0; a < 3; ++a) {
            const double x = rf[b][a] + t[a] - frac[b2 * 3 + a];
            if (std::fabs(x - std::nearbyint(x)) > tol) same = false;
            dd[a] = (i64)std::nearbyint(x);
          }
          if (same) hit = b2;
        }
        if (hit < 0) ok = false;
        op.perm.push_back(hit);
        op.d.push_back(dd);
      }
      if (ok) ops.push_back(op);
    }
  }
  return ops;
}

struct XSite {
  int b;  // prim sublattice
  i64 u[3];
};

std::vector<i64> xtal_key(const std::vector<XOp> &ops, const std::vector<XSite> &sites,
                          const std::vector<int> &lab) {
  std::vector<i64> best;
  const int n = (int)sites.size();
  std::vector<std::array<i64, 5>> m(n);
  for (const XOp &op : ops) {
    for (int q = 0; q < n; ++q) {
      const XSite &s = sites[q];
      for (int a = 0; a < 3; ++a)
        m[q][a] = op.R[a][0] * s.u[0] + op.R[a][1] * s.u[1] + op.R[a][2] * s.u[2] + op.d[s.b][a];
      m[q][3] = op.perm[s.b];
      m[q][4] = lab[q];
    }
    std::sort(m.begin(), m.end());
    std::vector<i64> key;
    key.reserve(5 * n);
    for (int q = 0; q < n; ++q)
      for (int a = 0; a < 5; ++a) key.push_back(a < 3 ? m[q][a] - m[0][a] : m[q][a]);
    if (best.empty() || key < best) best = key;
  }
  return best;
}

// func_sites: per function 4 sites (prim sublattice, i, j, k); func_occ: the
// occupant (1-based site-function index + 1) on each site.
void build_xtal(System &s, const double *lat, int nb_all, const double *frac, const int *kind,
                const int *dof, const double *max_length, const int *func_size,
                const i64 *func_sites, const int *func_occ) {
  const double tol = 1e-5;
  std::vector<XOp> ops = xtal_factor_group(lat, nb_all, frac, kind, tol);
  if (ops.empty()) throw std::runtime_error("empty factor group");
  std::vector<int> kb(nb_all, -1), dof_b;
  for (int b = 0; b < nb_all; ++b)
    if (dof[b]) {
      kb[b] = (int)dof_b.size();
      dof_b.push_back(b);
    }
  if ((int)dof_b.size() != s.n_basis) throw std::runtime_error("n_basis != sublattices with dof");
  auto cart = [&](int b, const i64 *u, double *c) {
    for (int a = 0; a < 3; ++a) {
      c[a] = 0;
      for (int r = 0; r < 3; ++r) c[a] += ((double)u[r] + frac[b * 3 + r]) * lat[r * 3 + a];
    }
  };
  // 1. functions and orbits by canonical form
  std::map<std::vector<i64>, int> fmap, omap;
  s.func_orbit.assign(s.n_funcs, -1);
  for (int f = 1; f < s.n_funcs; ++f) {
    const int n = func_size[f];
    std::vector<XSite> p(n);
    std::vector<int> o(n), z(n, 0);
    for (int i = 0; i < n; ++i) {
      const i64 *q = func_sites + (f * 4 + i) * 4;
      p[i].b = (int)q[0];
      p[i].u[0] = q[1];
      p[i].u[1] = q[2];
      p[i].u[2] = q[3];
      o[i] = func_occ[f * 4 + i];
    }
    auto key = xtal_key(ops, p, o);
    if (fmap.count(key)) throw std::runtime_error("two functions share a canonical form");
    fmap[key] = f;
    auto okey = xtal_key(ops, p, z);
    if (!omap.count(okey)) {
      const int id = (int)omap.size();
      omap[okey] = id;
    }
    s.func_orbit[f] = omap[okey];
  }
  const int n_orbit = (int)omap.size();
  std::vector<double> orbit_count(n_orbit, 0.0);
  double rmax = 0;
  for (int n = 2; n <= 4; ++n) rmax = std::max(rmax, max_length[n]);
  // search box: |u_a| <= rmax * |column a of the inverse lattice| + 2
  double inv[3][3];
  {
    const double *A = lat;
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    inv[0][0] = (A[4] * A[8] - A[5] * A[7]) / det;
    inv[0][1] = (A[2] * A[7] - A[1] * A[8]) / det;
    inv[0][2] = (A[1] * A[5] - A[2] * A[4]) / det;
    inv[1][0] = (A[5] * A[6] - A[3] * A[8]) / det;
    inv[1][1] = (A[0] * A[8] - A[2] * A[6]) / det;
    inv[1][2] = (A[2] * A[3] - A[0] * A[5]) / det;
    inv[2][0] = (A[3] * A[7] - A[4] * A[6]) / det;
    inv[2][1] = (A[1] * A[6] - A[0] * A[7]) / det;
    inv[2][2] = (A[0] * A[4] - A[1] * A[3]) / det;
  }
  int box[3];
  for (int a = 0; a < 3; ++a) {
    const double nrm = std::sqrt(inv[0][a] * inv[0][a] + inv[1][a] * inv[1][a] + inv[2][a] * inv[2][a]);
    box[a] = (int)std::ceil(rmax * nrm) + 2;
  }
  s.types.assign(s.n_basis, {});
  for (int b : dof_b) {
    const i64 zero[3] = {0, 0, 0};
    double c0[3];
    cart(b, zero, c0);
    struct Nb {
      XSite site;
      double c[3];
    };
    std::vector<Nb> nb;
    for (i64 u0 = -box[0]; u0 <= box[0]; ++u0)
      for (i64 u1 = -box[1]; u1 <= box[1]; ++u1)
        for (i64 u2 = -box[2]; u2 <= box[2]; ++u2)
          for (int bb : dof_b) {
            Nb e;
            e.site.b = bb;
            e.site.u[0] = u0;
            e.site.u[1] = u1;
            e.site.u[2] = u2;
            cart(bb, e.site.u, e.c);
            double d2 = 0;
            for (int a = 0; a < 3; ++a) d2 += (e.c[a] - c0[a]) * (e.c[a] - c0[a]);
            if (d2 > 0 && std::sqrt(d2) <= rmax + tol) nb.push_back(e);
          }
    auto dist = [](const double *a, const double *b) {
      double d2 = 0;
      for (int k = 0; k < 3; ++k) d2 += (a[k] - b[k]) * (a[k] - b[k]);
      return std::sqrt(d2);
    };
    auto site_less = [](const XSite &x, const XSite &y) {  // by (i, j, k, b)
      for (int a = 0; a < 3; ++a)
        if (x.u[a] != y.u[a]) return x.u[a] < y.u[a];
      return x.b < y.b;
    };
    XSite centre{b, {0, 0, 0}};
    auto add_type = [&](const std::vector<int> &idx) {
      const int n = (int)idx.size() + 1;
      const double lim = max_length[n] + tol;
      std::vector<XSite> p(n);
      std::vector<const double *> c(n);
      p[0] = centre;
      c[0] = c0;
      for (int i = 1; i < n; ++i) {
        p[i] = nb[idx[i - 1]].site;
        c[i] = nb[idx[i - 1]].c;
      }
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
          if (dist(c[i], c[j]) > lim) return;
      for (int i = 1; i < n; ++i)
        if (site_less(p[i], p[0])) return;  // anchor = the smallest site
      std::vector<int> z(n, 0);
      auto it = omap.find(xtal_key(ops, p, z));
      if (it == omap.end()) return;
      AnchorType t;
      t.size = n;
      t.orbit = it->second;
      for (int i = 0; i < n; ++i) {
        t.b[i] = kb[p[i].b];
        for (int a = 0; a < 3; ++a) t.du[i][a] = p[i].u[a];
      }
      int ncode = 1;
      for (int i = 0; i < n; ++i) ncode *= s.n_occ;
      t.lut.assign(ncode, -1);
      std::vector<int> occ(n);
      for (int code = 0; code < ncode; ++code) {
        int cc = code;
        bool all_nonref = true;
        for (int i = 0; i < n; ++i) {
          occ[i] = cc % s.n_occ;
          cc /= s.n_occ;
          if (occ[i] == 0) all_nonref = false;
        }
        if (!all_nonref) continue;
        auto f = fmap.find(xtal_key(ops, p, occ));
        if (f == fmap.end()) throw std::runtime_error("decorated cluster has no function");
        t.lut[code] = f->second;
      }
      orbit_count[t.orbit] += 1.0;
      s.types[kb[b]].push_back(t);
    };
    add_type({});
    const int m = (int)nb.size();
    for (int i = 0; i < m; ++i) {
      if (max_length[2] > 0) add_type({i});
      for (int j = i + 1; j < m; ++j) {
        if (max_length[3] > 0) add_type({i, j});
        if (max_length[4] > 0)
          for (int k = j + 1; k < m; ++k) add_type({i, j, k});
      }
    }
  }
  finish_build(s, orbit_count);
}

inline int cluster_code(const System &s, int c, const signed char *occ, int site, int site_occ) {
  const System::Cl &k = s.cls[c];
  int code = 0, mul = 1;
  for (int q = 0; q < k.size; ++q) {
    const int st = k.sites[q];
    code += ((st == site) ? site_occ : occ[st]) * mul;
    mul *= s.n_occ;
  }
  return code;
}

// Integer count change of every function for occ[site]: occ_i -> occ_f.
void site_delta_counts(const System &s, const signed char *occ, int site, int occ_f,
                       i64 *dcount) {
  const int occ_i = occ[site];
  const int no = s.n_occ;
  for (int e = s.inc_off[site]; e < s.inc_off[site + 1]; ++e) {
    const System::Inc &k = s.inc[e];
    int rest = 0, mul = 1, mul_pos = 1;
    for (int q = 0; q < k.size; ++q) {
      if (q == k.pos)
        mul_pos = mul;
      else
        rest += occ[k.sites[q]] * mul;
      mul *= no;
    }
    const int fo = k.lut[rest + occ_i * mul_pos];
    const int fn = k.lut[rest + occ_f * mul_pos];
    if (fo >= 0) dcount[fo] -= 1;
    if (fn >= 0) dcount[fn] += 1;
  }
}

double counts_to_energy(const System &s, const i64 *count) {
  double e = s.weight[0] * s.n_uc;
  for (int f = 1; f < s.n_funcs; ++f) e += s.weight[f] * (double)count[f];
  return e;
}

void all_counts(const System &s, const signed char *occ, i64 *count) {
  for (int f = 0; f < s.n_funcs; ++f) count[f] = 0;
  const int ncl = (int)s.cls.size();
  for (int c = 0; c < ncl; ++c) {
    const int f = s.cls[c].lut[cluster_code(s, c, occ, -1, 0)];
    if (f >= 0) count[f] += 1;
  }
}

// ---- event delta with the reference's sequential semantics: each change is
// applied before the next is evaluated (canonical/canonical.hh:42-45).
// Energy change of a series of site changes applied in order (the state is
// restored); saved holds the n previous occupants.
double event_delta_into(const System &s, std::vector<signed char> &occ, int n, const i64 *sites,
                        const int *new_occ, i64 *dcount, signed char *saved) {
  thread_local std::vector<i64> d;
  d.assign(s.n_funcs, 0);
  for (int i = 0; i < n; ++i) {
    saved[i] = occ[sites[i]];
    site_delta_counts(s, occ.data(), (int)sites[i], new_occ[i], d.data());
    occ[sites[i]] = (signed char)new_occ[i];
  }
  for (int i = n - 1; i >= 0; --i) occ[sites[i]] = saved[i];
  double de = 0.0;
  for (int f = 1; f < s.n_funcs; ++f) de += s.weight[f] * (double)d[f];
  if (dcount)
    for (int f = 0; f < s.n_funcs; ++f) dcount[f] = d[f];
  return de;
}

double event_delta(const System &s, std::vector<signed char> &occ, int n, const i64 *sites,
                   const int *new_occ, i64 *dcount) {
  if (n > 4) {  // longer events (tests): a heap buffer
    std::vector<signed char> saved(n);
    return event_delta_into(s, occ, n, sites, new_occ, dcount, saved.data());
  }
  signed char saved[4];
  return event_delta_into(s, occ, n, sites, new_occ, dcount, saved);
}

// SGC chemical-potential term: param_chem_pot . (R^T dN), dN per component
// (SemiGrandCanonicalCalculator.cc:201-212).
double sgc_mu_term(const System &s, const double *mu, int n, const i64 *sites, const int *new_occ,
                   const signed char *occ) {
  std::vector<double> dN(s.n_occ, 0.0);
  for (int i = 0; i < n; ++i) {
    dN[occ[sites[i]]] += -1.0;
    dN[new_occ[i]] += 1.0;
  }
  double t = 0.0;
  for (int a = 0; a < s.n_occ - 1; ++a) {
    double x = 0.0;
    for (int c = 0; c < s.n_occ; ++c) x += s.RT[a * s.n_occ + c] * dN[c];
    t += mu[a] * x;
  }
  return t;
}

// ---- occupant location lists (restatement of libcasm-monte OccLocation for
// one asymmetric unit with all sites mutable): one list per species,
// initialised in increasing site order; apply() removes a site from its old
// list by moving the last element into its slot and appends it to the new.
struct OccLoc {
  std::vector<std::vector<int>> lists;
  std::vector<int> pos;
  void init(const signed char *occ, int n, int n_occ) {
    lists.assign(n_occ, {});
    pos.assign(n, 0);
    for (int l = 0; l < n; ++l) {
      pos[l] = (int)lists[occ[l]].size();
      lists[occ[l]].push_back(l);
    }
  }
  void move(int l, int from, int to) {
    auto &a = lists[from];
    int p = pos[l];
    int last = a.back();
    a[p] = last;
    pos[last] = p;
    a.pop_back();
    pos[l] = (int)lists[to].size();
    lists[to].push_back(l);
  }
};

// ---- random draws exactly as libcasm-monte's RandomNumberGenerator does
// them: std::uniform_int_distribution<long>(0, max) and
// std::uniform_real_distribution<double>(0, max) over std::mt19937_64.
struct Rng {
  std::mt19937_64 eng;
  u64 draws = 0;
  struct Counting {
    Rng *r;
    using result_type = u64;
    static constexpr u64 min() { return std::mt19937_64::min(); }
    static constexpr u64 max() { return std::mt19937_64::max(); }
    u64 operator()() {
      r->draws++;
      return r->eng();
    }
  };
  long random_int(long max) {
    Counting c{this};
    return std::uniform_int_distribution<long>(0, max)(c);
  }
  double random_real(double max) {
    Counting c{this};
    return std::uniform_real_distribution<double>(0.0, max)(c);
  }
};

// Metropolis acceptance (libcasm-monte metropolis_acceptance, restated):
// accept if dE < 0, otherwise draw u in [0,1) and accept if u < exp(-beta dE).
bool accept_metropolis(double de, double beta, Rng &rng) {
  if (de < 0.0) return true;
  return rng.random_real(1.0) < std::exp(-de * beta);
}

struct RunOut {
  i64 n_accept = 0, n_reject = 0;
  std::vector<double> energy_uc;     // formation energy per unit cell, per sample
  std::vector<double> potential_uc;  // potential per unit cell, per sample
  std::vector<double> comp;          // per sample, (n_occ-1) param compositions
};

}  // namespace

extern "C" {

const char *ora_last_error() { return g_err.c_str(); }

void *ora_system_create(int n_basis, const i64 *lattice, const i64 *basis, double grid, int n_occ,
                        const double *max_length, int n_funcs, const int *func_size,
                        const i64 *func_pts, const int *func_occ, const double *eci,
                        const double *coeff, const double *RT, int Lx, int Ly, int Lz,
                        int t10, int t20, int t21) {
  try {
    auto s = std::make_unique<System>();
    s->tw[0] = t10;
    s->tw[1] = t20;
    s->tw[2] = t21;
    s->n_basis = n_basis;
    s->n_occ = n_occ;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) s->lat[r][c] = lattice[r * 3 + c];
    for (int b = 0; b < n_basis; ++b) s->basis.push_back({basis[b * 3], basis[b * 3 + 1], basis[b * 3 + 2]});
    s->grid = grid;
    s->L[0] = Lx;
    s->L[1] = Ly;
    s->L[2] = Lz;
    s->n_funcs = n_funcs;
    s->eci.assign(eci, eci + n_funcs);
    s->coeff.assign(coeff, coeff + n_funcs);
    s->RT.assign(RT, RT + (n_occ - 1) * n_occ);
    build(*s, max_length, func_size, func_pts, func_occ);
    return s.release();
  } catch (std::exception &e) {
    g_err = e.what();
    return nullptr;
  }
}

void *ora_system_create_xtal(int n_basis_all, const double *lattice, const double *frac,
                             const int *site_kind, const int *site_dof, int n_occ,
                             const double *max_length, int n_funcs, const int *func_size,
                             const i64 *func_sites, const int *func_occ, const double *eci,
                             const double *coeff, const double *RT, int Lx, int Ly, int Lz,
                             int t10, int t20, int t21) {
  try {
    auto s = std::make_unique<System>();
    s->tw[0] = t10;
    s->tw[1] = t20;
    s->tw[2] = t21;
    int nd = 0;
    for (int b = 0; b < n_basis_all; ++b) nd += site_dof[b] ? 1 : 0;
    s->n_basis = nd;
    s->n_occ = n_occ;
    s->L[0] = Lx;
    s->L[1] = Ly;
    s->L[2] = Lz;
    s->n_funcs = n_funcs;
    s->eci.assign(eci, eci + n_funcs);
    s->coeff.assign(coeff, coeff + n_funcs);
    s->RT.assign(RT, RT + (n_occ - 1) * n_occ);
    build_xtal(*s, lattice, n_basis_all, frac, site_kind, site_dof, max_length, func_size,
               func_sites, func_occ);
    return s.release();
  } catch (std::exception &e) {
    g_err = e.what();
    return nullptr;
  }
}

void ora_system_destroy(void *h) { delete (System *)h; }

int ora_n_sites(void *h) { return ((System *)h)->n_sites; }
int ora_n_clusters(void *h) { return (int)((System *)h)->cl_type_b.size(); }
void ora_multiplicities(void *h, double *out) {
  System &s = *(System *)h;
  for (int f = 0; f < s.n_funcs; ++f) out[f] = s.mult[f];
}

// Integer function counts over the supercell (count[0] = number of unit cells).
void ora_counts(void *h, const signed char *occ, i64 *count) {
  System &s = *(System *)h;
  all_counts(s, occ, count);
  count[0] = s.n_uc;
}

// Formation energy per supercell.
double ora_energy(void *h, const signed char *occ) {
  System &s = *(System *)h;
  std::vector<i64> c(s.n_funcs);
  all_counts(s, occ, c.data());
  return counts_to_energy(s, c.data());
}

// Extensive correlations per unit cell: coeff_f * count_f / (mult_f n_uc).
void ora_corr(void *h, const signed char *occ, double *corr) {
  System &s = *(System *)h;
  std::vector<i64> c(s.n_funcs);
  all_counts(s, occ, c.data());
  corr[0] = 1.0;
  for (int f = 1; f < s.n_funcs; ++f) corr[f] = s.coeff[f] * (double)c[f] / (s.mult[f] * s.n_uc);
}

// occ_delta_per_supercell of the formation energy (canonical potential).
double ora_delta(void *h, const signed char *occ, int n, const i64 *sites, const int *new_occ,
                 i64 *dcount) {
  System &s = *(System *)h;
  std::vector<signed char> o(occ, occ + s.n_sites);
  return event_delta(s, o, n, sites, new_occ, dcount);
}

// Single-thread timing of n independent one-site energy changes on one
// occupation (each evaluated as ora_delta does, the state left unchanged):
// the oracle's counterpart of a Clexulator's per-site delta evaluation.
// Returns seconds; *checksum receives the sum of the energy changes.
double ora_time_delta(void *h, const signed char *occ, i64 n, const i64 *sites, const int *new_occ,
                      double *checksum) {
  System &s = *(System *)h;
  std::vector<signed char> o(occ, occ + s.n_sites);
  double sum = 0.0;
  const auto t0 = std::chrono::steady_clock::now();
  for (i64 e = 0; e < n; ++e) sum += event_delta(s, o, 1, sites + e, new_occ + e, nullptr);
  const auto t1 = std::chrono::steady_clock::now();
  if (checksum) *checksum = sum;
  return std::chrono::duration<double>(t1 - t0).count();
}

// occ_delta_per_supercell of the semi-grand canonical potential.
double ora_delta_sgc(void *h, const signed char *occ, int n, const i64 *sites,
                     const int *new_occ, const double *mu, i64 *dcount) {
  System &s = *(System *)h;
  std::vector<signed char> o(occ, occ + s.n_sites);
  double de = event_delta(s, o, n, sites, new_occ, dcount);
  return de - sgc_mu_term(s, mu, n, sites, new_occ, occ);
}

// Sequential Metropolis run (occupation_metropolis_v2 restated).
// ensemble: 0 = semi-grand canonical (flip), 1 = canonical (swap).
// Per step records (optional, may be null): site0, site1, dE, accept.
// Samples are taken after every pass (steps_per_pass = n_sites).
int ora_run(void *h, signed char *occ, int ensemble, double temperature, const double *mu,
            u64 seed, i64 n_passes, i64 record_steps, i64 *rec_site0, i64 *rec_site1,
            double *rec_de, unsigned char *rec_accept, double *samp_energy,
            double *samp_potential, double *samp_comp, i64 *n_accept_out,
            u64 *draws_out) {
  try {
    System &s = *(System *)h;
    const double kb = 8.617333262e-5;
    double beta = (std::fabs(temperature) < 1e-10) ? INFINITY : 1.0 / (kb * temperature);
    Rng rng;
    rng.eng.seed(seed);
    OccLoc loc;
    loc.init(occ, s.n_sites, s.n_occ);
    std::vector<signed char> o(occ, occ + s.n_sites);
    // swap types: SGC (a -> b) for all a != b; canonical (a, b) for a < b
    std::vector<std::pair<int, int>> swaps;
    for (int a = 0; a < s.n_occ; ++a)
      for (int b = 0; b < s.n_occ; ++b) {
        if (a == b) continue;
        if (ensemble == 1 && b < a) continue;
        swaps.push_back({a, b});
      }
    i64 steps_per_pass = s.n_sites;
    i64 n_acc = 0, step = 0;
    std::vector<i64> cnt(s.n_funcs);
    i64 sites[2];
    int nocc[2];
    std::vector<long> cum(swaps.size());
    for (i64 pass = 0; pass < n_passes; ++pass) {
      for (i64 st = 0; st < steps_per_pass; ++st, ++step) {
        // propose
        long tsum = 0;
        for (size_t i = 0; i < swaps.size(); ++i) {
          long w = (long)loc.lists[swaps[i].first].size();
          if (ensemble == 1) w *= (long)loc.lists[swaps[i].second].size();
          tsum += w;
          cum[i] = tsum;
        }
        if (tsum == 0) throw std::runtime_error("no event can be proposed");
        long count = rng.random_int(tsum - 1);
        size_t it = std::upper_bound(cum.begin(), cum.end(), count) - cum.begin();
        int a = swaps[it].first, b = swaps[it].second;
        int n;
        if (ensemble == 1) {
          long ia = rng.random_int((long)loc.lists[a].size() - 1);
          long ib = rng.random_int((long)loc.lists[b].size() - 1);
          sites[0] = loc.lists[a][ia];
          sites[1] = loc.lists[b][ib];
          nocc[0] = b;
          nocc[1] = a;
          n = 2;
        } else {
          long ia = rng.random_int((long)loc.lists[a].size() - 1);
          sites[0] = loc.lists[a][ia];
          nocc[0] = b;
          n = 1;
        }
        double de = event_delta(s, o, n, sites, nocc, nullptr);
        if (ensemble == 0) de -= sgc_mu_term(s, mu, n, sites, nocc, o.data());
        bool acc = accept_metropolis(de, beta, rng);
        if (step < record_steps) {
          if (rec_site0) rec_site0[step] = sites[0];
          if (rec_site1) rec_site1[step] = (n == 2) ? sites[1] : -1;
          if (rec_de) rec_de[step] = de;
          if (rec_accept) rec_accept[step] = acc ? 1 : 0;
        }
        if (acc) {
          ++n_acc;
          for (int i = 0; i < n; ++i) {
            loc.move((int)sites[i], o[sites[i]], nocc[i]);
            o[sites[i]] = (signed char)nocc[i];
          }
        }
      }
      // sample: potential_energy = potential.per_unitcell() (full recompute,
      // sampling_functions.cc:274-283), param composition
      all_counts(s, o.data(), cnt.data());
      double ef = counts_to_energy(s, cnt.data());
      std::vector<double> nk(s.n_occ, 0.0);
      for (int l = 0; l < s.n_sites; ++l) nk[o[l]] += 1.0;
      double pot = ef;
      for (int a = 0; a < s.n_occ - 1; ++a) {
        double x = 0.0;  // param composition per unit cell
        for (int c = 0; c < s.n_occ; ++c) x += s.RT[a * s.n_occ + c] * (nk[c] - (c == 0 ? s.n_sites : 0));
        x /= s.n_uc;
        if (samp_comp) samp_comp[pass * (s.n_occ - 1) + a] = x;
        if (ensemble == 0) pot -= s.n_uc * mu[a] * x;
      }
      if (samp_energy) samp_energy[pass] = ef / s.n_uc;
      if (samp_potential) samp_potential[pass] = pot / s.n_uc;
    }
    std::memcpy(occ, o.data(), s.n_sites);
    if (n_accept_out) *n_accept_out = n_acc;
    if (draws_out) *draws_out = rng.draws;
    return 0;
  } catch (std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// Greedy composition enforcement (clexmonte::enforce_composition restated,
// include/casm/clexmonte/state/enforce_composition.hh:56-126 and 172-210):
// flip types a -> b (a != b) in a-major order; the distance is the Euclidean
// norm of (mol composition per unit cell - target); a type is a candidate if
// it improves the distance by more than tol = 1e-3 / volume; ties within tol
// are broken by random_real(sum of their site counts); the flipped site is
// the random_int-th entry of the species' occupant list. Returns the number
// of flips (or -1 on error) and the engine draws consumed.
i64 ora_enforce_composition(void *h, signed char *occ, const double *target, u64 seed,
                            u64 *draws_out) {
  try {
    System &s = *(System *)h;
    const int n = s.n_sites, no = s.n_occ;
    Rng rng;
    rng.eng.seed(seed);
    OccLoc loc;
    loc.init(occ, n, no);
    const double volume = (double)(n / s.n_basis);
    const double dn = 1. / volume;
    const double tol = dn * 1e-3;
    std::vector<double> cur(no);
    for (int c = 0; c < no; ++c) cur[c] = (double)loc.lists[c].size() / volume;
    auto dist = [&](const std::vector<double> &m) {
      double q = 0.0;
      for (int c = 0; c < no; ++c) {
        double d = m[c] - target[c];
        q += d * d;
      }
      return std::sqrt(q);
    };
    struct Choice {
      int a, b;
      long count;
      std::vector<double> mol;
    };
    i64 flips = 0;
    while (true) {
      const double orig = dist(cur);
      double best = orig;
      std::vector<Choice> ch;
      for (int a = 0; a < no; ++a)
        for (int b = 0; b < no; ++b) {
          if (a == b || loc.lists[a].empty()) continue;
          std::vector<double> t = cur;
          t[a] -= dn;
          t[b] += dn;
          double d = dist(t);
          if (d > orig - tol) {
            continue;
          } else if (d < best - tol) {
            ch.clear();
            ch.push_back({a, b, (long)loc.lists[a].size(), t});
            best = d;
          } else if (d < best + tol) {
            ch.push_back({a, b, (long)loc.lists[a].size(), t});
          }
        }
      if (ch.empty()) break;
      double sum = 0.0;
      for (auto &c : ch) sum += c.count;
      double u = rng.random_real(sum);
      sum = 0.0;
      const Choice *pick = nullptr;
      for (auto &c : ch) {
        sum += c.count;
        if (u < sum) {
          pick = &c;
          break;
        }
      }
      if (!pick) throw std::runtime_error("failed enforcing composition");
      cur = pick->mol;
      long ia = rng.random_int((long)loc.lists[pick->a].size() - 1);
      int l = loc.lists[pick->a][ia];
      loc.move(l, pick->a, pick->b);
      occ[l] = (signed char)pick->b;
      ++flips;
    }
    if (draws_out) *draws_out = rng.draws;
    return flips;
  } catch (std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

// ---- n-fold way (Bortz-Kalos-Lebowitz rejection-free semi-grand canonical
// Monte Carlo; clexmonte::nfold::Nfold::run, include/casm/clexmonte/nfold/
// nfold_impl.hh:20-108, rates as CompleteEventCalculator::calculate_rate,
// src/casm/clexmonte/nfold/nfold_events.cc:24-60). Restated sequentially:
// events are (site l, k-th other occupant), e = l (n_occ - 1) + k; rate =
// 1 if dE <= 0 else exp(-beta dE) with dE = sum_f w_f dcount_f - dmu (one
// fused multiply-add per function, in function order); a
// 32-ary sum tree whose nodes are pairwise sums of their children (the 32
// children, zero-padded, summed as a balanced binary tree: (c0 + c1) +
// (c2 + c3), ...); each step weights the current state by n_possible /
// total, draws a uniform u53 from Philox4x32-10 (counter = event index, tag
// 3), descends the tree (inside a node, down the same binary tree: left when
// the right half is empty or the target lies below the left half's sum, else
// right with the left sum subtracted), applies the event. All rates are recomputed after every event (the GPU
// recomputes only the changed site's flower), so the comparison also checks
// the GPU's impact lists.
extern "C" void ora_philox4x32_10(const unsigned *ctr_in, const unsigned *key_in, unsigned *out);

// exp(x) for x <= 0: Cody-Waite reduction with the fdlibm split of ln2,
// degree-13 Taylor polynomial by fused multiply-adds in Estrin's scheme,
// scaling by 2^n.
static double exp_neg_restated(double x) {
  if (!(x >= -745.0)) return 0.0;
  if (x > 0.0) x = 0.0;
  const double log2e = 0x1.71547652b82fep+0;
  const double ln2_hi = 0x1.62e42fee00000p-1;
  const double ln2_lo = 0x1.a39ef35793c76p-33;
  const double n = std::nearbyint(x * log2e);
  double r = std::fma(-n, ln2_hi, x);
  r = std::fma(-n, ln2_lo, r);
  static const double c[14] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                               0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                               0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                               0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                               0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};
  // p = 1 + (r + r^2 T(r)), T = c2 + ... + c13 r^11 in Estrin's scheme, the
  // same association as the product's
  const double r2 = r * r, r4 = r2 * r2;
  const double a0 = std::fma(c[3], r, c[2]), a1 = std::fma(c[5], r, c[4]),
               a2 = std::fma(c[7], r, c[6]), a3 = std::fma(c[9], r, c[8]),
               a4 = std::fma(c[11], r, c[10]), a5 = std::fma(c[13], r, c[12]);
  const double b0 = std::fma(a1, r2, a0), b1 = std::fma(a3, r2, a2), b2 = std::fma(a5, r2, a4);
  const double t = std::fma(std::fma(b2, r4, b1), r4, b0);
  const double p = std::fma(r2, t, r) + c[0];
  return std::ldexp(p, (int)n);
}

extern "C" double ora_exp_neg(double x) { return exp_neg_restated(x); }

// The 32 children of a tree node (zero beyond the level's end).
static void children32(const std::vector<double> &lev, size_t node, double *v) {
  for (int c = 0; c < 32; ++c) {
    const size_t i = node * 32 + (size_t)c;
    v[c] = i < lev.size() ? lev[i] : 0.0;
  }
}

// stats_out: [0] total weight, [1] sum w ep, [2] sum w ep^2, [3] sum w ef,
// [4..6] sum w x_k, [7..15] sum w x_k x_k', [16..18] sum w ep x_k.
// Returns the number of events applied (-1 on error).
extern "C" i64 ora_nfold(void *h, signed char *occ, double temperature, const double *mu,
                         const double *w, u64 seed, i64 n_events, i64 n_equil, i64 rec_cap,
                         i64 *rec_site, int *rec_occ, double *rec_dt, double *stats_out) {
  try {
    System &s = *(System *)h;
    const int no = s.n_occ, N = s.n_sites;
    const double kb = 8.617333262e-5;
    const double beta = (std::fabs(temperature) < 1e-10) ? INFINITY : 1.0 / (kb * temperature);
    std::vector<double> dmu(no * no, 0.0);
    for (int oi = 0; oi < no; ++oi)
      for (int of = 0; of < no; ++of) {
        double t = 0.0;
        for (int k = 0; k < no - 1; ++k) {
          double x = s.RT[k * no + of] - s.RT[k * no + oi];
          t += mu[k] * x;
        }
        dmu[oi * no + of] = t;
      }
    std::vector<i64> dc(s.n_funcs);
    auto de_f = [&](int l, int of) {
      std::fill(dc.begin(), dc.end(), 0);
      site_delta_counts(s, occ, l, of, dc.data());
      double d = 0.0;
      for (int f = 1; f < s.n_funcs; ++f) d = std::fma(w[f], (double)dc[f], d);
      return d;
    };
    const i64 n_ev = (i64)N * (no - 1);
    // tree levels
    std::vector<std::vector<double>> lev;
    lev.push_back(std::vector<double>(n_ev));
    while (lev.back().size() > 1) lev.push_back(std::vector<double>((lev.back().size() + 31) / 32));
    auto rebuild = [&]() {
      for (i64 e = 0; e < n_ev; ++e) {
        const int l = (int)(e / (no - 1)), k = (int)(e % (no - 1));
        const int oi = occ[l], of = k < oi ? k : k + 1;
        const double de = de_f(l, of) - dmu[oi * no + of];
        lev[0][e] = de <= 0.0 ? 1.0 : exp_neg_restated(-beta * de);
      }
      for (size_t L = 1; L < lev.size(); ++L)
        for (size_t node = 0; node < lev[L].size(); ++node) {
          double v[32];
          children32(lev[L - 1], node, v);
          for (int wdt = 1; wdt < 32; wdt *= 2)
            for (int i = 0; i < 32; i += 2 * wdt) v[i] = v[i] + v[i + wdt];
          lev[L][node] = v[0];
        }
    };
    // observables
    std::vector<i64> nspec(no, 0);
    for (int l = 0; l < N; ++l) nspec[occ[l]]++;
    std::vector<i64> cnt(s.n_funcs);
    all_counts(s, occ, cnt.data());
    double energy = counts_to_energy(s, cnt.data());
    for (int k = 0; k < 19; ++k) stats_out[k] = 0.0;
    const double n_possible = (double)N * (double)(no * (no - 1));
    const unsigned key[2] = {(unsigned)seed, (unsigned)(seed >> 32)};
    rebuild();
    i64 done = 0;
    for (i64 it = 0; it < n_equil + n_events; ++it) {
      const double total = lev.back()[0];
      if (!(total > 0.0)) break;
      const double dt = n_possible / total;
      if (it >= n_equil) {
        double x[3] = {0.0, 0.0, 0.0}, mux = 0.0;
        for (int k = 0; k < no - 1; ++k) {
          double t = 0.0;
          for (int a = 0; a < no; ++a) {
            const double c = (double)nspec[a] - (a == 0 ? (double)N : 0.0);
            t = t + s.RT[k * no + a] * c;
          }
          x[k] = t / (double)s.n_uc;
          mux = mux + mu[k] * x[k];
        }
        const double ef = energy / (double)s.n_uc;
        const double ep = ef - mux;
        stats_out[0] = stats_out[0] + dt;
        stats_out[1] = stats_out[1] + dt * ep;
        stats_out[2] = stats_out[2] + dt * (ep * ep);
        stats_out[3] = stats_out[3] + dt * ef;
        for (int k = 0; k < no - 1; ++k) {
          stats_out[4 + k] = stats_out[4 + k] + dt * x[k];
          stats_out[16 + k] = stats_out[16 + k] + dt * (ep * x[k]);
          for (int k2 = 0; k2 < no - 1; ++k2)
            stats_out[7 + k * 3 + k2] = stats_out[7 + k * 3 + k2] + dt * (x[k] * x[k2]);
        }
      }
      const unsigned ctr[4] = {(unsigned)it, (unsigned)(it >> 32), 0u, 3u << 16};
      unsigned rr[4];
      ora_philox4x32_10(ctr, key, rr);
      const double u = ((double)(rr[0] >> 5) * 67108864.0 + (double)(rr[1] >> 6)) * 0x1.0p-53;
      double tgt = u * total;
      i64 node = 0;
      for (int L = (int)lev.size() - 1; L >= 1; --L) {
        // the node's binary tree: part[k][i] = sum of children i 2^k ..
        // (i + 1) 2^k - 1, zero-padded to 32 children
        double part[6][32];
        children32(lev[L - 1], (size_t)node, part[0]);
        for (int k = 1; k <= 5; ++k)
          for (int i = 0; i < (32 >> k); ++i) part[k][i] = part[k - 1][2 * i] + part[k - 1][2 * i + 1];
        int j = 0;  // current sub-node at level k
        for (int k = 4; k >= 0; --k) {
          const double left = part[k][2 * j], right = part[k][2 * j + 1];
          if (right == 0.0 || (left > 0.0 && tgt < left)) {
            j = 2 * j;
          } else {
            tgt = tgt - left;
            j = 2 * j + 1;
          }
        }
        node = node * 32 + j;
      }
      const int l = (int)(node / (no - 1)), k = (int)(node % (no - 1));
      const int oi = occ[l], of = k < oi ? k : k + 1;
      if (it < rec_cap) {
        rec_site[it] = l;
        rec_occ[it] = of;
        rec_dt[it] = dt;
      }
      energy = energy + de_f(l, of);
      nspec[oi]--;
      nspec[of]++;
      occ[l] = (signed char)of;
      rebuild();
      ++done;
    }
    return done;
  } catch (std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

// Many independent sequential chains on host threads (CPU baseline):
// replica r uses occ + r*n_sites, seed + r, temperature[r], mu[r*(n_occ-1)].
// Returns wall seconds; n_steps_out = total proposals.
double ora_run_threads(void *h, signed char *occ, int n_rep, int ensemble, const double *temps,
                       const double *mus, u64 seed, i64 n_passes, int n_threads,
                       i64 *n_steps_out) {
  System &s = *(System *)h;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  int nt = std::max(1, std::min(n_threads, n_rep));
  for (int w = 0; w < nt; ++w)
    th.emplace_back([&, w]() {
      for (int r = w; r < n_rep; r += nt) {
        ora_run(h, occ + (size_t)r * s.n_sites, ensemble, temps[r], mus + r * (s.n_occ - 1),
                seed + r, n_passes, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                nullptr, nullptr, nullptr);
      }
    });
  for (auto &t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  if (n_steps_out) *n_steps_out = (i64)n_rep * n_passes * s.n_sites;
  return std::chrono::duration<double>(t1 - t0).count();
}

// Independent sequential chains with their per-pass samples: chain r runs on
// occupation block r with engine seed + r (the loop of ora_run, i.e.
// occupation_metropolis.hh:92-120 restated); chains are spread over n_threads
// host threads. samp_potential [n_rep][n_passes] and samp_comp
// [n_rep][n_passes][n_occ - 1] receive potential energy and param
// composition per unit cell after each pass. Returns wall seconds, or -1 on
// error (ora_last_error).
double ora_run_chains(void *h, signed char *occ, int n_rep, int ensemble, const double *temps,
                      const double *mus, u64 seed, i64 n_passes, int n_threads,
                      double *samp_potential, double *samp_comp) {
  System &s = *(System *)h;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  std::vector<int> rc(n_rep, 0);
  const int nc = s.n_occ - 1;
  int nt = std::max(1, std::min(n_threads, n_rep));
  for (int w = 0; w < nt; ++w)
    th.emplace_back([&, w]() {
      for (int r = w; r < n_rep; r += nt) {
        rc[r] = ora_run(h, occ + (size_t)r * s.n_sites, ensemble, temps[r], mus + r * nc,
                        seed + r, n_passes, 0, nullptr, nullptr, nullptr, nullptr, nullptr,
                        samp_potential ? samp_potential + (size_t)r * n_passes : nullptr,
                        samp_comp ? samp_comp + (size_t)r * n_passes * nc : nullptr, nullptr,
                        nullptr);
      }
    });
  for (auto &t : th) t.join();
  for (int r = 0; r < n_rep; ++r)
    if (rc[r]) return -1.0;
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// ---- random-stream probes used to pin the transforms the GPU restates.
void ora_mt19937_64(u64 seed, i64 n, u64 *out) {
  std::mt19937_64 e(seed);
  for (i64 i = 0; i < n; ++i) out[i] = e();
}
void ora_std_uniform_int(u64 seed, i64 n, const long *maxv, long *out, u64 *draws) {
  Rng r;
  r.eng.seed(seed);
  for (i64 i = 0; i < n; ++i) out[i] = r.random_int(maxv[i]);
  *draws = r.draws;
}
void ora_std_uniform_real(u64 seed, i64 n, double *out) {
  Rng r;
  r.eng.seed(seed);
  for (i64 i = 0; i < n; ++i) out[i] = r.random_real(1.0);
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011), written from the paper's round function.
void ora_philox4x32_10(const unsigned *ctr_in, const unsigned *key_in, unsigned *out) {
  unsigned c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  unsigned k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    u64 p0 = (u64)0xD2511F53u * c0;
    u64 p1 = (u64)0xCD9E8D57u * c2;
    unsigned hi0 = (unsigned)(p0 >> 32), lo0 = (unsigned)p0;
    unsigned hi1 = (unsigned)(p1 >> 32), lo1 = (unsigned)p1;
    unsigned n0 = hi1 ^ c1 ^ k0;
    unsigned n1 = lo1;
    unsigned n2 = hi0 ^ c3 ^ k1;
    unsigned n3 = lo0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

}  // extern "C"
