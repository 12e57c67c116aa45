// Minimal base class for generated Clexulators, written for the oracle's
// golden-vector probe from the members and overrides the generated code uses.
// `_occ(nlist_ind)` reads occupation[nlist[nlist_ind]] as CASM's does.
#pragma once
#include <set>
#include <vector>

#include "casm/clexulator/BasicClexParamPack.hh"
#include "casm/global/eigen.hh"

namespace CASM {
namespace xtal {
struct UnitCell {
  long i, j, k;
  UnitCell(long a, long b, long c) : i(a), j(b), k(c) {}
  bool operator<(UnitCell const &o) const {
    if (i != o.i) return i < o.i;
    if (j != o.j) return j < o.j;
    return k < o.k;
  }
};
struct UnitCellCoord {
  long b, i, j, k;
  UnitCellCoord(long s, long a, long bb, long c) : b(s), i(a), j(bb), k(c) {}
  bool operator<(UnitCellCoord const &o) const {
    if (b != o.b) return b < o.b;
    if (i != o.i) return i < o.i;
    if (j != o.j) return j < o.j;
    return k < o.k;
  }
};
}  // namespace xtal

namespace clexulator {

class BaseClexulator {
 public:
  typedef unsigned int size_type;
  BaseClexulator(size_type nlist_size, size_type corr_size, size_type n_point_corr)
      : m_nlist_size(nlist_size), m_corr_size(corr_size), m_n_point_corr(n_point_corr) {}
  virtual ~BaseClexulator() {}

  size_type corr_size() const { return m_corr_size; }
  size_type nlist_size() const { return m_nlist_size; }

  void set_pointers(int const *occ, long const *nlist) {
    m_occ_ptr = occ;
    m_nlist_ptr = nlist;
  }
  void global_corr(double *out) const { _calc_global_corr_contribution(out); }
  void delta_point_corr(int nlist_ind, int occ_i, int occ_f, double *out) const {
    _calc_delta_point_corr(nlist_ind, occ_i, occ_f, out);
  }
  void point_corr(int nlist_ind, double *out) const { _calc_point_corr(nlist_ind, out); }

  std::set<xtal::UnitCell> const &neighborhood() const { return m_neighborhood; }
  long weight(int r, int c) const { return m_weight_matrix.v[r][c]; }
  std::set<int> const &sublat_indices() const { return m_sublat_indices; }

  virtual ClexParamPack const &param_pack() const = 0;
  virtual ClexParamPack &param_pack() = 0;

 protected:
  int const &_occ(int nlist_ind) const { return m_occ_ptr[m_nlist_ptr[nlist_ind]]; }

  Eigen::Matrix3l m_weight_matrix;
  std::set<int> m_sublat_indices;
  int m_n_sublattices = 0;
  std::set<xtal::UnitCell> m_neighborhood;
  std::vector<std::set<xtal::UnitCell>> m_orbit_neighborhood;
  std::vector<std::set<xtal::UnitCellCoord>> m_orbit_site_neighborhood;

 private:
  size_type m_nlist_size, m_corr_size, m_n_point_corr;
  int const *m_occ_ptr = nullptr;
  long const *m_nlist_ptr = nullptr;

  virtual BaseClexulator *_clone() const = 0;
  virtual void _calc_global_corr_contribution() const = 0;
  virtual void _calc_global_corr_contribution(double *corr_begin) const = 0;
  virtual void _calc_restricted_global_corr_contribution(size_type const *, size_type const *) const = 0;
  virtual void _calc_restricted_global_corr_contribution(double *, size_type const *,
                                                         size_type const *) const = 0;
  virtual void _calc_point_corr(int nlist_ind) const = 0;
  virtual void _calc_point_corr(int nlist_ind, double *corr_begin) const = 0;
  virtual void _calc_restricted_point_corr(int, size_type const *, size_type const *) const = 0;
  virtual void _calc_restricted_point_corr(int, double *, size_type const *,
                                           size_type const *) const = 0;
  virtual void _calc_delta_point_corr(int nlist_ind, int occ_i, int occ_f) const = 0;
  virtual void _calc_delta_point_corr(int nlist_ind, int occ_i, int occ_f,
                                      double *corr_begin) const = 0;
  virtual void _calc_restricted_delta_point_corr(int, int, int, size_type const *,
                                                 size_type const *) const = 0;
  virtual void _calc_restricted_delta_point_corr(int, int, int, double *, size_type const *,
                                                 size_type const *) const = 0;
};

}  // namespace clexulator
}  // namespace CASM
