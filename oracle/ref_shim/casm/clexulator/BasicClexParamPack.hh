// Minimal parameter pack for generated Clexulators: a named set of dense
// double matrices, read/written by (key, row, col). Written for the oracle's
// golden-vector probe from the calls the generated code makes.
#pragma once
#include <string>
#include <vector>

namespace CASM {
namespace clexulator {

class ClexParamPack {
 public:
  virtual ~ClexParamPack() {}
};

class BasicClexParamPack : public ClexParamPack {
 public:
  enum EvalMode { DEFAULT, READ };
  struct Key {
    int index = -1;
    int rows = 0;
  };
  Key allocate(std::string const &, int rows, int cols, bool) {
    Key k;
    k.index = (int)m_data.size();
    k.rows = rows;
    m_data.emplace_back((size_t)rows * (size_t)cols, 0.0);
    return k;
  }
  double const &read(Key const &k, int i, int j) const {
    return m_data[k.index][(size_t)j * k.rows + i];
  }
  double const &read(Key const &k, int i) const { return m_data[k.index][i]; }
  EvalMode eval_mode(Key const &) const { return DEFAULT; }
  void pre_eval() const {}
  void post_eval() const {}

  template <typename Scalar>
  struct Val {
    static void set(BasicClexParamPack const &p, Key const &k, int i, int j, Scalar v) {
      p.m_data[k.index][(size_t)j * k.rows + i] = v;
    }
    static void set(BasicClexParamPack const &p, Key const &k, int i, Scalar v) {
      p.m_data[k.index][i] = v;
    }
    static Scalar get(BasicClexParamPack const &p, Key const &k, int i) {
      return p.m_data[k.index][i];
    }
  };

 private:
  mutable std::vector<std::vector<double>> m_data;
};

}  // namespace clexulator
}  // namespace CASM
