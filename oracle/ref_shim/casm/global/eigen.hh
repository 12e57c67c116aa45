// Minimal stand-in for the one Eigen use in generated Clexulators:
// `m_weight_matrix.row(i) << a, b, c;` on a 3x3 integer matrix.
// Written for the oracle's golden-vector probe; not Eigen.
#pragma once
namespace Eigen {
struct Matrix3l {
  long v[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  struct RowFill {
    long *row;
    int k;
    RowFill &operator,(long x) {
      row[k++] = x;
      return *this;
    }
  };
  struct Row {
    long *row;
    RowFill operator<<(long x) {
      row[0] = x;
      return RowFill{row, 1};
    }
  };
  Row row(int i) { return Row{v[i]}; }
};
}  // namespace Eigen
