// Host build of the FP64 exp used for n-fold rates (cem_common.cuh): prints
// the bits of cem_exp_neg(x) for each hex-float x read from stdin.
#include <cstdio>
#include <cstring>
#include "../casmcode_clexmonte_gb300/csrc/cem_common.cuh"
int main() {
  double x;
  while (std::scanf("%la", &x) == 1) {
    const double y = cem::cem_exp_neg(x);
    unsigned long long b;
    std::memcpy(&b, &y, 8);
    std::printf("%016llx\n", b);
  }
  return 0;
}
