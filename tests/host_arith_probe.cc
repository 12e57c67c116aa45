// Host build of the device arithmetic helpers (cem_common.cuh): prints
// cem_expf_neg(x) for x read from stdin and float-float dot products.
#include <cstdio>
#include "../casmcode_clexmonte_gb300/csrc/cem_common.cuh"
int main() {
  double x;
  while (std::scanf("%lf", &x) == 1) std::printf("%.9e\n", (double)cem::cem_expf_neg((float)x));
  return 0;
}
