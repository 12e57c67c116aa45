// Sweep kernels that walk the run-time tables one orbit at a time: cluster
// expansions with more orbits than the register accumulators hold (real CASM
// basis sets, e.g. 73 orbits and 1591 clusters per site for hcp Zr-O).
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, -1, SWEEP_THREADS>(const CeTables &, const SweepParams &, int,
                                                          int, cudaStream_t);
template cudaError_t launch_sweep_t<3, -1, SWEEP_THREADS>(const CeTables &, const SweepParams &, int,
                                                          int, cudaStream_t);
}  // namespace cem
