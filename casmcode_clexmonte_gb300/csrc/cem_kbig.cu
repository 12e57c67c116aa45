// Sweep kernels for cluster expansions with more orbits than the register
// accumulators hold (real CASM basis sets, e.g. 73 orbits and 1591 clusters
// per site for hcp Zr-O): one thread per site walking the run-time tables one
// orbit at a time (-1), or, for binary systems, one warp per site change with
// the flower split over the lanes (-2).
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, -1, SWEEP_THREADS>(const CeTables &, const SweepParams &, int,
                                                          int, cudaStream_t);
template cudaError_t launch_sweep_t<3, -1, SWEEP_THREADS>(const CeTables &, const SweepParams &, int,
                                                          int, cudaStream_t);
// binary, one warp per site change (per-cluster split weights)
template cudaError_t launch_sweep_t<2, -2, SWEEP_THREADS>(const CeTables &, const SweepParams &, int,
                                                          int, cudaStream_t);
}  // namespace cem
