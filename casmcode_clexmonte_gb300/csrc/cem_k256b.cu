// 256-thread sweep kernels (two replicas per SM): generated binary FCC
// evaluator at pitches 52 and 64, run-time tables for two and three occupants.
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, 52, 256>(const CeTables &, const SweepParams &, int, int,
                                                cudaStream_t);
template cudaError_t launch_sweep_t<2, 64, 256>(const CeTables &, const SweepParams &, int, int,
                                                cudaStream_t);
template cudaError_t launch_sweep_t<2, 0, 256>(const CeTables &, const SweepParams &, int, int,
                                               cudaStream_t);
template cudaError_t launch_sweep_t<3, 0, 256>(const CeTables &, const SweepParams &, int, int,
                                               cudaStream_t);
}  // namespace cem
