// 256-thread sweep kernels (two replicas per SM) with the generated binary
// FCC evaluator, pitches 14, 28 and 36.
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, 14, 256>(const CeTables &, const SweepParams &, int, int,
                                                cudaStream_t);
template cudaError_t launch_sweep_t<2, 28, 256>(const CeTables &, const SweepParams &, int, int,
                                                cudaStream_t);
template cudaError_t launch_sweep_t<2, 36, 256>(const CeTables &, const SweepParams &, int, int,
                                                cudaStream_t);
}  // namespace cem
