// Sweep kernels with the generated binary FCC site evaluator for the
// shared-memory pitches 14, 36 and 64 (10^3, 32^3 and other supercells).
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, 14, SWEEP_THREADS>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
template cudaError_t launch_sweep_t<2, 36, SWEEP_THREADS>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
template cudaError_t launch_sweep_t<2, 64, SWEEP_THREADS>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
}  // namespace cem
