// Sweep kernels with the generated binary FCC site evaluator for the
// shared-memory pitches 28 and 52 (24^3 and 48^3 supercells).
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, 28, SWEEP_THREADS>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
template cudaError_t launch_sweep_t<2, 52, SWEEP_THREADS>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
}  // namespace cem
