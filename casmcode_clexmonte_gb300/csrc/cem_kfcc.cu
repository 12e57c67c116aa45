// Sweep kernels with the generated binary FCC site evaluator, one per
// shared-memory pitch (32, 48, 64 bytes per row and rows per plane).
#include "cem_kernels.cuh"
namespace cem {
template cudaError_t launch_sweep_t<2, 32>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
template cudaError_t launch_sweep_t<2, 48>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
template cudaError_t launch_sweep_t<2, 64>(const CeTables &, const SweepParams &, int, int,
                                           cudaStream_t);
}  // namespace cem
