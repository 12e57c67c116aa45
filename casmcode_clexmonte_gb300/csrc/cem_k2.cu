// Kernel instantiations for two occupants per site (binary alloys).
#include "cem_kernels.cuh"
namespace cem {
CEM_INSTANTIATE(2)
}
