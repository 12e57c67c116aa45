// Kernel instantiations for three occupants per site (ternary alloys).
#include "cem_kernels.cuh"
namespace cem {
CEM_INSTANTIATE(3)
}
