// The kernels with every multiply and add separately rounded (-fmad=false),
// IEEE division and square root and the reference's cube root: the numerics
// variant DGSWE_NUMERICS_EXACT.
#define DGSWE_FAST 0
#define DGSWE_NS exact
#include "kernels.cuh"
#include "adjoint_kernels.cuh"
#include "launch.cuh"

namespace dgswe {
const KernelSet* kernels_exact() { return &exact::kSet; }
}  // namespace dgswe
