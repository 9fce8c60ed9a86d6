// The kernels with FMA contraction (-fmad=true) and the division-free
// Manning rate: the numerics variant DGSWE_NUMERICS_FAST.
#define DGSWE_FAST 1
#define DGSWE_NS fast
#include "kernels.cuh"
#include "adjoint_kernels.cuh"
#include "launch.cuh"

namespace dgswe {
const KernelSet* kernels_fast() { return &fast::kSet; }
}  // namespace dgswe
