// View-table kernel variants of one block shape: four warps per block, stacks in per-thread local memory.
#include "views_kernel.cuh"

namespace csgrt {
template cudaError_t launch_views_shape<128, true>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);
}  // namespace csgrt
