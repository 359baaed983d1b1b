// View-table kernel variants of one block shape: two warps per block, stacks in shared memory.
#include "views_kernel.cuh"

namespace csgrt {
template cudaError_t launch_views_shape<64, false>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);
}  // namespace csgrt
