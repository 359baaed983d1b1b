// The recording form of the single-view render kernel (render_tiled with REC = true: the
// tile order of the cost-ordered dispatch and per-block durations), instantiated in a
// translation unit of its own so that it compiles in parallel with render.cu.
#include "render_tiled.cuh"

namespace csgrt {
namespace tiled {

template cudaError_t launch_tiled<true>(const RenderParams& p, cudaStream_t stream);

}  // namespace tiled
}  // namespace csgrt
