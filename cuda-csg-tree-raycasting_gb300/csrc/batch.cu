// Persistent batched render kernel: many views of many scenes in one launch.
//
// The grid fills the GPU once.  Each block repeatedly takes the next work item -- one
// 128-pixel block tile of one view -- from a counter and renders it with the same per-pixel
// code as the single-view kernel (pixel.cuh), so the results equal per-view renders bit
// for bit.  Items are ordered longest-first by the host, so the expensive views start
// early and the launch's tail is short.  The warp tile shape (8x4, 4x8, 16x2, 32x1) is a
// launch parameter chosen by the autotuner.
#include "batch.hpp"
#include "pixel.cuh"

namespace csgrt {
namespace {

using pix::kThreads;

template <int SD, bool ROLLED>
__global__ void __launch_bounds__(kThreads) render_batch(const BatchLaunch p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint16_t tab[27];
    __shared__ int s_item;
    pix::load_table(tab);
    dev::SmemStacks<SD> st = pix::block_stacks<SD>(smem_raw);
    const pix::BlockSmem bs = pix::block_smem<SD>(smem_raw, p.live_words);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tw = 1 << p.tw_log2, th = 32 >> p.tw_log2;
    // 4 warps arranged 2x2 in a block tile of (2 tw) x (2 th) pixels
    const int ox = (warp & 1) * tw + (lane & (tw - 1));
    const int oy = (warp >> 1) * th + (lane >> p.tw_log2);
    while (true) {
        __syncthreads();  // everyone has read s_item before it is overwritten
        if (threadIdx.x == 0) s_item = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= p.n_items) break;
        const BatchItem wi = p.items[it];
        const BatchView& bv = p.views[wi.view];
        const int tx = wi.tile % bv.tiles_x, ty = wi.tile / bv.tiles_x;
        const int x = tx * 2 * tw + ox, y = ty * 2 * th + oy;
        const bool inside = x < bv.view.w && y < bv.view.h;
        pix::render_pixel<SD, ROLLED>(bv.view, p.status, p.iter_cap, x, y, inside, st, bs, tab);
    }
}

template <int SD, bool ROLLED>
cudaError_t launch_variant(const BatchLaunch& l, cudaStream_t stream, bool size_only, int* grid)
{
    const size_t smem = pix::smem_bytes(SD, l.live_words);
    static bool attr_set = false;
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(render_batch<SD, ROLLED>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)pix::smem_bytes(SD, kLiveWordsMax));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    if (size_only) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, render_batch<SD, ROLLED>, kThreads, smem);
        if (e != cudaSuccess) return e;
        *grid = sms * (per_sm > 0 ? per_sm : 1);
        return cudaSuccess;
    }
    cudaError_t e = cudaMemsetAsync(l.counter, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    int g = l.grid;
    if (g > l.n_items) g = l.n_items;
    if (g < 1) g = 1;
    render_batch<SD, ROLLED><<<g, kThreads, smem, stream>>>(l);
    return cudaGetLastError();
}

cudaError_t dispatch(const BatchLaunch& l, cudaStream_t stream, bool size_only, int* grid)
{
    const bool r = l.rolled != 0;
    switch (l.stack_class) {
        case 4: return r ? launch_variant<4, true>(l, stream, size_only, grid)
                         : launch_variant<4, false>(l, stream, size_only, grid);
        case 8: return r ? launch_variant<8, true>(l, stream, size_only, grid)
                         : launch_variant<8, false>(l, stream, size_only, grid);
        case 12: return r ? launch_variant<12, true>(l, stream, size_only, grid)
                          : launch_variant<12, false>(l, stream, size_only, grid);
        case 16: return r ? launch_variant<16, true>(l, stream, size_only, grid)
                          : launch_variant<16, false>(l, stream, size_only, grid);
        default: return r ? launch_variant<32, true>(l, stream, size_only, grid)
                          : launch_variant<32, false>(l, stream, size_only, grid);
    }
}

}  // namespace

cudaError_t batch_grid_size(BatchLaunch& l)
{
    int g = 0;
    const cudaError_t e = dispatch(l, nullptr, true, &g);
    if (e == cudaSuccess) l.grid = g;
    return e;
}

cudaError_t launch_batch(const BatchLaunch& l, cudaStream_t stream)
{
    return dispatch(l, stream, false, nullptr);
}

}  // namespace csgrt
