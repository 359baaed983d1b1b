// The persistent view-table kernel (views.hpp), templated on its block shape: warps per
// block and the placement of the per-ray primitive and time stacks (block shared memory,
// or per-thread local memory).  Each translation unit that includes this header
// instantiates launch_views_shape for one shape, so the shapes compile in parallel.
#pragma once

#include <algorithm>
#include <mutex>

#include "pixel.cuh"
#include "views.hpp"

namespace csgrt {

// Minimum resident 128-thread blocks per SM asked of the register allocator (a tuning
// knob; other block sizes ask for the same number of threads): six blocks (80 registers)
// ran the 1,024-view batch 8% faster than five (96 registers).
#ifndef CSG_VIEWS_MIN_BLOCKS
#define CSG_VIEWS_MIN_BLOCKS 6
#endif

// The persistent loop runs per warp: each warp takes its next 32-pixel warp tile from the
// counter on its own, so no warp of a block waits for another (no block barrier in the
// loop).  The item's view is the last one whose first item is not after it (binary
// search of the prefix by lane 0).
template <int SD, bool ROLLED, int NT, bool LOCAL>
__global__ void __launch_bounds__(NT, CSG_VIEWS_MIN_BLOCKS * pix::kThreads / NT) render_views(const ViewsLaunch p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint16_t tab[27];
    pix::load_table(tab);
    typename std::conditional<LOCAL, dev::LocalStacks<SD>, dev::SmemStacks<SD>>::type st;
    if constexpr (LOCAL) pix::init_stacks(st);
    else st = pix::block_stacks<SD, NT>(smem_raw);
    const pix::BlockSmem bs = pix::block_smem<SD, NT, LOCAL>(smem_raw, p.live_words);
    const int lane = threadIdx.x & 31;
    const int tw = 1 << p.tw_log2, th = 32 >> p.tw_log2;
    const int ox = lane & (tw - 1), oy = lane >> p.tw_log2;
    __syncthreads();  // the table is loaded
    for (int taken = 0; p.items_per_warp == 0 || taken < p.items_per_warp; ++taken) {
        int it = 0, vi = 0;
        if (lane == 0) {
            it = atomicAdd(p.counter, 1);
            if (it < p.n_items) {
                int lo = 0, hi = p.n_views - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (__ldg(&p.prefix[mid]) <= it) lo = mid;
                    else hi = mid - 1;
                }
                vi = lo;
            }
        }
        it = __shfl_sync(0xffffffffu, it, 0);
        vi = __shfl_sync(0xffffffffu, vi, 0);
        if (it >= p.n_items) break;
        const ViewRecord& v = p.views[vi];
        const int tile = it - __ldg(&p.prefix[vi]);
        const int tx = tile % v.tiles_x, ty = tile / v.tiles_x;
        const int x = tx * tw + ox, y = ty * th + oy;
        const bool inside = x < v.view.w && y < v.view.h;
        pix::render_pixel<SD, ROLLED>(v.view, v.status, p.iter_cap, x, y, inside, st, bs, tab,
                                      dev::ray_frame(v.view.cam.v, (float)v.view.w, (float)v.view.h));
        if (p.remaining) {
            if (v.host_out) __threadfence_system();  // this lane's host-mapped plane
            else __threadfence();
            __syncwarp();
            if (lane == 0 && atomicSub(&p.remaining[vi], 1) == 1) {
                __threadfence_system();
                *reinterpret_cast<volatile unsigned int*>(&p.done_flags[vi]) = p.epoch;
            }
        }
    }
}

template <int SD, bool ROLLED, int NT, bool LOCAL>
cudaError_t launch_views_variant(const ViewsLaunch& l, int device, cudaStream_t stream, int* grid_out)
{
    const auto kernel = render_views<SD, ROLLED, NT, LOCAL>;
    const size_t smem = pix::smem_bytes(SD, l.live_words, NT, LOCAL);
    // Resident blocks of the whole device for each (device, live-mask size), found once:
    // the opt-in for the largest shared-memory layout, the SM count and the occupancy query
    // cost more host time than the launch itself.  A fixed table (no heap allocation, for
    // the allocation-free entry point); keys that do not fit are recomputed every time.
    constexpr int kEntries = 64;
    static std::mutex mu;
    static int keys[kEntries];  // device * 256 + live words + 1; 0 = empty
    static int slots_of[kEntries];
    const int key = device * 256 + (int)l.live_words + 1;
    int slots = 0;
    {
        std::lock_guard<std::mutex> g(mu);
        int free_at = -1;
        for (int i = 0; i < kEntries; ++i) {
            if (keys[i] == key) {
                slots = slots_of[i];
                break;
            }
            if (keys[i] == 0) {
                free_at = i;
                break;
            }
        }
        if (slots == 0) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)pix::smem_bytes(SD, kLiveWordsMax, NT, LOCAL));
            int sms = 0, per_sm = 0;
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, smem);
            if (e != cudaSuccess) return e;
            slots = sms * std::max(per_sm, 1);
            if (free_at >= 0) {
                keys[free_at] = key;
                slots_of[free_at] = slots;
            }
        }
    }
    // one block per resident slot, but no more warps than items; with a bound on the items
    // per warp, enough blocks for every item
    const int warps_needed = (l.n_items + NT / 32 - 1) / (NT / 32);
    const int grid = l.items_per_warp > 0
                         ? std::max(1, (l.n_items + l.items_per_warp * (NT / 32) - 1) / (l.items_per_warp * (NT / 32)))
                         : std::max(1, std::min(slots, warps_needed));
    if (grid_out) {
        *grid_out = grid;
        return cudaSuccess;
    }
    kernel<<<grid, NT, smem, stream>>>(l);
    return cudaGetLastError();
}

template <int NT, bool LOCAL>
cudaError_t launch_views_shape(const ViewsLaunch& l, int stack_class, bool rolled, int device, cudaStream_t stream,
                               int* grid_out)
{
    switch (stack_class) {
        case 4:
            return rolled ? launch_views_variant<4, true, NT, LOCAL>(l, device, stream, grid_out)
                          : launch_views_variant<4, false, NT, LOCAL>(l, device, stream, grid_out);
        case 8:
            return rolled ? launch_views_variant<8, true, NT, LOCAL>(l, device, stream, grid_out)
                          : launch_views_variant<8, false, NT, LOCAL>(l, device, stream, grid_out);
        case 12:
            return rolled ? launch_views_variant<12, true, NT, LOCAL>(l, device, stream, grid_out)
                          : launch_views_variant<12, false, NT, LOCAL>(l, device, stream, grid_out);
        case 16:
            return rolled ? launch_views_variant<16, true, NT, LOCAL>(l, device, stream, grid_out)
                          : launch_views_variant<16, false, NT, LOCAL>(l, device, stream, grid_out);
        default:
            return rolled ? launch_views_variant<32, true, NT, LOCAL>(l, device, stream, grid_out)
                          : launch_views_variant<32, false, NT, LOCAL>(l, device, stream, grid_out);
    }
}

}  // namespace csgrt
