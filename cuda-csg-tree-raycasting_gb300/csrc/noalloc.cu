// The view-table kernel (views.hpp) and csg_render_views_noalloc, the batched persistent
// render for callers that must not allocate device memory.
//
// Some callers cannot allocate at render time.  A server running at its device-memory
// budget has no headroom for a per-request batch object, and a failed cudaMalloc there
// would drop the request.  A frame loop cannot afford cudaFree, which synchronises the
// whole device and stalls every other stream.  This entry point therefore keeps all of
// its scratch -- the work counter, the view table and the per-view tile prefix -- in one
// file-scope device array of fixed size (kScratchBytes, room for kMaxViews views), and
// the call itself allocates nothing on the device or on the host heap.  The descriptors
// are built in fixed-size stack buffers and reach the array as kernel parameters of small
// fill launches (so no host buffer has to outlive the call, and no copy from pageable
// memory is involved).
//
// Work items are not listed: item i is warp tile i - prefix[v] of the view v found by a
// binary search of the tile prefix, and the views are stored longest-first, so the launch
// needs O(views) scratch, not a list of its tiles.  The per-pixel
// code is pix::render_pixel, shared with the single-view and batched kernels, so every
// view's planes are the bytes csg_render_planes writes.
//
// Only the work counter must start at zero; every call's first fill launch clears it on
// the call's stream, ahead of the render launch.  Rays stopped at the iteration cap are
// counted in each view's scene, as csg_render_planes counts them, and csg_scene_check
// reports them.
//
// All calls share the one array per device: two calls whose work can overlap on the
// device (different streams, or different host threads without ordering) race on it and
// must be serialised by the caller.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstring>

#include "csgrt.h"
#include "pixel.cuh"
#include "scene_handle.hpp"
#include "views.hpp"

namespace csgrt {
namespace {

using pix::kThreads;

constexpr int kMaxViews = CSG_NOALLOC_MAX_VIEWS;

// Scratch layout: [work counter | pad to 256 B][views, longest first][tile prefix].
constexpr size_t kViewsOffset = 256;
constexpr size_t kPrefixOffset = kViewsOffset + sizeof(ViewRecord) * kMaxViews;
constexpr size_t kScratchBytes = 1u << 20;
static_assert(kPrefixOffset + sizeof(int32_t) * (kMaxViews + 1) <= kScratchBytes, "scratch too small");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The persistent loop runs per warp: each warp takes its next 32-pixel warp tile from the
// counter on its own, so no warp of a block waits for another (no block barrier in the
// loop).  The item's view is the last one whose first item is not after it (binary
// search of the prefix by lane 0).
// Minimum resident blocks per SM asked of the register allocator (a tuning knob): six
// blocks (80 registers) ran the 1,024-view batch 8% faster than five (96 registers).
#ifndef CSG_VIEWS_MIN_BLOCKS
#define CSG_VIEWS_MIN_BLOCKS 6
#endif
template <int SD, bool ROLLED>
__global__ void __launch_bounds__(kThreads, CSG_VIEWS_MIN_BLOCKS) render_views(const ViewsLaunch p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint16_t tab[27];
    pix::load_table(tab);
    dev::SmemStacks<SD> st = pix::block_stacks<SD>(smem_raw);
    const pix::BlockSmem bs = pix::block_smem<SD>(smem_raw, p.live_words);
    const int lane = threadIdx.x & 31;
    const int tw = 1 << p.tw_log2, th = 32 >> p.tw_log2;
    const int ox = lane & (tw - 1), oy = lane >> p.tw_log2;
    __syncthreads();  // the table is loaded
    while (true) {
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
        pix::render_pixel<SD, ROLLED>(v.view, v.status, p.iter_cap, x, y, inside, st, bs, tab);
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

// One fill launch: up to kChunk view records and their tile prefixes, passed by value.
constexpr int kChunk = 112;
struct FillChunk {
    ViewRecord rec[kChunk];
    int32_t prefix[kChunk];
    int32_t k0, n;       // first view slot, records in this chunk
    int32_t total;       // items of the whole call (written after the last view's prefix)
    int32_t last;        // this chunk holds the last view
};
static_assert(sizeof(FillChunk) <= 32000, "kernel parameter space");

__global__ void fill_scratch(const __grid_constant__ FillChunk c, unsigned char* scratch)
{
    constexpr int kWords = sizeof(ViewRecord) / 8;
    const uint64_t* src = reinterpret_cast<const uint64_t*>(&c.rec[0]);
    uint64_t* dst = reinterpret_cast<uint64_t*>(scratch + kViewsOffset + sizeof(ViewRecord) * c.k0);
    for (int i = threadIdx.x; i < c.n * kWords; i += blockDim.x) dst[i] = src[i];
    int32_t* pf = reinterpret_cast<int32_t*>(scratch + kPrefixOffset);
    for (int i = threadIdx.x; i < c.n; i += blockDim.x) pf[c.k0 + i] = c.prefix[i];
    if (threadIdx.x == 0) {
        if (c.last) pf[c.k0 + c.n] = c.total;
        if (c.k0 == 0) *reinterpret_cast<int*>(scratch) = 0;  // the work counter
    }
}

template <int SD, bool ROLLED>
cudaError_t launch_variant(const ViewsLaunch& l, int device, cudaStream_t stream, int* grid_out)
{
    const auto kernel = render_views<SD, ROLLED>;
    const size_t smem = pix::smem_bytes(SD, l.live_words);
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int sms = 0, per_sm = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
    if (e != cudaSuccess) return e;
    // one block per resident slot, but no more warps than items
    int grid = sms * std::max(per_sm, 1);
    grid = std::max(1, std::min(grid, (l.n_items + kThreads / 32 - 1) / (kThreads / 32)));
    if (grid_out) {
        *grid_out = grid;
        return cudaSuccess;
    }
    kernel<<<grid, kThreads, smem, stream>>>(l);
    return cudaGetLastError();
}

// Address of the scratch array on each device, looked up on the first call there.
constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_scratch_addr[kMaxDevices];

unsigned char* scratch_on(int device)
{
    if (device < 0 || device >= kMaxDevices) return nullptr;
    unsigned char* p = g_scratch_addr[device].load(std::memory_order_acquire);
    if (p) return p;
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_scratch) != cudaSuccess || !addr) return nullptr;
    p = static_cast<unsigned char*>(addr);
    g_scratch_addr[device].store(p, std::memory_order_release);
    return p;
}

double view_cost(const csg_view& v)
{
    return (double)v.w * (double)v.h * (1.0 + v.scene->dev.n_prims);
}

}  // namespace

namespace {

cudaError_t dispatch(const ViewsLaunch& l, int stack_class, bool rolled, int device, cudaStream_t stream,
                     int* grid)
{
    switch (stack_class) {
        case 4:
            return rolled ? launch_variant<4, true>(l, device, stream, grid)
                          : launch_variant<4, false>(l, device, stream, grid);
        case 8:
            return rolled ? launch_variant<8, true>(l, device, stream, grid)
                          : launch_variant<8, false>(l, device, stream, grid);
        case 12:
            return rolled ? launch_variant<12, true>(l, device, stream, grid)
                          : launch_variant<12, false>(l, device, stream, grid);
        case 16:
            return rolled ? launch_variant<16, true>(l, device, stream, grid)
                          : launch_variant<16, false>(l, device, stream, grid);
        default:
            return rolled ? launch_variant<32, true>(l, device, stream, grid)
                          : launch_variant<32, false>(l, device, stream, grid);
    }
}

}  // namespace

cudaError_t launch_views(const ViewsLaunch& l, int stack_class, bool rolled, int device, cudaStream_t stream)
{
    return dispatch(l, stack_class, rolled, device, stream, nullptr);
}

cudaError_t views_grid(const ViewsLaunch& l, int stack_class, bool rolled, int device, int* grid)
{
    return dispatch(l, stack_class, rolled, device, nullptr, grid);
}

}  // namespace csgrt

extern "C" int csg_render_views_noalloc(const csg_view* views, int32_t n_views, int32_t warp_tile_w, void* stream)
{
    using namespace csgrt;
    if (!views || n_views <= 0) return CSG_E_ARG;
    if (n_views > kMaxViews) return CSG_E_CAPACITY;
    if (warp_tile_w == 0) warp_tile_w = 8;
    if (warp_tile_w != 4 && warp_tile_w != 8 && warp_tile_w != 16 && warp_tile_w != 32) return CSG_E_ARG;
    const int tw = warp_tile_w;
    int32_t sd = 4, live = 1;
    bool rolled = false;
    for (int32_t i = 0; i < n_views; ++i) {
        const csg_view& v = views[i];
        if (!v.scene || v.w <= 0 || v.h <= 0) return CSG_E_ARG;
        if (v.out.rgba32f && (reinterpret_cast<uintptr_t>(v.out.rgba32f) & 15u)) return CSG_E_ARG;
        sd = std::max(sd, v.scene->dev.stack_class);
        live = std::max(live, v.scene->dev.live_words);
        rolled = rolled || v.scene->dev.rolled;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return CSG_E_CUDA;
    unsigned char* scratch = scratch_on(device);
    if (!scratch) return CSG_E_CUDA;

    // Longest-first order and the tile prefix, in fixed-size stack buffers.
    int32_t order[kMaxViews];
    int32_t prefix[kMaxViews + 1];
    for (int32_t i = 0; i < n_views; ++i) order[i] = i;
    std::sort(order, order + n_views, [&](int32_t a, int32_t b) {
        const double ca = view_cost(views[a]), cb = view_cost(views[b]);
        return ca > cb || (ca == cb && a < b);
    });
    long long total = 0;
    for (int32_t k = 0; k < n_views; ++k) {
        const csg_view& v = views[order[k]];
        prefix[k] = static_cast<int32_t>(total);
        total += view_tiles(v.w, v.h, tw);
        if (total > INT_MAX) return CSG_E_CAPACITY;
    }
    prefix[n_views] = static_cast<int32_t>(total);

    // View records and prefixes, by value through the fill launches' parameters.
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    FillChunk c;
    for (int32_t k0 = 0; k0 < n_views; k0 += kChunk) {
        const int32_t n = std::min<int32_t>(kChunk, n_views - k0);
        for (int32_t j = 0; j < n; ++j) {
            const csg_view& v = views[order[k0 + j]];
            const Planes out{v.out.rgba8, reinterpret_cast<float4*>(v.out.rgba32f), v.out.t, v.out.prim,
                             v.out.normal};
            make_view_record(v.scene->dev, v.scene->status, reinterpret_cast<const float*>(&v.cam), v.light_dir,
                             v.w, v.h, out, tw, c.rec[j]);
            c.prefix[j] = prefix[k0 + j];
        }
        c.k0 = k0;
        c.n = n;
        c.total = static_cast<int32_t>(total);
        c.last = (k0 + n == n_views) ? 1 : 0;
        fill_scratch<<<1, 256, 0, st>>>(c, scratch);
        if (cudaGetLastError() != cudaSuccess) return CSG_E_CUDA;
    }

    ViewsLaunch l;
    l.views = reinterpret_cast<const ViewRecord*>(scratch + kViewsOffset);
    l.prefix = reinterpret_cast<const int32_t*>(scratch + kPrefixOffset);
    l.counter = reinterpret_cast<int*>(scratch);
    l.n_views = n_views;
    l.n_items = static_cast<int32_t>(total);
    l.tw_log2 = tile_log2(tw);
    l.live_words = live;
    l.iter_cap = kIterCap;
    l.remaining = nullptr;
    l.done_flags = nullptr;
    l.epoch = 0;
    return launch_views(l, stack_class_for_depth(sd), rolled, device, st) == cudaSuccess ? CSG_OK : CSG_E_CUDA;
}
