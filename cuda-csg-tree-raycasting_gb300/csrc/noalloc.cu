// The view-table launcher (views.hpp; the default block shape is instantiated here, the
// kernel lives in views_kernel.cuh) and csg_render_views_noalloc, the batched persistent
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
// One call renders all its views with one kernel variant: the largest stack class and
// live mask of its views, and the rolled GoTo loop if any view's scene has it.  The planes
// are the same whatever the variant, but one large tree gives every view of the call its
// large live mask, and one tree deeper than 15 operator levels its 32-entry stacks (fewer
// resident blocks, and the guard on every skip), so callers should group views by tree
// class, as csg_batch does.
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
#include "planes.hpp"
#include "scene_handle.hpp"
#include "views_kernel.cuh"

namespace csgrt {
namespace {

constexpr int kMaxViews = CSG_NOALLOC_MAX_VIEWS;

// Scratch layout: [work counter | pad to 256 B][views, longest first][tile prefix].
constexpr size_t kViewsOffset = 256;
constexpr size_t kPrefixOffset = kViewsOffset + sizeof(ViewRecord) * kMaxViews;
constexpr size_t kScratchBytes = 1u << 20;
static_assert(kPrefixOffset + sizeof(int32_t) * (kMaxViews + 1) <= kScratchBytes, "scratch too small");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// One fill launch: up to kChunk view records and their tile prefixes, passed by value
// (12 KB of the calling thread's stack; the whole call uses about 21 KB of it).
constexpr int kChunk = 56;
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

// The other shapes are instantiated in views_shapes_*.cu (compiled in parallel).
extern template cudaError_t launch_views_shape<64, false>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);
extern template cudaError_t launch_views_shape<256, false>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);
extern template cudaError_t launch_views_shape<128, true>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);

cudaError_t launch_views(const ViewsLaunch& l, int stack_class, bool rolled, ViewsShape shape, int device,
                         cudaStream_t stream)
{
    if (shape.local_stacks) return launch_views_shape<128, true>(l, stack_class, rolled, device, stream, nullptr);
    if (shape.warps == 2) return launch_views_shape<64, false>(l, stack_class, rolled, device, stream, nullptr);
    if (shape.warps == 8) return launch_views_shape<256, false>(l, stack_class, rolled, device, stream, nullptr);
    return launch_views_shape<128, false>(l, stack_class, rolled, device, stream, nullptr);
}

cudaError_t views_grid(const ViewsLaunch& l, int stack_class, bool rolled, ViewsShape shape, int device, int* grid)
{
    if (shape.local_stacks) return launch_views_shape<128, true>(l, stack_class, rolled, device, nullptr, grid);
    if (shape.warps == 2) return launch_views_shape<64, false>(l, stack_class, rolled, device, nullptr, grid);
    if (shape.warps == 8) return launch_views_shape<256, false>(l, stack_class, rolled, device, nullptr, grid);
    return launch_views_shape<128, false>(l, stack_class, rolled, device, nullptr, grid);
}

template cudaError_t launch_views_shape<128, false>(const ViewsLaunch&, int, bool, int, cudaStream_t, int*);

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
        csg_planes dp = v.out;  // checked before anything is enqueued
        if (device_planes(dp) != CSG_OK) return CSG_E_ARG;
        sd = std::max(sd, v.scene->dev.stack_class);
        live = std::max(live, v.scene->dev.live_words);
        rolled = rolled || v.scene->dev.rolled;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return CSG_E_CUDA;
    unsigned char* scratch = scratch_on(device);
    if (!scratch) return CSG_E_CUDA;

    // Longest-first order (a fixed-size stack buffer of 16-bit view numbers) and the
    // total of warp tiles, checked before anything is enqueued.
    static_assert(kMaxViews <= 32768, "view numbers are 16-bit");
    int16_t order[kMaxViews];
    for (int32_t i = 0; i < n_views; ++i) order[i] = static_cast<int16_t>(i);
    std::sort(order, order + n_views, [&](int16_t a, int16_t b) {
        const double ca = view_cost(views[a]), cb = view_cost(views[b]);
        return ca > cb || (ca == cb && a < b);
    });
    long long total = 0;
    for (int32_t k = 0; k < n_views; ++k) {
        const csg_view& v = views[order[k]];
        total += view_tiles(v.w, v.h, tw);
        if (total > INT_MAX) return CSG_E_CAPACITY;
    }

    // View records and tile prefixes, by value through the fill launches' parameters.
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    FillChunk c;
    long long first_item = 0;
    for (int32_t k0 = 0; k0 < n_views; k0 += kChunk) {
        const int32_t n = std::min<int32_t>(kChunk, n_views - k0);
        for (int32_t j = 0; j < n; ++j) {
            const csg_view& v = views[order[k0 + j]];
            csg_planes dp = v.out;
            device_planes(dp);  // checked above
            const Planes out{dp.rgba8, reinterpret_cast<float4*>(dp.rgba32f), dp.t, dp.prim, dp.normal};
            make_view_record(v.scene->dev, v.scene->status, reinterpret_cast<const float*>(&v.cam), v.light_dir,
                             v.w, v.h, out, tw, c.rec[j]);
            c.prefix[j] = static_cast<int32_t>(first_item);
            first_item += view_tiles(v.w, v.h, tw);
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
    l.iter_cap = iteration_cap();
    l.remaining = nullptr;
    l.done_flags = nullptr;
    l.epoch = 0;
    return launch_views(l, stack_class_for_depth(sd), rolled, ViewsShape{}, device, st) == cudaSuccess ? CSG_OK
                                                                                                  : CSG_E_CUDA;
}
