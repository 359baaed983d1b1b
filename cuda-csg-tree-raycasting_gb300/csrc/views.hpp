// Launch interface of the view-table kernel (views_kernel.cuh): many views of many scenes
// in one persistent launch whose work items are found by a binary search of a per-view
// tile prefix, so its tables are O(views).  Used by csg_batch (a table per tree-size
// class), csg_render_views_noalloc (tables in a fixed device array) and the render server
// (tables per in-flight batch).
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "render.hpp"

namespace csgrt {

// One view in the device table.
struct ViewRecord {
    ViewParams view;
    unsigned long long* status;  // the scene's capped-ray counter
    int32_t tiles_x;              // warp tiles per row
    int32_t host_out;             // an output plane is host memory (system-scope fences)
};
static_assert(sizeof(ViewRecord) % 8 == 0, "view record alignment");

struct ViewsLaunch {
    const ViewRecord* views;
    const int32_t* prefix;  // prefix[v] = first item of view v; prefix[n_views] = n_items
    int* counter;           // work counter: must be zero when the kernel starts
    int32_t n_views;
    int32_t n_items;
    int32_t tw_log2;        // warp tile width 1 << tw_log2, height 32 >> tw_log2
    int32_t live_words;     // max over the views
    uint32_t iter_cap;
    // Optional per-view completion (null: none).  remaining[v] starts at view v's tile
    // count; the block that renders a view's last tile stores `epoch` to done_flags[v], a
    // host-mapped word the host polls.  Every block fences its writes before counting its
    // tile (system-wide if the view writes host memory), and the last one fences again
    // system-wide before the flag.
    int* remaining;
    unsigned int* done_flags;
    unsigned int epoch;
    // Work items each warp takes before its block exits (0: persistent, the block runs until
    // the items are gone).  With a bound the grid holds enough blocks for every item and
    // blocks retire every few items, so a launch on a higher-priority stream starts as soon
    // as blocks of this one retire.
    int32_t items_per_warp = 0;
};

// Work items of a w x h view: warp tiles of tw x (32 / tw) pixels.
inline int64_t view_tiles(int32_t w, int32_t h, int tw)
{
    const int th = 32 / tw;
    return (int64_t)((w + tw - 1) / tw) * ((h + th - 1) / th);
}

inline int tile_log2(int tw)
{
    return tw == 4 ? 2 : tw == 8 ? 3 : tw == 16 ? 4 : 5;
}

inline void make_view_record(const DeviceScene& scene, unsigned long long* status, const float cam[15],
                             const float light[3], int32_t w, int32_t h, const Planes& out, int tw, ViewRecord& r)
{
    r = ViewRecord{};
    r.view.scene = scene;
    std::memcpy(r.view.cam.v, cam, sizeof(r.view.cam.v));
    r.view.light[0] = light[0];
    r.view.light[1] = light[1];
    r.view.light[2] = light[2];
    r.view.w = w;
    r.view.h = h;
    r.view.out = out;
    r.status = status;
    r.tiles_x = (w + tw - 1) / tw;
    r.host_out = 0;
}

// Block shape of a view-table launch: warps per block (2, 4 or 8) and where the per-ray
// primitive and time stacks live (block shared memory, or per-thread local memory, which
// leaves shared memory to the live masks and more of the SM's L1 to the scene).  Every
// shape renders the same bytes; the batch autotuner picks one per tree-size class.
struct ViewsShape {
    int warps = 4;
    bool local_stacks = false;
};
constexpr ViewsShape kViewsShapes[4] = {{4, false}, {2, false}, {8, false}, {4, true}};

inline bool valid_shape(const ViewsShape& s)
{
    for (const ViewsShape& k : kViewsShapes)
        if (k.warps == s.warps && k.local_stacks == s.local_stacks) return true;
    return false;
}

// Enqueues the view-table kernel variant for (stack_class, rolled, shape) on `stream`,
// with a grid that fills `device` once (capturable: the host calls it makes enqueue
// nothing else).
cudaError_t launch_views(const ViewsLaunch& l, int stack_class, bool rolled, ViewsShape shape, int device,
                         cudaStream_t stream);
// The grid launch_views would use.
cudaError_t views_grid(const ViewsLaunch& l, int stack_class, bool rolled, ViewsShape shape, int device, int* grid);

// One block shape's launcher (views_kernel.cuh), instantiated for the shapes of
// kViewsShapes; grid_out != null only computes the grid.
template <int NT, bool LOCAL>
cudaError_t launch_views_shape(const ViewsLaunch& l, int stack_class, bool rolled, int device, cudaStream_t stream,
                               int* grid_out);

}  // namespace csgrt
