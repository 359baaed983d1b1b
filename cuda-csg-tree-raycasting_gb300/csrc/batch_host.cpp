// C ABI of batched rendering (csg_batch_* in include/csgrt.h): view descriptors, the
// longest-first work list, CUDA-graph capture of the persistent launch, and the tile-shape
// autotuner.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "batch.hpp"
#include "csgrt.h"
#include "scene_handle.hpp"

struct csg_batch {
    std::vector<csgrt::BatchView> views;  // host copies (tiles_x depends on the tile shape)
    std::vector<double> cost;             // per-view cost estimate, for the longest-first order
    csgrt::BatchView* d_views = nullptr;
    csgrt::BatchItem* d_items = nullptr;
    int* d_counter = nullptr;
    unsigned long long* d_status = nullptr;
    size_t item_capacity = 0;
    csgrt::BatchLaunch launch{};
    cudaStream_t capture = nullptr;
    cudaGraphExec_t graph = nullptr;
    size_t bytes = 0;
    int device = 0;
};

namespace {

constexpr int kTileShapes[4] = {8, 4, 16, 32};  // warp tile widths tried by the autotuner

int log2i(int v)
{
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

size_t tiles_of(int w, int h, int tw)
{
    const int th = 32 / tw;
    return (size_t)((w + 2 * tw - 1) / (2 * tw)) * (size_t)((h + 2 * th - 1) / (2 * th));
}

void drop_graph(csg_batch* b)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

// Work list for warp tile width `tw`: every view's block tiles, views in decreasing cost
// order (a longest-processing-time-first schedule), uploaded to the device.
int build_items(csg_batch* b, int tw)
{
    const int th = 32 / tw;
    std::vector<int> order(b->views.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->cost[a] > b->cost[c]; });
    std::vector<csgrt::BatchItem> items;
    for (auto& v : b->views) v.tiles_x = (v.view.w + 2 * tw - 1) / (2 * tw);
    for (int vi : order) {
        const csgrt::BatchView& v = b->views[vi];
        const int ntiles = v.tiles_x * ((v.view.h + 2 * th - 1) / (2 * th));
        for (int t = 0; t < ntiles; ++t) items.push_back(csgrt::BatchItem{vi, t});
    }
    if (items.size() > b->item_capacity) return CSG_E_CAPACITY;
    cudaError_t e = cudaMemcpy(b->d_views, b->views.data(), b->views.size() * sizeof(csgrt::BatchView),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(csgrt::BatchItem), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return CSG_E_CUDA;
    b->launch.n_items = static_cast<int32_t>(items.size());
    b->launch.tw_log2 = log2i(tw);
    drop_graph(b);
    return CSG_OK;
}

int capture(csg_batch* b)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return CSG_E_CUDA;
    const cudaError_t le = csgrt::launch_batch(b->launch, b->capture);
    e = cudaStreamEndCapture(b->capture, &g);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return CSG_E_CUDA;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    return e == cudaSuccess ? CSG_OK : CSG_E_CUDA;
}

void free_batch(csg_batch* b)
{
    drop_graph(b);
    if (b->capture) cudaStreamDestroy(b->capture);
    cudaFree(b->d_views);
    cudaFree(b->d_items);
    cudaFree(b->d_counter);
    cudaFree(b->d_status);
    delete b;
}

}  // namespace

extern "C" {

int csg_batch_create(const csg_view* views, int32_t n_views, csg_batch** out)
{
    if (!out || !views || n_views <= 0) return CSG_E_ARG;
    *out = nullptr;
    csg_batch* b = new (std::nothrow) csg_batch();
    if (!b) return CSG_E_CUDA;
    cudaGetDevice(&b->device);
    int32_t sd = 4, live = 1;
    bool rolled = false;
    size_t cap = 0;
    for (int32_t i = 0; i < n_views; ++i) {
        const csg_view& v = views[i];
        if (!v.scene || v.w <= 0 || v.h <= 0) {
            delete b;
            return CSG_E_ARG;
        }
        if (v.out.rgba32f && (reinterpret_cast<uintptr_t>(v.out.rgba32f) & 15u)) {
            delete b;
            return CSG_E_ARG;
        }
        csgrt::BatchView bv{};
        bv.view.scene = v.scene->dev;
        std::memcpy(bv.view.cam.v, &v.cam, sizeof(bv.view.cam.v));
        bv.view.light[0] = v.light_dir[0];
        bv.view.light[1] = v.light_dir[1];
        bv.view.light[2] = v.light_dir[2];
        bv.view.w = v.w;
        bv.view.h = v.h;
        bv.view.out.rgba8 = v.out.rgba8;
        bv.view.out.rgba32f = reinterpret_cast<float4*>(v.out.rgba32f);
        bv.view.out.t = v.out.t;
        bv.view.out.prim = v.out.prim;
        bv.view.out.normal = v.out.normal;
        b->views.push_back(bv);
        b->cost.push_back((double)v.w * v.h * (1.0 + v.scene->dev.n_prims));
        sd = std::max(sd, v.scene->dev.stack_class);
        live = std::max(live, v.scene->dev.live_words);
        rolled = rolled || v.scene->dev.rolled;
        size_t most = 0;
        for (int tw : kTileShapes) most = std::max(most, tiles_of(v.w, v.h, tw));
        cap += most;
    }
    b->item_capacity = cap;
    cudaError_t e = cudaMalloc(&b->d_views, b->views.size() * sizeof(csgrt::BatchView));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_items, cap * sizeof(csgrt::BatchItem));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_batch(b);
        return CSG_E_CUDA;
    }
    b->bytes = b->views.size() * sizeof(csgrt::BatchView) + cap * sizeof(csgrt::BatchItem) + 16;
    csgrt::BatchLaunch& l = b->launch;
    l.views = b->d_views;
    l.items = b->d_items;
    l.counter = b->d_counter;
    l.status = b->d_status;
    l.live_words = live;
    l.iter_cap = csgrt::kIterCap;
    l.stack_class = csgrt::stack_class_for_depth(sd);
    l.rolled = rolled ? 1 : 0;
    if (csgrt::batch_grid_size(l) != cudaSuccess) {
        free_batch(b);
        return CSG_E_CUDA;
    }
    const int rc = build_items(b, 8);
    if (rc != CSG_OK) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return CSG_OK;
}

int csg_batch_destroy(csg_batch* b)
{
    if (!b) return CSG_E_ARG;
    free_batch(b);
    return CSG_OK;
}

int csg_batch_set_tile(csg_batch* b, int32_t warp_tile_w)
{
    if (!b) return CSG_E_ARG;
    if (warp_tile_w != 4 && warp_tile_w != 8 && warp_tile_w != 16 && warp_tile_w != 32) return CSG_E_ARG;
    return build_items(b, warp_tile_w);
}

int csg_batch_render(csg_batch* b, void* stream)
{
    if (!b) return CSG_E_ARG;
    if (!b->graph) {
        const int rc = capture(b);
        if (rc != CSG_OK) return rc;
    }
    return cudaGraphLaunch(b->graph, static_cast<cudaStream_t>(stream)) == cudaSuccess ? CSG_OK : CSG_E_CUDA;
}

int csg_batch_tune(csg_batch* b, void* stream, int32_t* best_tile_w, float* best_ms)
{
    if (!b) return CSG_E_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return CSG_E_CUDA;
    int best = 8;
    float best_t = 0.f;
    int rc = CSG_OK;
    for (int tw : kTileShapes) {
        if ((rc = build_items(b, tw)) != CSG_OK) break;
        if ((rc = csg_batch_render(b, stream)) != CSG_OK) break;  // warm-up (and capture)
        float total = 0.f;
        for (int r = 0; r < 3 && rc == CSG_OK; ++r) {
            cudaEventRecord(e0, st);
            rc = csg_batch_render(b, stream);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = CSG_E_CUDA;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            total += ms;
        }
        if (rc != CSG_OK) break;
        if (best_t == 0.f || total / 3 < best_t) {
            best_t = total / 3;
            best = tw;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != CSG_OK) return rc;
    rc = build_items(b, best);
    if (best_tile_w) *best_tile_w = best;
    if (best_ms) *best_ms = best_t;
    return rc;
}

int csg_batch_get_info(const csg_batch* b, csg_batch_info* info)
{
    if (!b || !info) return CSG_E_ARG;
    info->n_views = static_cast<int32_t>(b->views.size());
    info->n_items = b->launch.n_items;
    info->warp_tile_w = 1 << b->launch.tw_log2;
    info->stack_class = b->launch.stack_class;
    info->rolled = b->launch.rolled;
    info->grid = b->launch.grid;
    info->device_bytes = b->bytes;
    return CSG_OK;
}

int csg_batch_check(csg_batch* b, void* stream, uint64_t* n_capped)
{
    if (!b) return CSG_E_ARG;
    unsigned long long v = 0;
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaMemcpy(&v, b->d_status, sizeof(v), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(v));
    if (e != cudaSuccess) return CSG_E_CUDA;
    if (n_capped) *n_capped = v;
    return v ? CSG_E_TIMEOUT : CSG_OK;
}

}  // extern "C"
