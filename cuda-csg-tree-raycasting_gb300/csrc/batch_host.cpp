// C ABI of batched rendering (csg_batch_* in include/csgrt.h): the batch's view table in
// longest-first order, CUDA-graph capture of the persistent view-table launch (views.hpp),
// and the tile-shape autotuner.
#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "csgrt.h"
#include "scene_handle.hpp"
#include "views.hpp"

struct csg_batch {
    std::vector<csg_view> src;             // the caller's view descriptors
    std::vector<int> order;                // views, most expensive first
    csgrt::ViewRecord* d_views = nullptr;  // device table: records, prefix, counter, status
    int32_t* d_prefix = nullptr;
    int* d_counter = nullptr;
    unsigned long long* d_status = nullptr;
    void* dmem = nullptr;
    csgrt::ViewsLaunch launch{};
    int stack_class = 4;
    bool rolled = false;
    int tile_w = 8;
    int grid = 0;
    cudaStream_t capture = nullptr;
    cudaGraphExec_t graph = nullptr;
    size_t bytes = 0;
    int device = 0;
};

namespace {

constexpr int kTileShapes[4] = {8, 4, 16, 32};  // warp tile widths tried by the autotuner

void drop_graph(csg_batch* b)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

// View table for warp tile width `tw`: records in decreasing cost order (a
// longest-processing-time-first schedule) and their tile prefix, uploaded to the device.
// Capped rays of every view are counted in the batch's own status word.
int build_table(csg_batch* b, int tw)
{
    const size_t n = b->src.size();
    std::vector<csgrt::ViewRecord> rec(n);
    std::vector<int32_t> prefix(n + 1);
    int64_t total = 0;
    for (size_t k = 0; k < n; ++k) {
        const csg_view& v = b->src[b->order[k]];
        const csgrt::Planes out{v.out.rgba8, reinterpret_cast<float4*>(v.out.rgba32f), v.out.t, v.out.prim,
                                v.out.normal};
        csgrt::make_view_record(v.scene->dev, b->d_status, reinterpret_cast<const float*>(&v.cam), v.light_dir, v.w,
                                v.h, out, tw, rec[k]);
        prefix[k] = (int32_t)total;
        total += csgrt::view_tiles(v.w, v.h, tw);
        if (total > INT_MAX) return CSG_E_CAPACITY;
    }
    prefix[n] = (int32_t)total;
    cudaError_t e = cudaMemcpy(b->d_views, rec.data(), n * sizeof(csgrt::ViewRecord), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_prefix, prefix.data(), (n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return CSG_E_CUDA;
    b->launch.n_items = (int32_t)total;
    b->launch.tw_log2 = csgrt::tile_log2(tw);
    b->tile_w = tw;
    drop_graph(b);
    if (csgrt::views_grid(b->launch, b->stack_class, b->rolled, b->device, &b->grid) != cudaSuccess) return CSG_E_CUDA;
    return CSG_OK;
}

int capture(csg_batch* b)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return CSG_E_CUDA;
    cudaError_t le = cudaMemsetAsync(b->d_counter, 0, sizeof(int), b->capture);
    if (le == cudaSuccess) le = csgrt::launch_views(b->launch, b->stack_class, b->rolled, b->device, b->capture);
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
    cudaFree(b->dmem);
    delete b;
}

}  // namespace

extern "C" {

int csg_batch_create(const csg_view* views, int32_t n_views, csg_batch** out)
{
    if (!out || !views || n_views <= 0) return CSG_E_ARG;
    *out = nullptr;
    for (int32_t i = 0; i < n_views; ++i) {
        const csg_view& v = views[i];
        if (!v.scene || v.w <= 0 || v.h <= 0) return CSG_E_ARG;
        if (v.out.rgba32f && (reinterpret_cast<uintptr_t>(v.out.rgba32f) & 15u)) return CSG_E_ARG;
    }
    csg_batch* b = new (std::nothrow) csg_batch();
    if (!b) return CSG_E_CUDA;
    cudaGetDevice(&b->device);
    b->src.assign(views, views + n_views);
    int32_t sd = 4, live = 1;
    std::vector<double> cost(n_views);
    for (int32_t i = 0; i < n_views; ++i) {
        const csg_view& v = views[i];
        cost[i] = (double)v.w * v.h * (1.0 + v.scene->dev.n_prims);
        sd = std::max(sd, v.scene->dev.stack_class);
        live = std::max(live, v.scene->dev.live_words);
        b->rolled = b->rolled || v.scene->dev.rolled;
    }
    b->order.resize(n_views);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    b->stack_class = csgrt::stack_class_for_depth(sd);

    // [records][prefix: n + 1][counter][status]
    const size_t n = (size_t)n_views;
    const size_t off_prefix = n * sizeof(csgrt::ViewRecord);
    const size_t off_counter = (off_prefix + (n + 1) * sizeof(int32_t) + 15) & ~size_t(15);
    const size_t total = off_counter + 16;
    cudaError_t e = cudaMalloc(&b->dmem, total);
    if (e == cudaSuccess) e = cudaMemset(b->dmem, 0, total);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_batch(b);
        return CSG_E_CUDA;
    }
    char* base = static_cast<char*>(b->dmem);
    b->d_views = reinterpret_cast<csgrt::ViewRecord*>(base);
    b->d_prefix = reinterpret_cast<int32_t*>(base + off_prefix);
    b->d_counter = reinterpret_cast<int*>(base + off_counter);
    b->d_status = reinterpret_cast<unsigned long long*>(base + off_counter + 8);
    b->bytes = total;
    csgrt::ViewsLaunch& l = b->launch;
    l.views = b->d_views;
    l.prefix = b->d_prefix;
    l.counter = b->d_counter;
    l.n_views = n_views;
    l.live_words = live;
    l.iter_cap = csgrt::kIterCap;
    l.remaining = nullptr;
    l.done_flags = nullptr;
    l.epoch = 0;
    const int rc = build_table(b, 8);
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
    return build_table(b, warp_tile_w);
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
        if ((rc = build_table(b, tw)) != CSG_OK) break;
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
    rc = build_table(b, best);
    if (best_tile_w) *best_tile_w = best;
    if (best_ms) *best_ms = best_t;
    return rc;
}

int csg_batch_get_info(const csg_batch* b, csg_batch_info* info)
{
    if (!b || !info) return CSG_E_ARG;
    info->n_views = static_cast<int32_t>(b->src.size());
    info->n_items = b->launch.n_items;
    info->warp_tile_w = b->tile_w;
    info->stack_class = b->stack_class;
    info->rolled = b->rolled ? 1 : 0;
    info->grid = b->grid;
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
