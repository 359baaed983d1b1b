// C ABI of batched rendering (csg_batch_* in include/csgrt.h).
//
// A batch is split into tree-size classes: views whose scenes need the same kernel
// variant (stack capacity, rolled or unrolled GoTo) and a similar live-mask size (the
// shared memory per block, hence the blocks per SM) form one class.  Each class has its
// own view table (views most expensive first), its own persistent view-table launch
// (views.hpp) with that class's variant, and its own warp tile shape and block shape
// (warps per block, stack placement), chosen by the autotuner per class.  All class launches are captured into one CUDA graph as
// independent branches, so they share the GPU: the light classes fill the SMs the heavy
// class's tail leaves idle.
#include <algorithm>
#include <climits>
#include <cstring>
#include <map>
#include <new>
#include <numeric>
#include <tuple>
#include <vector>

#include "csgrt.h"
#include "planes.hpp"
#include "scene_handle.hpp"
#include "views.hpp"

namespace {

struct BatchClass {
    int stack_class = 4;
    bool rolled = false;
    int live_words = 1;
    std::vector<int> views;  // indices into the batch's views, most expensive first
    csgrt::ViewRecord* d_views = nullptr;
    int32_t* d_prefix = nullptr;
    int* d_counter = nullptr;
    csgrt::ViewsLaunch launch{};
    int tile_w = 8;
    csgrt::ViewsShape shape{};
    float tuned_ms = 0.f;  // this class alone at its chosen configuration (after tuning)
    int grid = 0;
    cudaStream_t stream = nullptr;  // its branch of the captured graph
    cudaEvent_t done = nullptr;
};

}  // namespace

struct csg_batch {
    std::vector<csg_view> src;
    std::vector<BatchClass> classes;
    unsigned long long* d_status = nullptr;
    void* dmem = nullptr;
    cudaStream_t capture = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t graph = nullptr;
    size_t bytes = 0;
    int device = 0;
};

namespace {

constexpr int kTileShapes[4] = {8, 4, 16, 32};  // warp tile widths tried by the autotuner

int live_bucket(int words)
{
    int b = 1;
    while (b < words) b <<= 1;
    return b;
}

void drop_graph(csg_batch* b)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

// Class c's table for warp tile width `tw`: its views' records in order and their tile
// prefix.  Capped rays of every view are counted in the batch's own status word.
int build_table(csg_batch* b, BatchClass& c, int tw)
{
    const size_t n = c.views.size();
    std::vector<csgrt::ViewRecord> rec(n);
    std::vector<int32_t> prefix(n + 1);
    int64_t total = 0;
    for (size_t k = 0; k < n; ++k) {
        const csg_view& v = b->src[c.views[k]];
        const csgrt::Planes out{v.out.rgba8, reinterpret_cast<float4*>(v.out.rgba32f), v.out.t, v.out.prim,
                                v.out.normal};
        csgrt::make_view_record(v.scene->dev, b->d_status, reinterpret_cast<const float*>(&v.cam), v.light_dir, v.w,
                                v.h, out, tw, rec[k]);
        prefix[k] = (int32_t)total;
        total += csgrt::view_tiles(v.w, v.h, tw);
        if (total > INT_MAX) return CSG_E_CAPACITY;
    }
    prefix[n] = (int32_t)total;
    cudaError_t e = cudaMemcpy(c.d_views, rec.data(), n * sizeof(csgrt::ViewRecord), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c.d_prefix, prefix.data(), (n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return CSG_E_CUDA;
    c.launch.n_items = (int32_t)total;
    c.launch.tw_log2 = csgrt::tile_log2(tw);
    c.tile_w = tw;
    drop_graph(b);
    if (csgrt::views_grid(c.launch, c.stack_class, c.rolled, c.shape, b->device, &c.grid) != cudaSuccess)
        return CSG_E_CUDA;
    return CSG_OK;
}

// Class c's block shape (warps per block, stack placement).
int set_shape(csg_batch* b, BatchClass& c, csgrt::ViewsShape s)
{
    c.shape = s;
    drop_graph(b);
    if (csgrt::views_grid(c.launch, c.stack_class, c.rolled, c.shape, b->device, &c.grid) != cudaSuccess)
        return CSG_E_CUDA;
    return CSG_OK;
}

// One class's work on `st`: counter reset and the persistent launch.
cudaError_t enqueue_class(const csg_batch* b, const BatchClass& c, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(c.d_counter, 0, sizeof(int), st);
    if (e == cudaSuccess) e = csgrt::launch_views(c.launch, c.stack_class, c.rolled, c.shape, b->device, st);
    return e;
}

int capture(csg_batch* b)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return CSG_E_CUDA;
    cudaError_t le = cudaEventRecord(b->fork, b->capture);
    for (const BatchClass& c : b->classes) {  // heaviest class first: its blocks start first
        if (le == cudaSuccess) le = cudaStreamWaitEvent(c.stream, b->fork, 0);
        if (le == cudaSuccess) le = enqueue_class(b, c, c.stream);
        if (le == cudaSuccess) le = cudaEventRecord(c.done, c.stream);
        if (le == cudaSuccess) le = cudaStreamWaitEvent(b->capture, c.done, 0);
    }
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
    for (BatchClass& c : b->classes) {
        if (c.stream) cudaStreamDestroy(c.stream);
        if (c.done) cudaEventDestroy(c.done);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->capture) cudaStreamDestroy(b->capture);
    cudaFree(b->dmem);
    delete b;
}

// Mean time of `reps` launches of class c alone, after one warm-up.
int time_class(csg_batch* b, BatchClass& c, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, int reps, float* ms)
{
    if (enqueue_class(b, c, st) != cudaSuccess) return CSG_E_CUDA;
    float total = 0.f;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, st);
        if (enqueue_class(b, c, st) != cudaSuccess) return CSG_E_CUDA;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) return CSG_E_CUDA;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        total += t;
    }
    *ms = total / reps;
    return CSG_OK;
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
    for (csg_view& v : b->src) {
        const int rc = csgrt::device_planes(v.out);
        if (rc != CSG_OK) {
            delete b;
            return rc;
        }
    }

    // tree-size classes, keyed by kernel variant and live-mask size
    std::vector<double> cost(n_views);
    std::map<std::tuple<int, int, int>, std::vector<int>> groups;
    for (int32_t i = 0; i < n_views; ++i) {
        const csgrt::DeviceScene& d = views[i].scene->dev;
        cost[i] = (double)views[i].w * views[i].h * (1.0 + d.n_prims);
        groups[{csgrt::stack_class_for_depth(d.stack_class), d.rolled ? 1 : 0, live_bucket(d.live_words)}].push_back(i);
    }
    for (auto& kv : groups) {
        BatchClass c;
        c.stack_class = std::get<0>(kv.first);
        c.rolled = std::get<1>(kv.first) != 0;
        c.live_words = std::get<2>(kv.first);
        c.views = kv.second;
        std::stable_sort(c.views.begin(), c.views.end(), [&](int a, int z) { return cost[a] > cost[z]; });
        b->classes.push_back(std::move(c));
    }
    auto class_cost = [&](const BatchClass& c) {
        double s = 0;
        for (int v : c.views) s += cost[v];
        return s;
    };
    std::stable_sort(b->classes.begin(), b->classes.end(),
                     [&](const BatchClass& a, const BatchClass& z) { return class_cost(a) > class_cost(z); });

    // one allocation: [status | per class: records, prefix, counter]
    size_t total = 16;
    std::vector<size_t> off(b->classes.size());
    for (size_t k = 0; k < b->classes.size(); ++k) {
        const size_t n = b->classes[k].views.size();
        off[k] = total;
        total += n * sizeof(csgrt::ViewRecord) + (n + 1) * sizeof(int32_t);
        total = ((total + 15) & ~size_t(15)) + 16;  // + the counter
    }
    cudaError_t e = cudaMalloc(&b->dmem, total);
    if (e == cudaSuccess) e = cudaMemset(b->dmem, 0, total);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (BatchClass& c : b->classes) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        free_batch(b);
        return CSG_E_CUDA;
    }
    char* base = static_cast<char*>(b->dmem);
    b->d_status = reinterpret_cast<unsigned long long*>(base);
    b->bytes = total;
    for (size_t k = 0; k < b->classes.size(); ++k) {
        BatchClass& c = b->classes[k];
        const size_t n = c.views.size();
        c.d_views = reinterpret_cast<csgrt::ViewRecord*>(base + off[k]);
        c.d_prefix = reinterpret_cast<int32_t*>(base + off[k] + n * sizeof(csgrt::ViewRecord));
        const size_t end = off[k] + n * sizeof(csgrt::ViewRecord) + (n + 1) * sizeof(int32_t);
        c.d_counter = reinterpret_cast<int*>(base + ((end + 15) & ~size_t(15)));
        csgrt::ViewsLaunch& l = c.launch;
        l.views = c.d_views;
        l.prefix = c.d_prefix;
        l.counter = c.d_counter;
        l.n_views = (int32_t)n;
        l.live_words = c.live_words;
        l.iter_cap = csgrt::iteration_cap();
        l.remaining = nullptr;
        l.done_flags = nullptr;
        l.epoch = 0;
        const int rc = build_table(b, c, 8);
        if (rc != CSG_OK) {
            free_batch(b);
            return rc;
        }
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
    for (BatchClass& c : b->classes) {
        const int rc = build_table(b, c, warp_tile_w);
        if (rc != CSG_OK) return rc;
    }
    return CSG_OK;
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

// Autotuner, per class alone (one warm-up and three timed launches per configuration):
// every warp tile shape with the default block shape, then every other block shape
// (warps per block, stack placement) with the best tile; keeps each class's fastest,
// then times the whole batch.
int csg_batch_tune(csg_batch* b, void* stream, int32_t* best_tile_w, float* best_ms)
{
    if (!b) return CSG_E_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return CSG_E_CUDA;
    int rc = CSG_OK;
    for (BatchClass& c : b->classes) {
        int best = 8;
        float best_t = 0.f;
        if ((rc = set_shape(b, c, csgrt::kViewsShapes[0])) != CSG_OK) break;
        for (int tw : kTileShapes) {
            float ms = 0.f;
            if ((rc = build_table(b, c, tw)) != CSG_OK) break;
            if ((rc = time_class(b, c, st, e0, e1, 3, &ms)) != CSG_OK) break;
            if (best_t == 0.f || ms < best_t) {
                best_t = ms;
                best = tw;
            }
        }
        if (rc != CSG_OK) break;
        if ((rc = build_table(b, c, best)) != CSG_OK) break;
        csgrt::ViewsShape best_shape = csgrt::kViewsShapes[0];
        for (int k = 1; k < 4 && rc == CSG_OK; ++k) {
            float ms = 0.f;
            if ((rc = set_shape(b, c, csgrt::kViewsShapes[k])) != CSG_OK) break;
            if ((rc = time_class(b, c, st, e0, e1, 3, &ms)) != CSG_OK) break;
            if (ms < best_t) {
                best_t = ms;
                best_shape = csgrt::kViewsShapes[k];
            }
        }
        if (rc != CSG_OK) break;
        if ((rc = set_shape(b, c, best_shape)) != CSG_OK) break;
        c.tuned_ms = best_t;
    }
    float whole = 0.f;
    if (rc == CSG_OK) rc = csg_batch_render(b, stream);  // capture and warm-up
    if (rc == CSG_OK) {
        cudaEventRecord(e0, st);
        rc = csg_batch_render(b, stream);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = CSG_E_CUDA;
        cudaEventElapsedTime(&whole, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != CSG_OK) return rc;
    if (best_tile_w) *best_tile_w = b->classes.empty() ? 8 : b->classes.front().tile_w;
    if (best_ms) *best_ms = whole;
    return CSG_OK;
}

int csg_batch_set_shape(csg_batch* b, int32_t warps_per_block, int32_t local_stacks)
{
    if (!b) return CSG_E_ARG;
    const csgrt::ViewsShape s{warps_per_block, local_stacks != 0};
    if ((local_stacks != 0 && local_stacks != 1) || !csgrt::valid_shape(s)) return CSG_E_ARG;
    for (BatchClass& c : b->classes) {
        const int rc = set_shape(b, c, s);
        if (rc != CSG_OK) return rc;
    }
    return CSG_OK;
}

int csg_batch_set_class(csg_batch* b, int32_t k, int32_t warp_tile_w, int32_t warps_per_block,
                        int32_t local_stacks)
{
    if (!b || k < 0 || k >= (int32_t)b->classes.size()) return CSG_E_ARG;
    if (warp_tile_w != 4 && warp_tile_w != 8 && warp_tile_w != 16 && warp_tile_w != 32) return CSG_E_ARG;
    const csgrt::ViewsShape s{warps_per_block, local_stacks != 0};
    if ((local_stacks != 0 && local_stacks != 1) || !csgrt::valid_shape(s)) return CSG_E_ARG;
    BatchClass& c = b->classes[k];
    int rc = build_table(b, c, warp_tile_w);
    if (rc == CSG_OK) rc = set_shape(b, c, s);
    return rc;
}

int csg_batch_get_class(const csg_batch* b, int32_t k, csg_batch_class_info* info)
{
    if (!b || !info || k < 0 || k >= (int32_t)b->classes.size()) return CSG_E_ARG;
    const BatchClass& c = b->classes[k];
    info->n_views = (int32_t)c.views.size();
    info->stack_class = c.stack_class;
    info->rolled = c.rolled ? 1 : 0;
    info->live_words = c.live_words;
    info->warp_tile_w = c.tile_w;
    info->warps_per_block = c.shape.warps;
    info->local_stacks = c.shape.local_stacks ? 1 : 0;
    info->grid = c.grid;
    info->n_items = c.launch.n_items;
    info->tuned_ms = c.tuned_ms;
    return CSG_OK;
}

int csg_batch_get_info(const csg_batch* b, csg_batch_info* info)
{
    if (!b || !info) return CSG_E_ARG;
    info->n_views = static_cast<int32_t>(b->src.size());
    int64_t items = 0;
    int grid = 0, sd = 4, rolled = 0;
    for (const BatchClass& c : b->classes) {
        items += c.launch.n_items;
        grid = std::max(grid, c.grid);
        sd = std::max(sd, c.stack_class);
        rolled |= c.rolled ? 1 : 0;
    }
    info->n_items = (int32_t)std::min<int64_t>(items, INT_MAX);
    info->warp_tile_w = b->classes.empty() ? 8 : b->classes.front().tile_w;
    info->stack_class = sd;
    info->rolled = rolled;
    info->grid = grid;
    info->device_bytes = b->bytes;
    info->n_classes = (int32_t)b->classes.size();
    info->warps_per_block = b->classes.empty() ? 4 : b->classes.front().shape.warps;
    info->local_stacks = (!b->classes.empty() && b->classes.front().shape.local_stacks) ? 1 : 0;
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
