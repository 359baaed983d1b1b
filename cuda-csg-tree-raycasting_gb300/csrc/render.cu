// Single-view rendering: RaycastKernel + LightningKernel of the reference
// (CSGRayCasting/Graphics/RayCasting/Kernels/RaycastingKernels.cu:3-111) fused into one
// launch of render_tiled (render_tiled.cuh; its plain form is instantiated here, its
// recording form in render_rec.cu), one thread per pixel, each warp a 4x8 pixel tile,
// shading in the traversal's epilogue; and the cost-ordered dispatch of large frames.
// Nothing passes through global memory between the two stages (the reference
// round-trips a 36-byte RayHit per pixel); the only HBM traffic is the output
// planes.  Each ray first finds the primitives it can hit at all (liveness pre-pass over
// a BVH of the leaves), then runs the reference's traversal, skipping subtrees with no
// live primitive left (in trees deeper than 15 operator levels, whose stacks can
// overflow, only where no push can be dropped: trace.cuh, kGuard).
#include <algorithm>
#include <atomic>
#include <cmath>

#include "render_tiled.cuh"

namespace csgrt {

using namespace tiled;

// The recording form is instantiated in render_rec.cu, the plain form here.
extern template cudaError_t tiled::launch_tiled<true>(const RenderParams& p, cudaStream_t stream);
template cudaError_t tiled::launch_tiled<false>(const RenderParams& p, cudaStream_t stream);

namespace {

// Cost-ordered dispatch (a tuning knob: the fewest tiles a frame needs for it; 0: off).  On
// the cheese frame a dozen blocks of 600-830 us, away from the projected centre, started
// 420-600 us into the launch behind the heavy disc's blocks and ran on alone at its end; no
// order by position starts them first.  So the kernel records every block's duration, and the
// next frame of the scene on the same grid (launch_render) starts its tiles longest first:
// classes of half an octave of the recorded cycles, each class in centre-out order, built by
// two small kernels before the render kernel.  A frame's first launch, and every launch on
// a stream that does not own the scene's state, keeps the centre-out order.
#ifndef CSG_DISPATCH_MIN_TILES
#define CSG_DISPATCH_MIN_TILES 32768
#endif
// The gate (tuning knobs): the dispatch stays on while the previous frame's longest block is
// at least CSG_DISPATCH_TAIL_PCT percent of the frame's work per block slot (the cheese frame
// keeps it on); below that it is off for CSG_DISPATCH_OFF_FRAMES frames, then probed again.
// The order kernels and the recording form cost a 4K frame whose rays all miss 12%.
#ifndef CSG_DISPATCH_TAIL_PCT
#define CSG_DISPATCH_TAIL_PCT 25
#endif
#ifndef CSG_DISPATCH_OFF_FRAMES
#define CSG_DISPATCH_OFF_FRAMES 32
#endif

constexpr int kOrderThreads = 256, kOrderWarps = kOrderThreads / 32;
constexpr int kCostClasses = 32;   // one per lane of a warp
constexpr int kOrderBlocksMax = 256;
constexpr int kCostKeyTop = 45;    // class 0: 3 * 2^22 cycles or more

// Class of a recorded duration, longest first: key 2 floor(log2 c) + the next bit of c.
__device__ __forceinline__ int cost_class(uint32_t c)
{
    const int l = 31 - __clz(c | 1u);
    const int key = 2 * l + (l > 0 ? (int)((c >> (l - 1)) & 1u) : 0);
    return min(kCostClasses - 1, max(0, kCostKeyTop - key));
}

// The tile at centre-out position k (rows by tile_row, columns left to right), as row << 16 |
// column (the dispatch is used only on grids under 65,536 tiles a side).
__device__ __forceinline__ uint32_t centre_out_tile(uint32_t k, int tiles_x, int tiles_y, int center_row)
{
    const uint32_t r = k / (uint32_t)tiles_x;
    return (uint32_t)tile_row((int)r, center_row, tiles_y) << 16 | (k - r * (uint32_t)tiles_x);
}

struct OrderParams {
    uint32_t* cost;     // read, then (clear) cleared for the next frame's recording
    uint32_t* counts;  // [blocks][kCostClasses]
    uint32_t* order;
    float* summary;     // null, or where block 0 writes {longest block, all blocks}
    uint32_t n, chunk;  // tiles; centre-out positions per block (a multiple of kOrderThreads)
    int32_t tiles_x, tiles_y, center_row;
    int32_t shift_x, shift_y;  // tiles the view moved since the recording: tile t costs what t - shift did
    int32_t clear;             // no shift: order_scatter clears each entry it reads
};

// The recorded entry that stands for tile rc (row << 16 | column) of this frame.
__device__ __forceinline__ uint32_t cost_source(uint32_t rc, const OrderParams& p)
{
    const int r = min(max((int)(rc >> 16) - p.shift_y, 0), p.tiles_y - 1);
    const int c = min(max((int)(rc & 0xffffu) - p.shift_x, 0), p.tiles_x - 1);
    return (uint32_t)r * (uint32_t)p.tiles_x + (uint32_t)c;
}

// Pass 1: each block counts the cost classes of its chunk of centre-out positions.
__global__ void __launch_bounds__(kOrderThreads) order_count(const OrderParams p)
{
    __shared__ uint32_t cnt[kCostClasses];
    if (threadIdx.x < kCostClasses) cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t k0 = min(p.n, blockIdx.x * p.chunk), k1 = min(p.n, k0 + p.chunk);
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += kOrderThreads)
        atomicAdd(&cnt[cost_class(__ldg(p.cost + cost_source(centre_out_tile(k, p.tiles_x, p.tiles_y, p.center_row), p)))],
                  1u);
    __syncthreads();
    if (threadIdx.x < kCostClasses) p.counts[blockIdx.x * kCostClasses + threadIdx.x] = cnt[threadIdx.x];
}

// Pass 2: order = the tiles by class, and within a class by centre-out position.  A tile's
// place: its class's start (the classes before it), the same class's tiles in earlier
// blocks, in earlier slabs of this block, in earlier warps of the slab, in earlier lanes.
__global__ void __launch_bounds__(kOrderThreads) order_scatter(const OrderParams p)
{
    __shared__ uint32_t part[2][kOrderWarps][kCostClasses];
    __shared__ uint32_t next[kCostClasses];
    __shared__ uint32_t wcnt[kOrderWarps][kCostClasses];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    {
        uint32_t tot = 0, before = 0;
        for (uint32_t g = (uint32_t)warp; g < gridDim.x; g += kOrderWarps) {
            const uint32_t v = __ldg(p.counts + g * kCostClasses + lane);
            tot += v;
            if (g < blockIdx.x) before += v;
        }
        part[0][warp][lane] = tot;
        part[1][warp][lane] = before;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t tot = 0, before = 0;
        for (int w = 0; w < kOrderWarps; ++w) {
            tot += part[0][w][lane];
            before += part[1][w][lane];
        }
        uint32_t incl = tot;  // classes 0..lane
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        next[lane] = incl - tot + before;
        if (p.summary && blockIdx.x == 0) {
            // lower bounds in cycles: class c holds durations from lo(c) up to the next class's
            const int key = kCostKeyTop - lane;
            const float lo = ldexpf((key & 1) ? 1.5f : 1.f, key >> 1);
            float work = (float)tot * lo;
            for (int o = 16; o > 0; o >>= 1) work += __shfl_xor_sync(0xffffffffu, work, o);
            const uint32_t nz = __ballot_sync(0xffffffffu, tot != 0u);
            const float longest = __shfl_sync(0xffffffffu, lo, nz ? __ffs((int)nz) - 1 : 0);
            if (lane == 0) {
                p.summary[0] = nz ? longest : 0.f;
                p.summary[1] = work;
            }
        }
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t k0 = min(p.n, blockIdx.x * p.chunk), k1 = min(p.n, k0 + p.chunk);
    for (uint32_t s = k0; s < k1; s += kOrderThreads) {  // the same trip count in every thread
        const uint32_t k = s + threadIdx.x;
        const bool in = k < k1;
        const uint32_t t = in ? centre_out_tile(k, p.tiles_x, p.tiles_y, p.center_row) : 0u;
        const uint32_t src = cost_source(t, p);
        const int cls = in ? cost_class(p.cost[src]) : -1;
        if (in && p.clear) p.cost[src] = 0u;  // src is t itself: this kernel's last read of the entry
        uint32_t rank = 0, mine = 0;
#pragma unroll
        for (int c = 0; c < kCostClasses; ++c) {
            const uint32_t bal = __ballot_sync(0xffffffffu, cls == c);
            if (cls == c) rank = __popc(bal & lt);
            if (lane == c) mine = __popc(bal);
        }
        wcnt[warp][lane] = mine;
        __syncthreads();
        if (in) {
            uint32_t pos = next[cls] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][cls];
            if (pos < p.n) p.order[pos] = t;  // always (the positions are a permutation of [0, n))
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t a = 0;
            for (int w = 0; w < kOrderWarps; ++w) a += wcnt[w][lane];
            next[lane] += a;
        }
        __syncthreads();
    }
}

// Blocks of the order kernels for n tiles, and each block's chunk of positions.
inline void order_grid(uint32_t n, uint32_t* blocks, uint32_t* chunk)
{
    uint32_t g = (n + kOrderThreads - 1) / kOrderThreads;
    if (g > (uint32_t)kOrderBlocksMax) g = kOrderBlocksMax;
    if (g == 0) g = 1;
    const uint32_t per = (n + g - 1) / g;
    *chunk = (per + kOrderThreads - 1) / kOrderThreads * kOrderThreads;
    *blocks = g;
}

__global__ void tan_half_fov_kernel(float fov, float* out) { *out = tanf(__fmul_rn(fov, 0.5f)); }

}  // namespace

namespace {
std::atomic<uint32_t> g_iter_cap{kIterCap};
}  // namespace

uint32_t iteration_cap() { return g_iter_cap.load(std::memory_order_relaxed); }
void set_iteration_cap(uint32_t cap) { g_iter_cap.store(cap, std::memory_order_relaxed); }

cudaError_t device_tan_half_fov(float fov, float* host_out)
{
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float));
    if (e != cudaSuccess) return e;
    tan_half_fov_kernel<<<1, 1>>>(fov, d);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(host_out, d, sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

namespace {

// Sets p.cost (and p.order when the previous frame of this grid recorded its costs) for a
// launch on `stream`, with d.mu held; leaves both null where the state is not this stream's.
cudaError_t prepare_dispatch(DispatchState& d, RenderParams& p, uint32_t tiles, const ProjectedCentre& centre,
                             cudaStream_t stream)
{
    if (stream == cudaStreamPerThread) return cudaSuccess;  // one handle, a stream per host thread
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        return cudaSuccess;
    }
    if (cs != cudaStreamCaptureStatusNone) return cudaSuccess;  // a graph would replay a stale order
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    if (!d.owned) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return e;
        d.owned = true;
        d.stream = stream;
        d.device = device;
        d.slots = sms * 6;
        void* h = nullptr;
        void* hd = nullptr;
        if (cudaHostAlloc(&h, 4 * sizeof(float), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(&hd, h, 0) != cudaSuccess ||
            cudaEventCreateWithFlags(&d.summary_ready, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (h) cudaFreeHost(h);
            d.summary_ready = nullptr;
            d.failed = true;
        } else {
            d.summary = static_cast<float*>(h);
            d.summary_dev = static_cast<float*>(hd);
        }
    } else if (d.stream != stream || d.device != device) {
        return cudaSuccess;
    }
    if (d.failed) return cudaSuccess;
    if (d.capacity < tiles) {
        if (d.cost) {
            // the old buffers may still be read by this stream's earlier launches
            e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) return e;
            for (uint32_t* b : {d.cost, d.order, d.counts}) cudaFree(b);
            d.cost = d.order = d.counts = nullptr;
            d.capacity = 0;
        }
        const size_t count_words = (size_t)kOrderBlocksMax * kCostClasses;
        const bool ok = cudaMalloc(&d.cost, tiles * sizeof(uint32_t)) == cudaSuccess &&
                        cudaMalloc(&d.order, tiles * sizeof(uint32_t)) == cudaSuccess &&
                        cudaMalloc(&d.counts, count_words * sizeof(uint32_t)) == cudaSuccess &&
                        cudaMemsetAsync(d.order, 0, tiles * sizeof(uint32_t), stream) == cudaSuccess &&
                        cudaMemsetAsync(d.counts, 0, count_words * sizeof(uint32_t), stream) == cudaSuccess;
        if (!ok) {  // no room: this scene renders in the centre-out order from now on
            cudaGetLastError();
            for (uint32_t* b : {d.cost, d.order, d.counts})
                if (b) cudaFree(b);
            d.cost = d.order = d.counts = nullptr;
            d.costs_valid = false;
            d.failed = true;
            return cudaSuccess;
        }
        d.capacity = tiles;
        d.costs_valid = false;
    }
    if (d.tiles_x != p.tiles_x || d.tiles_y != p.tiles_y || d.tw_log2 != p.tw_log2) {
        d.tiles_x = p.tiles_x;
        d.tiles_y = p.tiles_y;
        d.tw_log2 = p.tw_log2;
        d.costs_valid = false;
        d.off_frames = 0;
        d.summary_pending = false;  // a summary still in flight describes the old grid
    }
    if (d.off_frames > 0) {  // the gate is closed: plain frames, then a new recording
        --d.off_frames;
        d.costs_valid = false;
        return cudaSuccess;
    }
    if (d.summary_pending) {
        const cudaError_t q = cudaEventQuery(d.summary_ready);
        if (q == cudaSuccess) {
            d.summary_pending = false;
            const float longest = d.summary[0], work = d.summary[1];
            if (longest * (float)d.slots * 100.f < (float)CSG_DISPATCH_TAIL_PCT * work) {
                d.off_frames = CSG_DISPATCH_OFF_FRAMES - 1;
                d.costs_valid = false;
                return cudaSuccess;
            }
        } else if (q == cudaErrorNotReady) {
            if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();
        } else {
            return q;
        }
    }
    if (!d.costs_valid) {  // the render kernel records maxima: start from zero
        e = cudaMemsetAsync(d.cost, 0, tiles * sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
    } else {
        OrderParams op;
        op.cost = d.cost;
        op.counts = d.counts;
        op.order = d.order;
        op.summary = d.summary_pending ? nullptr : d.summary_dev;
        op.n = tiles;
        op.tiles_x = p.tiles_x;
        op.tiles_y = p.tiles_y;
        op.center_row = p.center_row;
        op.shift_x = op.shift_y = 0;
        if (centre.ok && d.rec_centre.ok) {  // follow the scene across the screen
            const float dx = std::round(centre.x - d.rec_centre.x), dy = std::round(centre.y - d.rec_centre.y);
            op.shift_x = (int32_t)std::max(std::min(dx, (float)(p.tiles_x - 1)), (float)(1 - p.tiles_x));
            op.shift_y = (int32_t)std::max(std::min(dy, (float)(p.tiles_y - 1)), (float)(1 - p.tiles_y));
        }
        op.clear = op.shift_x == 0 && op.shift_y == 0;
        uint32_t blocks = 0;
        order_grid(tiles, &blocks, &op.chunk);
        order_count<<<blocks, kOrderThreads, 0, stream>>>(op);
        order_scatter<<<blocks, kOrderThreads, 0, stream>>>(op);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (op.summary) {
            e = cudaEventRecord(d.summary_ready, stream);
            if (e != cudaSuccess) return e;
            d.summary_pending = true;
        }
        if (!op.clear) {  // read through the shift: cleared here instead
            e = cudaMemsetAsync(d.cost, 0, tiles * sizeof(uint32_t), stream);
            if (e != cudaSuccess) return e;
        }
        p.order = d.order;
    }
    d.costs_valid = false;  // until this launch has been issued
    d.rec_centre = centre;
    p.cost = d.cost;
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_render(const DeviceScene& scene, const float center[3], const Camera& cam, const float light[3],
                          int32_t w, int32_t h, const Planes& out,
                          unsigned long long* status, cudaStream_t stream, bool host_out, DispatchState* dispatch)
{
    RenderParams p;
    p.view.scene = scene;
    p.view.cam = cam;
    p.view.light[0] = light[0];
    p.view.light[1] = light[1];
    p.view.light[2] = light[2];
    p.view.w = w;
    p.view.h = h;
    p.view.out = out;
    p.status = status;
    p.iter_cap = iteration_cap();
    p.tw_log2 = log2_width(host_out ? CSG_TILED_HOST_WARP_W : CSG_TILED_WARP_W);
    const int kTileW = 2 << p.tw_log2, kTileH = 64 >> p.tw_log2;
    p.tiles_x = (w + kTileW - 1) / kTileW;
    p.tiles_y = (h + kTileH - 1) / kTileH;
    // the pixel of the scene's centre (Raycaster's ray generation inverted: nx = (2 u - 1)
    // (w / h) tan(fov / 2), ny = (1 - 2 v) tan(fov / 2), u = (x + 0.5) / (w - 1),
    // v = (y + 0.5) / (h - 1)): its row starts the centre-out order (the middle row if the
    // centre is not in front of the camera), and the cost-ordered dispatch follows it
    ProjectedCentre centre;
    p.center_row = 0;
    {
        const float* c = cam.v;
        const float vx = center[0] - c[0], vy = center[1] - c[1], vz = center[2] - c[2];
        const float z = vx * c[6] + vy * c[7] + vz * c[8];
        const float thf = std::tan(0.5f * c[5]);
        float row = 0.5f * (float)h;
        if (z > 0.f && thf > 0.f) {
            const float nx = (vx * c[9] + vy * c[10] + vz * c[11]) / z;
            const float ny = (vx * c[12] + vy * c[13] + vz * c[14]) / z;
            row = 0.5f * (1.f - ny / thf) * (float)(h - 1) - 0.5f;
            const float col = 0.5f * (1.f + nx / (thf * (float)w / (float)h)) * (float)(w - 1) - 0.5f;
            centre.ok = std::isfinite(col) && std::isfinite(row) && std::fabs(col) < 1e7f && std::fabs(row) < 1e7f;
            centre.x = col / (float)kTileW;
            centre.y = row / (float)kTileH;
        }
        if (CSG_TILED_CENTER_OUT) {
            if (!(row >= 0.f)) row = 0.f;  // also NaN
            if (row > (float)(h - 1)) row = (float)(h - 1);
            p.center_row = std::min((int)row / kTileH, p.tiles_y - 1);
        }
    }
    p.order = nullptr;
    p.cost = nullptr;
    const uint32_t tiles = (uint32_t)p.tiles_x * (uint32_t)p.tiles_y;
    std::unique_lock<std::mutex> lock;
    if (dispatch && CSG_DISPATCH_MIN_TILES > 0 && tiles >= (uint32_t)CSG_DISPATCH_MIN_TILES && p.tiles_x < 65536 &&
        p.tiles_y < 65536) {
        lock = std::unique_lock<std::mutex>(dispatch->mu);
        const cudaError_t e = prepare_dispatch(*dispatch, p, tiles, centre, stream);
        if (e != cudaSuccess) return e;
    }
    const cudaError_t e = p.cost ? launch_tiled<true>(p, stream) : launch_tiled<false>(p, stream);
    if (p.cost) dispatch->costs_valid = e == cudaSuccess;
    return e;
}

cudaError_t release_dispatch(DispatchState& d)
{
    std::lock_guard<std::mutex> lock(d.mu);
    cudaError_t e = cudaSuccess;
    if (d.owned) {
        int prev = 0;
        cudaGetDevice(&prev);
        if (prev != d.device) cudaSetDevice(d.device);
        for (uint32_t* b : {d.cost, d.order, d.counts}) {
            const cudaError_t f = b ? cudaFree(b) : cudaSuccess;
            if (e == cudaSuccess) e = f;
        }
        if (d.summary_ready) {
            // the last summary write may still be in flight
            cudaError_t f = cudaEventSynchronize(d.summary_ready);
            if (e == cudaSuccess) e = f;
            f = cudaEventDestroy(d.summary_ready);
            if (e == cudaSuccess) e = f;
        }
        if (d.summary) {
            const cudaError_t f = cudaFreeHost(d.summary);
            if (e == cudaSuccess) e = f;
        }
        if (prev != d.device) cudaSetDevice(prev);
    }
    d.cost = d.order = d.counts = nullptr;
    d.summary = d.summary_dev = nullptr;
    d.summary_ready = nullptr;
    d.failed = false;
    d.summary_pending = false;
    d.owned = false;
    d.capacity = 0;
    d.costs_valid = false;
    return e;
}

}  // namespace csgrt
