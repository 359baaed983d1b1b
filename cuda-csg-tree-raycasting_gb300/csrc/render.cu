// Single-view render kernel: RaycastKernel + LightningKernel of the reference
// (CSGRayCasting/Graphics/RayCasting/Kernels/RaycastingKernels.cu:3-111) fused into one
// launch, one thread per pixel, each warp a 4x8 pixel tile, shading in the traversal's
// epilogue.  Nothing passes through global memory between the two stages (the
// reference round-trips a 36-byte RayHit per pixel); the only HBM traffic is the output
// planes.  Each ray first finds the primitives it can hit at all (liveness pre-pass over
// a BVH of the leaves), then runs the reference's traversal, skipping subtrees with no
// live primitive left (in trees deeper than 15 operator levels, whose stacks can
// overflow, only where no push can be dropped: trace.cuh, kGuard).
#include <algorithm>
#include <atomic>
#include <cmath>

#include "pixel.cuh"

namespace csgrt {
namespace {

using pix::kThreads;
// Warp tile (tuning knobs, chosen per launch): W x (32 / W) pixels, W = CSG_TILED_WARP_W for
// frames written to device memory and CSG_TILED_HOST_WARP_W for frames the kernel stores
// into page-locked host memory; a block's four warps form a 2 x 2 arrangement of warp tiles.
// Device frames: 4 x 8 (it was 8 x 4): with the cone pre-pass and the empty-mask skip the cheese
// frame 5% faster and the batch's trees as single views 2-8%, the README tree 2%; 16 x 2 was 3-8%
// slower on the small frames.  Host frames: a warp's row of W pixels is one store of 4W bytes
// over the host link, and 4-pixel rows took the cheese frame's end-to-end rate down 3%.
#ifndef CSG_TILED_WARP_W
#define CSG_TILED_WARP_W 4
#endif
#ifndef CSG_TILED_HOST_WARP_W
#define CSG_TILED_HOST_WARP_W 8
#endif
static_assert(CSG_TILED_WARP_W == 4 || CSG_TILED_WARP_W == 8 || CSG_TILED_WARP_W == 16, "warp tile width");
static_assert(CSG_TILED_HOST_WARP_W == 4 || CSG_TILED_HOST_WARP_W == 8 || CSG_TILED_HOST_WARP_W == 16,
              "warp tile width");
constexpr int log2_width(int w) { return w == 4 ? 2 : w == 8 ? 3 : 4; }

struct RenderParams {
    pix::ViewParams view;
    int32_t tiles_x, tiles_y;  // block tiles of the view
    int32_t tw_log2;           // warp tile: 2^tw_log2 x 2^(5 - tw_log2) pixels
    int32_t center_row;        // block row that starts first (see tile_row)
    unsigned long long* status;
    uint32_t iter_cap;
    const uint32_t* order;     // null: centre-out rows; else block k renders tile order[k] (row << 16 | column)
    uint32_t* cost;            // null, or each block's duration in SM cycles (per tile, row-major)
};

// Minimum resident blocks per SM asked of the register allocator, per variant (tuning
// knobs).  Six 128-thread blocks cap the kernel at 80 registers, with no spills; measured
// 3-6% faster than the unconstrained 83-86 registers (five blocks) on the cheese and
// random-tree frames, 0-4% slower on trees whose live masks already limit residency to
// five blocks by shared memory.
#ifndef CSG_ROLLED_MIN_BLOCKS
#define CSG_ROLLED_MIN_BLOCKS 6
#endif
#ifndef CSG_UNROLLED_MIN_BLOCKS
#define CSG_UNROLLED_MIN_BLOCKS 6
#endif
// Rolled variants with local-memory stacks and no cylinder code (the cheese frame's) fit in
// 72 registers, seven blocks per SM, unconstrained; the cap keeps the recording form of the
// kernel (REC below) there too: at 78 registers and six blocks it was 6% slower.
#ifndef CSG_ROLLED_LOCAL_NOCYL_MIN_BLOCKS
#define CSG_ROLLED_LOCAL_NOCYL_MIN_BLOCKS 7
#endif
template <bool ROLLED, bool LOCAL, bool CYL>
constexpr int min_blocks()
{
    return !ROLLED ? CSG_UNROLLED_MIN_BLOCKS : (LOCAL && !CYL) ? CSG_ROLLED_LOCAL_NOCYL_MIN_BLOCKS : CSG_ROLLED_MIN_BLOCKS;
}
// Placement of the per-ray primitive and time stacks (a tuning knob): rolled scenes whose
// live mask takes at least CSG_TILED_LOCAL_WORDS words keep the stacks in per-thread local
// memory (cached in L1), which leaves their blocks' shared memory to the masks; the others
// keep them in block shared memory (-1: always shared memory).  Measured with the operator
// short-circuit: local stacks are 3-8% faster on trees with 27-32 mask words (1,700-4,000
// leaves); after the cone pre-pass and the empty-mask skip also 3% on the cheese frame (17
// words) and 4-6% on batch trees of 650-700 leaves, so the threshold went from 24 words to
// 16 (4 words: up to 4% slower on trees of ~240 leaves).
#ifndef CSG_TILED_LOCAL_WORDS
#define CSG_TILED_LOCAL_WORDS 16
#endif
// The 32-entry stack class (trees deeper than 15 operator levels) keeps its stacks in local
// memory (a tuning knob; 0: shared memory, 48 KiB per block, four resident blocks per SM).
#ifndef CSG_DEEP_LOCAL_STACKS
#define CSG_DEEP_LOCAL_STACKS 1
#endif
// Preferred shared-memory carveout in percent of the maximum (a tuning knob; -1 leaves
// the choice to the driver, which sizes shared memory for the most resident blocks).
// Before the operator short-circuit, 80% (five blocks and a larger L1 for the largest live
// masks) was 5% faster on the heaviest batch view; with it, the driver's choice is 3% faster
// over the batch's 35 largest trees and 5% over its 1,024 views rendered one by one.
#ifndef CSG_TILED_CARVEOUT
#define CSG_TILED_CARVEOUT -1
#endif

// The unrolled variant with the operator short-circuit for scenes that have it (a tuning
// knob; 0: unrolled scenes traverse without it).
#ifndef CSG_UNROLLED_SHORT_CIRCUIT
#define CSG_UNROLLED_SHORT_CIRCUIT 1
#endif

// Block dispatch order (a tuning knob; 0: row by row from the top).  Blocks start in launch
// order, and the slowest warps of a frame, the ones whose rays cross the most primitives,
// lie near the object's centre on screen; started late, they ran on alone after the rest
// of the frame was done (the heaviest batched view's SMs were busy for 40% of its
// launch).  So block rows go out from the row of the projected centre of the scene's
// box: row c, then c - 1, c + 1, c - 2, ... (`tile_row`).  Each block's work is unchanged.
#ifndef CSG_TILED_CENTER_OUT
#define CSG_TILED_CENTER_OUT 1
#endif

// The k-th block row to dispatch: c, c - 1, c + 1, c - 2, c + 2, ... within [0, n).
__device__ __forceinline__ int tile_row(int k, int c, int n)
{
    const int m = min(c, n - 1 - c);  // rows on both sides of c
    if (k <= 2 * m) return (k & 1) ? c - ((k + 1) >> 1) : c + (k >> 1);
    return (c - m == 0) ? c + m + (k - 2 * m) : c - m - (k - 2 * m);
}

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
// at least CSG_DISPATCH_TAIL_PCT percent of the frame's work per block slot (the cheese frame:
// about 85%); below that it is off for CSG_DISPATCH_OFF_FRAMES frames, then probed again.
// Recording alone costs the frames that have no such blocks up to 20% (every ray missing).
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
__device__ __forceinline__ uint32_t tile_index(uint32_t rc, int tiles_x)
{
    return (rc >> 16) * (uint32_t)tiles_x + (rc & 0xffffu);
}

struct OrderParams {
    uint32_t* cost;     // read, then cleared for the next frame's recording
    uint32_t* counts;  // [blocks][kCostClasses]
    uint32_t* order;
    float* summary;     // null, or where block 0 writes {longest block, all blocks}
    uint32_t n, chunk;  // tiles; centre-out positions per block (a multiple of kOrderThreads)
    int32_t tiles_x, tiles_y, center_row;
};

// Pass 1: each block counts the cost classes of its chunk of centre-out positions.
__global__ void __launch_bounds__(kOrderThreads) order_count(const OrderParams p)
{
    __shared__ uint32_t cnt[kCostClasses];
    if (threadIdx.x < kCostClasses) cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t k0 = min(p.n, blockIdx.x * p.chunk), k1 = min(p.n, k0 + p.chunk);
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += kOrderThreads)
        atomicAdd(&cnt[cost_class(__ldg(p.cost + tile_index(centre_out_tile(k, p.tiles_x, p.tiles_y, p.center_row),
                                                            p.tiles_x)))],
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
        const uint32_t ti = tile_index(t, p.tiles_x);
        const int cls = in ? cost_class(p.cost[ti]) : -1;
        if (in) p.cost[ti] = 0u;  // this kernel's last read of the entry
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
            p.order[pos] = t;
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

// FINE: the scene's fine live mask (scenes with scene.fine set; rolled variants only).
// LOCAL: the per-ray stacks in local memory (rolled scenes with large live masks).
// SCU: the operator short-circuit in the unrolled variant (scenes with short_circuit set).
// CYL: the cylinder code (false only for unrolled scenes without cylinders, whose kernel is
// then smaller: fewer instruction-cache misses).
// REC: the cost-ordered dispatch's form: each block renders the tile p.order names (when set)
// and records its duration in p.cost.  Launches without it run the plain form, which has no
// code after the pixel's own.
template <int SD, bool ROLLED, bool FINE, bool LOCAL, bool SCU, bool CYL, bool REC>
__global__ void __launch_bounds__(kThreads, (min_blocks<ROLLED, LOCAL, CYL>()))
    render_tiled(const RenderParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint16_t tab[27];
    __shared__ dev::RayFrame frame;  // the view's ray-generation factors, computed once per block
    __shared__ long long t_begin;    // REC: the block's start (SM cycles)
    __shared__ uint32_t t_tile;      // REC: and its tile (row-major index)
    uint32_t rc = 0;                 // REC with an order: the tile as row << 16 | column
    if constexpr (REC) {
        if (p.order) rc = __ldg(p.order + blockIdx.x);
    }
    pix::load_table(tab);
    if (threadIdx.x == 32) frame = dev::ray_frame(p.view.cam.v, (float)p.view.w, (float)p.view.h);
    typename std::conditional<LOCAL, dev::LocalStacks<SD>, dev::SmemStacks<SD>>::type st;
    if constexpr (LOCAL) pix::init_stacks(st);
    else st = pix::block_stacks<SD, kThreads>(smem_raw);
    const pix::BlockSmem bs =
        pix::block_smem<SD, kThreads, LOCAL>(smem_raw, FINE ? p.view.scene.fine_words : p.view.scene.live_words);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int bx, by;
    if (REC && p.order) {
        by = (int)(rc >> 16);
        bx = (int)(rc & 0xffffu);
    } else {
        bx = (int)(blockIdx.x % (unsigned)p.tiles_x);
        by = tile_row((int)(blockIdx.x / (unsigned)p.tiles_x), p.center_row, p.tiles_y);
    }
    if (REC && threadIdx.x == 0) {
        t_begin = clock64();
        t_tile = (unsigned)by * (unsigned)p.tiles_x + (unsigned)bx;
    }
    const int ww = 1 << p.tw_log2, wh = 32 >> p.tw_log2;
    const int x = bx * 2 * ww + (warp & 1) * ww + (lane & (ww - 1));
    const int y = by * 2 * wh + (warp >> 1) * wh + (lane >> p.tw_log2);
    __syncthreads();
    pix::render_pixel<SD, ROLLED, FINE, SCU, CYL>(p.view, p.status, p.iter_cap, x, y, x < p.view.w && y < p.view.h, st,
                                             bs, tab, frame);
    if constexpr (REC) {
        // the block's duration is its last warp's end: no block barrier here, which would
        // hold every finished warp's registers until the block's slowest warp is done
        // (6.5% slower on the cheese frame)
        __syncwarp();
        if (lane == 0) {
            const long long d = clock64() - t_begin;
            atomicMax(p.cost + t_tile, d < 0 ? 0u : d > 0xffffffffLL ? 0xffffffffu : (uint32_t)d);
        }
    }
}

template <int SD, bool ROLLED, bool FINE, bool LOCAL, bool SCU = false, bool CYL = true>
cudaError_t launch_variant(const RenderParams& p, cudaStream_t stream)
{
    const int words = FINE ? p.view.scene.fine_words : p.view.scene.live_words;
    const size_t smem = pix::smem_bytes(SD, words, kThreads, LOCAL);
    // Above the default 48 KiB per block the kernel needs the opt-in; set it once per device
    // for the largest layout any scene can ask for (kLiveWordsMax live words), with the
    // carveout preference.
    static std::atomic<unsigned long long> attr_set{0};  // bit d: done on device d
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = device < 64 ? 1ull << device : 0ull;
    if (!(attr_set.load(std::memory_order_acquire) & bit) || !bit) {
        for (const auto kernel : {render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, false>,
                                  render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, true>}) {
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pix::smem_bytes(SD, FINE ? kFineWordsMax : kLiveWordsMax, kThreads, LOCAL));
            if (e == cudaSuccess && CSG_TILED_CARVEOUT >= 0)
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, CSG_TILED_CARVEOUT);
            if (e != cudaSuccess) return e;
        }
        attr_set.fetch_or(bit, std::memory_order_release);
    }
    const unsigned grid = (unsigned)p.tiles_x * (unsigned)p.tiles_y;
    if (p.cost)
        render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, true><<<grid, kThreads, smem, stream>>>(p);
    else
        render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, false><<<grid, kThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

template <int SD>
cudaError_t launch_sd(const RenderParams& p, cudaStream_t stream)
{
    if (!p.view.scene.rolled) {
        const bool sc = CSG_UNROLLED_SHORT_CIRCUIT && p.view.scene.short_circuit;
        if (p.view.scene.cylinders)
            return sc ? launch_variant<SD, false, false, false, true, true>(p, stream)
                      : launch_variant<SD, false, false, false, false, true>(p, stream);
        return sc ? launch_variant<SD, false, false, false, true, false>(p, stream)
                  : launch_variant<SD, false, false, false, false, false>(p, stream);
    }
    if (p.view.scene.fine) return launch_variant<SD, true, true, false>(p, stream);
    const bool local = (CSG_TILED_LOCAL_WORDS >= 0 && p.view.scene.live_words >= CSG_TILED_LOCAL_WORDS) ||
                       (CSG_DEEP_LOCAL_STACKS && SD >= 32);
    if (!p.view.scene.cylinders)
        return local ? launch_variant<SD, true, false, true, false, false>(p, stream)
                     : launch_variant<SD, true, false, false, false, false>(p, stream);
    return local ? launch_variant<SD, true, false, true>(p, stream) : launch_variant<SD, true, false, false>(p, stream);
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
cudaError_t prepare_dispatch(DispatchState& d, RenderParams& p, uint32_t tiles, cudaStream_t stream)
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
        const bool ok = cudaMalloc(&d.cost, tiles * sizeof(uint32_t)) == cudaSuccess &&
                        cudaMalloc(&d.order, tiles * sizeof(uint32_t)) == cudaSuccess &&
                        cudaMalloc(&d.counts, kOrderBlocksMax * kCostClasses * sizeof(uint32_t)) == cudaSuccess;
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
        p.order = d.order;
    }
    d.costs_valid = false;  // until this launch has been issued
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
    p.center_row = 0;
    if (CSG_TILED_CENTER_OUT) {
        // the pixel row of the scene's centre (Raycaster's ray generation inverted:
        // ny = (1 - 2 v) tan(fov / 2), v = (y + 0.5) / (h - 1)); the middle row if it is not
        // in front of the camera
        const float* c = cam.v;
        const float vx = center[0] - c[0], vy = center[1] - c[1], vz = center[2] - c[2];
        const float z = vx * c[6] + vy * c[7] + vz * c[8];
        const float thf = std::tan(0.5f * c[5]);
        float row = 0.5f * (float)h;
        if (z > 0.f && thf > 0.f) {
            const float ny = (vx * c[12] + vy * c[13] + vz * c[14]) / z;
            row = 0.5f * (1.f - ny / thf) * (float)(h - 1) - 0.5f;
        }
        if (!(row >= 0.f)) row = 0.f;  // also NaN
        if (row > (float)(h - 1)) row = (float)(h - 1);
        p.center_row = std::min((int)row / kTileH, p.tiles_y - 1);
    }
    p.order = nullptr;
    p.cost = nullptr;
    const uint32_t tiles = (uint32_t)p.tiles_x * (uint32_t)p.tiles_y;
    std::unique_lock<std::mutex> lock;
    if (dispatch && CSG_DISPATCH_MIN_TILES > 0 && tiles >= (uint32_t)CSG_DISPATCH_MIN_TILES && p.tiles_x < 65536 &&
        p.tiles_y < 65536) {
        lock = std::unique_lock<std::mutex>(dispatch->mu);
        const cudaError_t e = prepare_dispatch(*dispatch, p, tiles, stream);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e;
    switch (scene.stack_class) {
        case 4: e = launch_sd<4>(p, stream); break;
        case 8: e = launch_sd<8>(p, stream); break;
        case 12: e = launch_sd<12>(p, stream); break;
        case 16: e = launch_sd<16>(p, stream); break;
        default: e = launch_sd<32>(p, stream); break;
    }
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
