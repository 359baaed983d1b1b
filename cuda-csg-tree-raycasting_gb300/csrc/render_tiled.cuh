// The single-view render kernel (render_tiled) and its launch by scene variant, shared by
// the two translation units that instantiate it, compiled in parallel: render.cu (the plain
// form) and render_rec.cu (the recording form of the cost-ordered dispatch).  Reference:
// RaycastKernel + LightningKernel (CSGRayCasting/Graphics/RayCasting/Kernels/
// RaycastingKernels.cu:3-111) fused into one launch.
#pragma once

#include <atomic>
#include <cstdint>
#include <type_traits>

#include "pixel.cuh"

namespace csgrt {
namespace tiled {

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
        if (lane == 0 && t_tile < (unsigned)p.tiles_x * (unsigned)p.tiles_y) {  // always (order holds tiles)
            const long long d = clock64() - t_begin;
            atomicMax(p.cost + t_tile, d < 0 ? 0u : d > 0xffffffffLL ? 0xffffffffu : (uint32_t)d);
        }
    }
}

template <bool REC, int SD, bool ROLLED, bool FINE, bool LOCAL, bool SCU = false, bool CYL = true>
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
        const auto kernel = render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, REC>;
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pix::smem_bytes(SD, FINE ? kFineWordsMax : kLiveWordsMax, kThreads, LOCAL));
        if (e == cudaSuccess && CSG_TILED_CARVEOUT >= 0)
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, CSG_TILED_CARVEOUT);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit, std::memory_order_release);
    }
    const unsigned grid = (unsigned)p.tiles_x * (unsigned)p.tiles_y;
    render_tiled<SD, ROLLED, FINE, LOCAL, SCU, CYL, REC><<<grid, kThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

template <bool REC, int SD>
cudaError_t launch_sd(const RenderParams& p, cudaStream_t stream)
{
    if (!p.view.scene.rolled) {
        const bool sc = CSG_UNROLLED_SHORT_CIRCUIT && p.view.scene.short_circuit;
        if (p.view.scene.cylinders)
            return sc ? launch_variant<REC, SD, false, false, false, true, true>(p, stream)
                      : launch_variant<REC, SD, false, false, false, false, true>(p, stream);
        return sc ? launch_variant<REC, SD, false, false, false, true, false>(p, stream)
                  : launch_variant<REC, SD, false, false, false, false, false>(p, stream);
    }
    if (p.view.scene.fine) return launch_variant<REC, SD, true, true, false>(p, stream);
    const bool local = (CSG_TILED_LOCAL_WORDS >= 0 && p.view.scene.live_words >= CSG_TILED_LOCAL_WORDS) ||
                       (CSG_DEEP_LOCAL_STACKS && SD >= 32);
    if (!p.view.scene.cylinders)
        return local ? launch_variant<REC, SD, true, false, true, false, false>(p, stream)
                     : launch_variant<REC, SD, true, false, false, false, false>(p, stream);
    return local ? launch_variant<REC, SD, true, false, true>(p, stream) : launch_variant<REC, SD, true, false, false>(p, stream);
}

// Launches the scene's kernel variant in the plain form (REC = false, instantiated in
// render.cu) or the recording form (REC = true, in render_rec.cu).
template <bool REC>
cudaError_t launch_tiled(const RenderParams& p, cudaStream_t stream)
{
    switch (p.view.scene.stack_class) {
        case 4: return launch_sd<REC, 4>(p, stream);
        case 8: return launch_sd<REC, 8>(p, stream);
        case 12: return launch_sd<REC, 12>(p, stream);
        case 16: return launch_sd<REC, 16>(p, stream);
        default: return launch_sd<REC, 32>(p, stream);
    }
}

}  // namespace tiled
}  // namespace csgrt
