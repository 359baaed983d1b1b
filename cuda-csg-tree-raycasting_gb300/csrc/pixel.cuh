// Per-pixel body shared by the single-view kernel (render_tiled.cuh) and the persistent
// view-table kernel (views_kernel.cuh): shared-memory layout of a block, and one pixel's
// ray generation, liveness pre-pass, traversal, details, shading and output planes.
#pragma once

#include "render.hpp"
#include "trace.cuh"

namespace csgrt {
namespace pix {

constexpr int kThreads = 128;  // 4 warps per block: the single-view kernel, the default view-table shape

// Shared memory of an nt-thread block: the per-ray primitive and time stacks (SD slots;
// none when the stacks are in local memory), the per-ray live masks (live_words words)
// with their restore records (one float per region of dev::kLiveRegionWords words) and
// one pre-pass scratch area per warp.
inline size_t smem_bytes(int sd, int live_words, int nt = kThreads, bool local_stacks = false)
{
    return (local_stacks ? 0 : (size_t)sd * nt * 12) + (size_t)live_words * nt * 4 +
           (size_t)dev::live_regions(live_words) * nt * 4 + (size_t)(nt / 32) * dev::kWarpScratch * 4;
}

struct BlockSmem {
    int* wstack;    // this warp's BVH stack
    uint32_t* live; // live-mask base (word k of thread t at live[k * nt + t], then the restore records)
    int nt;         // threads per block
};

template <int SD, int NT>
__device__ __forceinline__ dev::SmemStacks<SD> block_stacks(unsigned char* smem_raw)
{
    dev::SmemStacks<SD> st;
    st.nt = NT;
    st.tid = threadIdx.x;
    st.pt = reinterpret_cast<float*>(smem_raw);
    st.pb = reinterpret_cast<uint32_t*>(st.pt + SD * NT);
    st.tt = reinterpret_cast<float*>(st.pb + SD * NT);
    st.np = 0;
    st.ntm = 0;
    return st;
}

template <int SD>
__device__ __forceinline__ void init_stacks(dev::LocalStacks<SD>& st)
{
    st.np = 0;
    st.ntm = 0;
}

template <int SD, int NT, bool LOCAL>
__device__ __forceinline__ BlockSmem block_smem(unsigned char* smem_raw, int live_words_alloc)
{
    BlockSmem b;
    b.live = reinterpret_cast<uint32_t*>(smem_raw + (LOCAL ? 0 : (size_t)SD * NT * 12));
    b.wstack = reinterpret_cast<int*>(b.live + (size_t)(live_words_alloc + dev::live_regions(live_words_alloc)) * NT) +
               (threadIdx.x >> 5) * dev::kWarpScratch;
    b.nt = NT;
    return b;
}

using csgrt::ViewParams;

// Details, shading and the output planes of one finished ray.
template <bool CYL = true>
__device__ __forceinline__ void write_pixel(const ViewParams& p, unsigned long long* status, const dev::Ray& ray,
                                            const dev::Hit& h, bool capped, int x, int y)
{
    if (capped) atomicAdd(status, 1ull);
    const long long pix = (long long)y * p.w + x;
    const long long npix = (long long)p.w * p.h;
    // A hit always carries the index of a primitive it was computed from; the range check
    // only guards the loads below against a corrupted scene.
    const bool is_hit = (h.hit != dev::kMiss) && (uint32_t)h.idx < (uint32_t)p.scene.n_prims;
    float4 c;
    dev::V3 P = dev::mk(0.f, 0.f, 0.f), N = dev::mk(0.f, 0.f, 0.f);
    if (is_hit) {
        dev::hit_details<CYL>(ray, p.scene.geo, h, P, N);
        const float4 col = __ldg(&p.scene.color[h.idx]);
        c = dev::phong(p.cam.v, dev::mk(p.light[0], p.light[1], p.light[2]), P, N, col);
    } else {
        c = make_float4(0.08f, 0.08f, 0.11f, 1.0f);
    }
    if (p.out.rgba8) p.out.rgba8[pix] = dev::quantize_rgba8(c);
    if (p.out.rgba32f) p.out.rgba32f[pix] = c;
    if (p.out.t) p.out.t[pix] = is_hit ? h.t : __int_as_float(0x7f800000);
    if (p.out.prim) p.out.prim[pix] = is_hit ? h.idx : -1;
    if (p.out.normal) {
        p.out.normal[pix] = N.x;
        p.out.normal[npix + pix] = N.y;
        p.out.normal[2 * npix + pix] = N.z;
    }
}

// One pixel.  Must be called by all 32 lanes of a warp (the pre-pass walks the BVH
// warp-cooperatively); lanes with inside == false only follow the walk.
// FINE: the scene's fine live mask (single-view renders of large trees) instead of its own.
// SCU: the unrolled traversal with the operator short-circuit (no effect on rolled ones).
// CYL: the scene may hold cylinders (false: the cylinder code is left out).
template <int SD, bool ROLLED, bool FINE = false, bool SCU = false, bool CYL = true, class Stacks>
__device__ __forceinline__ void render_pixel(const ViewParams& p, unsigned long long* status, uint32_t iter_cap,
                                             int x, int y, bool inside, Stacks& st, const BlockSmem& bs,
                                             const uint16_t* tab, dev::RayFrame frame)
{
    typename std::conditional<FINE, dev::LiveMaskFine, dev::LiveMask>::type lm;
    lm.w = bs.live + threadIdx.x;
    lm.nt = bs.nt;
    lm.shift = FINE ? p.scene.fine_shift : p.scene.live_shift;
    lm.words = FINE ? p.scene.fine_words : p.scene.live_words;
    lm.sum = 0;
    const dev::Ray ray = dev::primary_ray(p.cam.v, inside ? x : 0, inside ? y : 0, (float)p.w, (float)p.h, frame);
    dev::live_prepass<ROLLED, CYL>(ray, inside, p.scene, lm, bs.wstack);
    if (!inside) return;
    // No live leaf: every leaf is a Miss at every tmin >= 0 (the pre-pass clears a bit only
    // for such a leaf), so every record the traversal could make or reload is a Miss, no table
    // cell loops on two Misses, and the ray ends as a Miss: the background, without a
    // traversal (in the 32-entry class too: whatever its stacks drop, they hold only Misses).
    if (lm.sum == 0) {
        write_pixel<CYL>(p, status, ray, dev::hit_default(), false, x, y);
        return;
    }
    bool capped = false;
    const dev::Hit h = dev::csg_traverse<SD, ROLLED, SCU, CYL>(p.scene, ray, st, tab, lm, iter_cap, &capped);
    write_pixel<CYL>(p, status, ray, h, capped, x, y);
}

__device__ __forceinline__ void load_table(uint16_t* tab)
{
    if (threadIdx.x < 27) tab[threadIdx.x] = dev::table_entry(threadIdx.x);
}

}  // namespace pix
}  // namespace csgrt
