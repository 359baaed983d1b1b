// Single-view render kernel: RaycastKernel + LightningKernel of the reference
// (CSGRayCasting/Graphics/RayCasting/Kernels/RaycastingKernels.cu:3-111) fused into one
// launch, one thread per pixel, each warp an 8x4 pixel tile, shading in the traversal's
// epilogue.  Nothing passes through global memory between the two stages (the
// reference round-trips a 36-byte RayHit per pixel); the only HBM traffic is the output
// planes.  Each ray first finds the primitives it can hit at all (liveness pre-pass over
// a BVH of the leaves), then runs the reference's traversal, skipping subtrees with no
// live primitive left.
#include "render.hpp"
#include "trace.cuh"

namespace csgrt {
namespace {

constexpr int kThreads = 128;  // 4 warps
constexpr int kTileW = 16, kTileH = 8;

struct RenderParams {
    DeviceScene scene;
    Camera cam;
    float light[3];
    int32_t w, h;
    Planes out;
    unsigned long long* status;
    uint32_t iter_cap;
};

// Details, shading and the output planes of one finished ray.
__device__ __forceinline__ void write_pixel(const RenderParams& p, const dev::Ray& ray, const dev::Hit& h,
                                            bool capped, int x, int y)
{
    if (capped) atomicAdd(p.status, 1ull);
    const long long pix = (long long)y * p.w + x;
    const long long npix = (long long)p.w * p.h;
    // A hit always carries the index of a primitive it was computed from; the range check
    // only guards the loads below against a corrupted scene.
    const bool is_hit = (h.hit != dev::kMiss) && (uint32_t)h.idx < (uint32_t)p.scene.n_prims;
    float4 c;
    dev::V3 P = dev::mk(0.f, 0.f, 0.f), N = dev::mk(0.f, 0.f, 0.f);
    if (is_hit) {
        dev::hit_details(ray, p.scene.geo, h, P, N);
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

// Shared memory of a block: the per-ray primitive and time stacks (SD slots), the per-ray
// live masks (scene.live_words words) and one BVH stack per warp.
template <int SD>
__host__ __device__ constexpr size_t stack_bytes()
{
    return (size_t)SD * kThreads * 12;
}
inline size_t smem_bytes(int sd, int live_words)
{
    return (size_t)sd * kThreads * 12 + (size_t)live_words * kThreads * 4 +
           (size_t)(kThreads / 32) * dev::kWarpStack * 4;
}

// Minimum resident blocks per SM asked of the register allocator for the rolled variant
// (a tuning knob; the unrolled variant fits in 72 registers on its own).
#ifndef CSG_ROLLED_MIN_BLOCKS
#define CSG_ROLLED_MIN_BLOCKS 1
#endif
template <int SD, bool ROLLED>
__global__ void __launch_bounds__(kThreads, ROLLED ? CSG_ROLLED_MIN_BLOCKS : 1) render_tiled(const RenderParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint16_t tab[27];
    if (threadIdx.x < 27) tab[threadIdx.x] = dev::table_entry(threadIdx.x);
    const int tid = threadIdx.x;
    dev::SmemStacks<SD> st;
    st.nt = kThreads;
    st.tid = tid;
    st.pt = reinterpret_cast<float*>(smem_raw);
    st.pb = reinterpret_cast<uint32_t*>(st.pt + SD * kThreads);
    st.tt = reinterpret_cast<float*>(st.pb + SD * kThreads);
    st.np = 0;
    st.ntm = 0;
    uint32_t* live_base = reinterpret_cast<uint32_t*>(smem_raw + stack_bytes<SD>());
    int* wstacks = reinterpret_cast<int*>(live_base + (size_t)p.scene.live_words * kThreads);
    dev::LiveMask lm;
    lm.w = live_base + tid;
    lm.nt = kThreads;
    lm.shift = p.scene.live_shift;
    lm.words = p.scene.live_words;
    lm.sum = 0;

    const int warp = tid >> 5, lane = tid & 31;
    const int x = blockIdx.x * kTileW + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * kTileH + (warp >> 1) * 4 + (lane >> 3);
    const bool inside = x < p.w && y < p.h;
    __syncthreads();
    const dev::Ray ray = dev::primary_ray(p.cam.v, inside ? x : 0, inside ? y : 0, (float)p.w, (float)p.h);
    // every lane of the warp takes part in the pre-pass walk; lanes outside the image
    // only follow it
    dev::live_prepass<ROLLED>(ray, inside, p.scene, lm, wstacks + warp * dev::kWarpStack);
    if (!inside) return;
    bool capped = false;
    const dev::Hit h = dev::csg_traverse<SD, ROLLED>(p.scene, ray, st, tab, lm, p.iter_cap, &capped);
    write_pixel(p, ray, h, capped, x, y);
}

template <int SD, bool ROLLED>
cudaError_t launch_variant(const RenderParams& p, cudaStream_t stream)
{
    const size_t smem = smem_bytes(SD, p.scene.live_words);
    // Above the default 48 KiB per block the kernel needs the opt-in; set it once for the
    // largest layout any scene can ask for (kLiveWordsMax live words).
    static bool attr_set = false;
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(render_tiled<SD, ROLLED>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem_bytes(SD, kLiveWordsMax));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const dim3 grid((p.w + kTileW - 1) / kTileW, (p.h + kTileH - 1) / kTileH);
    render_tiled<SD, ROLLED><<<grid, kThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

template <int SD>
cudaError_t launch_sd(const RenderParams& p, cudaStream_t stream)
{
    return p.scene.rolled ? launch_variant<SD, true>(p, stream) : launch_variant<SD, false>(p, stream);
}

__global__ void tan_half_fov_kernel(float fov, float* out) { *out = tanf(__fdiv_rn(fov, 2.0f)); }

}  // namespace

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

cudaError_t launch_render(const DeviceScene& scene, const Camera& cam, const float light[3],
                          int32_t w, int32_t h, const Planes& out,
                          unsigned long long* status, cudaStream_t stream)
{
    RenderParams p;
    p.scene = scene;
    p.cam = cam;
    p.light[0] = light[0];
    p.light[1] = light[1];
    p.light[2] = light[2];
    p.w = w;
    p.h = h;
    p.out = out;
    p.status = status;
    p.iter_cap = kIterCap;
    switch (scene.stack_class) {
        case 4: return launch_sd<4>(p, stream);
        case 8: return launch_sd<8>(p, stream);
        case 12: return launch_sd<12>(p, stream);
        case 16: return launch_sd<16>(p, stream);
        default: return launch_sd<32>(p, stream);
    }
}

}  // namespace csgrt
