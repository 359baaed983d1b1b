/* Runs the reference's own CUDA kernels (RaycastKernel + LightningKernel, compiled by
 * oracle/build_ref.py into oracle/_ref/ref_kernels.cubin) on the GPU, exactly as
 * Raycaster::Raycast launches them (Raycaster.cu:23-34): 8x4 blocks, the legacy default
 * stream, a device synchronisation after each kernel.
 *
 * TEST INFRASTRUCTURE ONLY: used by GPU parity tests (bit-exact comparison against the
 * reference kernel) and by bench.py to time the reference kernel beside the engine.
 * Uses the CUDA driver API on the primary context, so it shares the process's context
 * with the CUDA runtime.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static CUmodule g_mod;
static CUfunction g_ray, g_light;
static int g_ready;
static char g_err[256];

#define CK(x)                                                                      \
    do {                                                                           \
        CUresult r_ = (x);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                  \
            const char* s_ = 0;                                                    \
            cuGetErrorString(r_, &s_);                                             \
            snprintf(g_err, sizeof(g_err), "%s: %s", #x, s_ ? s_ : "?");          \
            rc = (int)r_;                                                          \
            goto done;                                                             \
        }                                                                          \
    } while (0)

const char* refcu_error(void) { return g_err; }

/* Names as nvcc mangles RaycastingKernels.cuh:39 and :42. */
int refcu_init(const char* cubin_path)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx;
    if (g_ready) return 0;
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CK(cuModuleLoad(&g_mod, cubin_path));
    CK(cuModuleGetFunction(&g_ray, g_mod, "_Z13RaycastKernel6Camera11CudaCSGTreeP6RayHitff"));
    CK(cuModuleGetFunction(&g_light, g_mod, "_Z15LightningKernel6CameraP6RayHitP9PrimitiveP6float46float3ff"));
    g_ready = 1;
done:
    return rc;
}

/* Kernel argument images with the reference's layouts. */
typedef struct { float v[15]; } ref_camera_t;                     /* Camera, 60 B */
typedef struct { CUdeviceptr nodes, prims; } ref_tree_t;          /* CudaCSGTree, 16 B */
typedef struct { float x, y, z; } ref_float3_t;

/* Renders one frame.  hits36 (w*h*36 bytes, the reference RayHit array) and rgba
 * (w*h float4) are host buffers; either may be NULL.  When reps > 0 the frame is then
 * launched `reps` more times and the mean device times are returned: ms_ray and
 * ms_light per kernel, ms_frame for both launches with the reference's synchronisation
 * in between (events on the default stream). */
int refcu_render(const void* nodes44, int n_nodes, const void* prims48, int n_prims,
                 const float cam[15], const float light[3], int w, int h,
                 void* hits36, float* rgba, int reps,
                 float* ms_ray, float* ms_light, float* ms_frame)
{
    int rc = 0;
    CUdeviceptr d_nodes = 0, d_prims = 0, d_hits = 0, d_out = 0;
    CUevent e0 = 0, e1 = 0, e2 = 0;
    if (!g_ready) { snprintf(g_err, sizeof(g_err), "refcu_init not called"); return -1; }
    const size_t npix = (size_t)w * (size_t)h;
    CK(cuMemAlloc(&d_nodes, (size_t)n_nodes * 44));
    CK(cuMemAlloc(&d_prims, (size_t)n_prims * 48));
    CK(cuMemAlloc(&d_hits, npix * 36));
    CK(cuMemAlloc(&d_out, npix * 16));
    CK(cuMemcpyHtoD(d_nodes, nodes44, (size_t)n_nodes * 44));
    CK(cuMemcpyHtoD(d_prims, prims48, (size_t)n_prims * 48));
    CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e2, CU_EVENT_DEFAULT));
    {
        ref_camera_t c;
        memcpy(c.v, cam, sizeof(c.v));
        ref_tree_t tree = {d_nodes, d_prims};
        ref_float3_t L = {light[0], light[1], light[2]};
        float wf = (float)w, hf = (float)h;
        void* a_ray[] = {&c, &tree, &d_hits, &wf, &hf};
        void* a_light[] = {&c, &d_hits, &d_prims, &d_out, &L, &wf, &hf};
        const unsigned gx = (unsigned)((w + 7) / 8), gy = (unsigned)((h + 3) / 4);
        double t_ray = 0, t_light = 0, t_frame = 0;
        for (int it = 0; it <= reps; ++it) {
            CK(cuEventRecord(e0, 0));
            CK(cuLaunchKernel(g_ray, gx, gy, 1, 8, 4, 1, 0, 0, a_ray, 0));
            CK(cuEventRecord(e1, 0));
            CK(cuCtxSynchronize());
            CK(cuLaunchKernel(g_light, gx, gy, 1, 8, 4, 1, 0, 0, a_light, 0));
            CK(cuEventRecord(e2, 0));
            CK(cuCtxSynchronize());
            if (it > 0) {
                float a = 0, b = 0, f = 0;
                CK(cuEventElapsedTime(&a, e0, e1));
                CK(cuEventElapsedTime(&b, e1, e2));
                CK(cuEventElapsedTime(&f, e0, e2));
                t_ray += a;
                t_light += b;
                t_frame += f;
            }
        }
        if (reps > 0) {
            if (ms_ray) *ms_ray = (float)(t_ray / reps);
            if (ms_light) *ms_light = (float)(t_light / reps);
            if (ms_frame) *ms_frame = (float)(t_frame / reps);
        }
    }
    if (hits36) CK(cuMemcpyDtoH(hits36, d_hits, npix * 36));
    if (rgba) CK(cuMemcpyDtoH(rgba, d_out, npix * 16));
done:
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    if (e2) cuEventDestroy(e2);
    if (d_nodes) cuMemFree(d_nodes);
    if (d_prims) cuMemFree(d_prims);
    if (d_hits) cuMemFree(d_hits);
    if (d_out) cuMemFree(d_out);
    return rc;
}
