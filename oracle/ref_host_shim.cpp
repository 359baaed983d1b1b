// Host build of the reference's own ray-casting code, used only as a test oracle.
//
// This translation unit is compiled by oracle/build_ref.py with g++ (no GPU) from the
// reference's source files where they lie.  It is NOT part of the product: only tests
// and the CPU-baseline leg of bench.py load it, to pin the C restatement in
// oracle/csg_oracle.c bit for bit against what the reference computes.
//
// What is included, unchanged except for one neutral patch applied by build_ref.py to a
// build copy of RaycastingKernels.cu (a `return true;` appended to cylinderHit, which
// otherwise falls off the end of a bool function, RaycastingKernels.cu:335-336; the
// return value is never read, RaycastingKernels.cu:113-133):
//   CSGRayCasting/Graphics/RayCasting/Kernels/RaycastingKernels.cu   (RaycastKernel, LightningKernel)
//   CSGRayCasting/Graphics/RayCasting/CSGTree/CSGTree.cu            (CSGTree::Parse, ConstructBVH)
//   CSGRayCasting/Graphics/RenderManager/Camera/Camera.cpp          (Camera::updateVectors, own TU)
//
// The CUDA built-in index variables are remapped to thread-local host variables so that
// each kernel body can be called once per pixel from an OpenMP loop (one "thread" per
// pixel, blockDim = 1x1, blockIdx = pixel coordinate).
#include <cuda_runtime.h>
#include <device_launch_parameters.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include <stdexcept>
#ifdef _OPENMP
#include <omp.h>
#endif

static thread_local uint3 shim_threadIdx;
static thread_local uint3 shim_blockIdx;
static thread_local dim3 shim_blockDim;
#define threadIdx shim_threadIdx
#define blockIdx shim_blockIdx
#define blockDim shim_blockDim

#include "RaycastingKernels.cu"  // patched build copy in oracle/_ref/src
#include "CSGTree.cu"
// Camera.cpp (Camera::updateVectors) is compiled as its own translation unit: Camera.h
// has no include guard.

extern "C" {

int ref_sizeof_node(void) { return (int)sizeof(CSGNode); }
int ref_sizeof_prim(void) { return (int)sizeof(Primitive); }
int ref_sizeof_camera(void) { return (int)sizeof(Camera); }
int ref_sizeof_rayhit(void) { return (int)sizeof(RayHit); }

// CSGTree::Parse (CSGTree.cu:5-152).  Copies the 44-byte CSGNode and 48-byte Primitive
// arrays out.  Returns 0 on success, 1 on a parse exception (message in err), 2 when the
// output arrays are too small.
int ref_parse(const char* text, size_t len, void* nodes_out, int max_nodes,
              void* prims_out, int max_prims, int* n_nodes, int* n_prims,
              char* err, size_t errlen)
{
    try {
        CSGTree tree = CSGTree::Parse(std::string(text, len));
        *n_nodes = (int)tree.nodes.size();
        *n_prims = (int)tree.primitives.primitives.size();
        if (*n_nodes > max_nodes || *n_prims > max_prims) return 2;
        std::memcpy(nodes_out, tree.nodes.data(), tree.nodes.size() * sizeof(CSGNode));
        std::memcpy(prims_out, tree.primitives.primitives.data(),
                    tree.primitives.primitives.size() * sizeof(Primitive));
        return 0;
    } catch (const std::exception& e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 1;
    }
}

// Camera (Camera.h:18-52, Camera.cpp:4-27): default-construct, then optionally
// setPosition / setRotation / setFOV, and copy out the 60-byte object.
void ref_camera(int set_pos, float px, float py, float pz,
                int set_rot, float pitch, float yaw,
                int set_fov, float fov_deg, float out[15])
{
    Camera cam;
    if (set_pos) cam.setPosition(px, py, pz);
    if (set_rot) cam.setRotation(pitch, yaw);
    if (set_fov) cam.setFOV(fov_deg);
    static_assert(sizeof(Camera) == 15 * sizeof(float), "Camera layout");
    std::memcpy(out, &cam, sizeof(Camera));
}

void ref_camera_move(float cam_io[15], float f, float r, float u)
{
    Camera cam;
    std::memcpy(&cam, cam_io, sizeof(Camera));
    cam.move(f, r, u);
    std::memcpy(cam_io, &cam, sizeof(Camera));
}

void ref_camera_rotate(float cam_io[15], float dpitch, float dyaw)
{
    Camera cam;
    std::memcpy(&cam, cam_io, sizeof(Camera));
    cam.rotate(dpitch, dyaw);
    std::memcpy(cam_io, &cam, sizeof(Camera));
}

// DirectionalLight::getLightDir (DirectionalLight.h:13-18); polar/azimuth in radians.
void ref_light_dir(int set, float polar, float azimuth, float out[3])
{
    DirectionalLight l;
    if (set) { l.polar = polar; l.azimuth = azimuth; }
    float3 d = l.getLightDir();
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

// Raycaster::Raycast (Raycaster.cu:23-34) on the host: RaycastKernel then LightningKernel
// for every pixel.  Outputs one plane per RayHit field (hit, t, position, normal,
// primitiveIdx) and the float4 colour.  Fields the reference leaves undefined on a miss
// (position, normal, primitiveIdx) are written as zero / -1 here.
void ref_render(const void* nodes, int n_nodes, const void* prims, int n_prims,
                const float cam_in[15], const float light[3], int w, int h,
                unsigned char* hit, float* t, float* pos, float* nrm, int* prim,
                float* rgba, int nthreads)
{
    (void)n_nodes; (void)n_prims;
    Camera cam;
    std::memcpy(&cam, cam_in, sizeof(Camera));
    CudaCSGTree tree;
    tree.nodes = (CSGNode*)nodes;
    tree.primitives = (Primitive*)prims;
    float3 ld = make_float3(light[0], light[1], light[2]);
    const long npix = (long)w * h;
    std::vector<RayHit> hits(npix);
    std::vector<float4> out(npix);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (long p = 0; p < npix; ++p) {
        shim_blockDim = dim3(1, 1, 1);
        shim_threadIdx = make_uint3(0, 0, 0);
        shim_blockIdx = make_uint3((unsigned)(p % w), (unsigned)(p / w), 0);
        RaycastKernel(cam, tree, hits.data(), (float)w, (float)h);
        LightningKernel(cam, hits.data(), tree.primitives, out.data(), ld, (float)w, (float)h);
    }
    for (long p = 0; p < npix; ++p) {
        const RayHit& r = hits[p];
        hit[p] = r.hit ? 1 : 0;
        t[p] = r.t;
        if (r.hit) {
            pos[3 * p] = r.position.x; pos[3 * p + 1] = r.position.y; pos[3 * p + 2] = r.position.z;
            nrm[3 * p] = r.normal.x; nrm[3 * p + 1] = r.normal.y; nrm[3 * p + 2] = r.normal.z;
            prim[p] = r.primitiveIdx;
        } else {
            pos[3 * p] = pos[3 * p + 1] = pos[3 * p + 2] = 0.f;
            nrm[3 * p] = nrm[3 * p + 1] = nrm[3 * p + 2] = 0.f;
            prim[p] = -1;
        }
        rgba[4 * p] = out[p].x; rgba[4 * p + 1] = out[p].y;
        rgba[4 * p + 2] = out[p].z; rgba[4 * p + 3] = out[p].w;
    }
}

}  // extern "C"
