// Launch interface of the CSG ray-casting kernels.
#pragma once

#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "scene.hpp"

namespace csgrt {

struct Planes {
    uint32_t* rgba8 = nullptr;
    float4* rgba32f = nullptr;
    float* t = nullptr;
    int32_t* prim = nullptr;
    float* normal = nullptr;  // three planes of w*h
};

struct Camera {
    float v[15];  // x y z rotX rotY fov forward[3] right[3] up[3] (reference Camera layout)
};

// Everything one view needs: scene, camera, light, size, output planes.
struct ViewParams {
    DeviceScene scene;
    Camera cam;
    float light[3];
    int32_t w, h;
    Planes out;
};

// Per-ray iteration cap of the traversal loop.  The reference has none; the largest
// count seen on the reference scenes is a few thousand (testCheese512), so the cap is
// never reached by a well-formed tree and only stops a runaway ray on a shared GPU.
constexpr uint32_t kIterCap = 1u << 20;

// The cap the next launches use (kIterCap unless csg_set_iteration_cap changed it).
uint32_t iteration_cap();
void set_iteration_cap(uint32_t cap);

// Where the scene's centre falls in a frame, in block tiles (ok: in front of the camera).
struct ProjectedCentre {
    bool ok = false;
    float x = 0.f, y = 0.f;
};

// Per-scene state of the cost-ordered block dispatch of large frames (launch_render).  The
// render kernel records each block's duration; the next frame of the same scene, on the same
// tile grid and stream, starts its tiles longest first.  One stream owns the state (the first
// that renders a large frame of the scene outside a graph capture); renders on any other
// stream use the plain centre-out order and leave the state alone.  Only the order in which
// blocks start changes, never a pixel.  Frames whose longest blocks are short against the
// whole frame gain nothing from the order and pay for the recording: a cost summary, written
// by the order kernels into mapped host memory, turns the dispatch off for a while.
struct DispatchState {
    std::mutex mu;
    bool owned = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    int slots = 0;                                   // SMs x 6 resident blocks
    int32_t tiles_x = 0, tiles_y = 0, tw_log2 = -1;  // the grid `cost` was recorded on
    ProjectedCentre rec_centre;                      // and where the scene's centre was
    bool costs_valid = false;
    uint32_t* cost = nullptr;    // per tile (row-major): SM cycles from the block's start to its end
    uint32_t* order = nullptr;   // the k-th block to start renders tile order[k]
    uint32_t* counts = nullptr;  // per order-building block and cost class
    size_t capacity = 0;         // tiles `cost` and `order` hold
    bool failed = false;         // an allocation failed: every frame plain
    float* summary = nullptr;    // mapped host memory: {longest block, all blocks} (cycles, lower bounds)
    float* summary_dev = nullptr;  // its device address
    cudaEvent_t summary_ready = nullptr;
    bool summary_pending = false;
    int off_frames = 0;          // frames left to render without the dispatch
};
// Frees the device buffers (on the device they were allocated on).
cudaError_t release_dispatch(DispatchState& d);

// Fused RaycastKernel + LightningKernel for one view of one scene.  `status` is a device
// counter incremented once per ray that stopped at the iteration cap; `center`, the centre
// of the scene's root box, sets the order in which the pixel tiles start; `dispatch` (may be
// null) the scene's cost-ordered dispatch state.
cudaError_t launch_render(const DeviceScene& scene, const float center[3], const Camera& cam, const float light[3],
                          int32_t w, int32_t h, const Planes& out,
                          unsigned long long* status, cudaStream_t stream, bool host_out = false,
                          DispatchState* dispatch = nullptr);

// tan(fov / 2) exactly as the kernels' ray generation computes it (device tanf);
// a diagnostic for host code that restates the ray generation.
cudaError_t device_tan_half_fov(float fov, float* host_out);

}  // namespace csgrt
