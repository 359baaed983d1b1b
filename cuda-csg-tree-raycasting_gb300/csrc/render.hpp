// Launch interface of the CSG ray-casting kernels.
#pragma once

#include <cstdint>
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

// Fused RaycastKernel + LightningKernel for one view of one scene.  `status` is a device
// counter incremented once per ray that stopped at the iteration cap; `center`, the centre
// of the scene's root box, sets the order in which the pixel tiles start.
cudaError_t launch_render(const DeviceScene& scene, const float center[3], const Camera& cam, const float light[3],
                          int32_t w, int32_t h, const Planes& out,
                          unsigned long long* status, cudaStream_t stream, bool host_out = false);

// tan(fov / 2) exactly as the kernels' ray generation computes it (device tanf);
// a diagnostic for host code that restates the ray generation.
cudaError_t device_tan_half_fov(float fov, float* host_out);

}  // namespace csgrt
