// Output-plane addresses of the batched entry points (csg_batch_create,
// csg_render_views_noalloc): device (or managed) memory is used as it is, page-locked host
// memory through its mapped device address (the kernel then writes host memory over the
// host link), and pageable host memory, which a kernel cannot write, is refused.
#pragma once

#include <cuda_runtime.h>

#include "csgrt.h"

namespace csgrt {

inline int plane_address(void* p, void** dev)
{
    *dev = nullptr;
    if (!p) return CSG_OK;
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    cudaGetLastError();  // an unregistered pointer may leave an error behind on older runtimes
    if (e != cudaSuccess) return CSG_E_ARG;
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        *dev = p;
        return CSG_OK;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) {
        *dev = a.devicePointer;
        return CSG_OK;
    }
    return CSG_E_ARG;
}

// Rewrites every non-null plane of `out` to the address the kernel writes it through.
inline int device_planes(csg_planes& out)
{
    void* d = nullptr;
    int rc = CSG_OK;
    if ((rc = plane_address(out.rgba8, &d)) != CSG_OK) return rc;
    out.rgba8 = static_cast<uint32_t*>(d);
    if ((rc = plane_address(out.rgba32f, &d)) != CSG_OK) return rc;
    out.rgba32f = static_cast<float*>(d);
    if ((rc = plane_address(out.t, &d)) != CSG_OK) return rc;
    out.t = static_cast<float*>(d);
    if ((rc = plane_address(out.prim, &d)) != CSG_OK) return rc;
    out.prim = static_cast<int32_t*>(d);
    if ((rc = plane_address(out.normal, &d)) != CSG_OK) return rc;
    out.normal = static_cast<float*>(d);
    return CSG_OK;
}

}  // namespace csgrt
