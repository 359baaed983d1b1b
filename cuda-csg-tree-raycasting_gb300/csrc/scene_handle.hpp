// The opaque scene handle of the C ABI (csg_scene in include/csgrt.h).
#pragma once

#include <cstddef>

#include "render.hpp"
#include "scene.hpp"

struct csg_scene {
    csgrt::HostTree tree;
    csgrt::DeviceScene dev;
    void* dmem = nullptr;                   // one allocation for every device array
    size_t bytes = 0;
    unsigned long long* status = nullptr;   // rays stopped at the traversal iteration cap
    int device = 0;
    float center[3] = {0.f, 0.f, 0.f};      // centre of the root's box (block order of single views)
    mutable csgrt::DispatchState dispatch;  // cost-ordered block dispatch of large frames
};

namespace csgrt {

// Byte offsets of a scene's arrays inside its one device allocation (16-byte aligned).
struct SceneLayout {
    size_t topo, kids, geo, color, lbox, bvh, status, total;
};
SceneLayout scene_layout(size_t n_nodes, size_t n_prims, size_t n_kids_f4, size_t n_bvh_f4);

}  // namespace csgrt
