// The opaque scene handle of the C ABI (csg_scene in include/csgrt.h).
#pragma once

#include <cstddef>

#include "scene.hpp"

struct csg_scene {
    csgrt::HostTree tree;
    csgrt::DeviceScene dev;
    void* dmem = nullptr;                   // one allocation for every device array
    size_t bytes = 0;
    unsigned long long* status = nullptr;   // rays stopped at the traversal iteration cap
    int device = 0;
};
