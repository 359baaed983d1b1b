// Batched rendering of many views of many scenes in one persistent launch.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "render.hpp"

namespace csgrt {

// Device descriptor of one view of a batch.
struct BatchView {
    ViewParams view;
    int32_t tiles_x;  // block tiles per row for the batch's tile shape
    int32_t pad[3];
};

// Work item: block tile `tile` of view `view`.
struct BatchItem {
    int32_t view;
    int32_t tile;
};

struct BatchLaunch {
    const BatchView* views;
    const BatchItem* items;
    int32_t n_items;
    int* counter;                  // scratch: next work item (zeroed before every launch)
    unsigned long long* status;    // rays stopped at the iteration cap
    int32_t tw_log2;               // warp tile width = 1 << tw_log2, height = 32 >> tw_log2
    int32_t live_words;            // live-mask words allocated per ray (max over the batch)
    uint32_t iter_cap;
    int32_t stack_class;           // max over the batch
    int32_t rolled;                // kernel variant (any view needs the rolled one)
    int32_t grid;                  // persistent grid size
};

// Grid size that fills the GPU once with the kernel variant of `l`.
cudaError_t batch_grid_size(BatchLaunch& l);
// Enqueues the counter reset and the persistent kernel on `stream` (capturable).
cudaError_t launch_batch(const BatchLaunch& l, cudaStream_t stream);

}  // namespace csgrt
