// Per-thread CUDA runtime state behind the C ABI: one non-blocking stream per
// calling host thread, grow-only device scratch for the host-buffer entry
// points, the time-budget stamp slot and the stats counters.  The reference
// lets several Python threads call the ABI at once (prefetch executor, live
// view); per-thread streams keep those calls independent.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>

#include "reference.h"

namespace fgb {

struct DeviceTables;

void check_cuda(cudaError_t status, const char* what);
int current_device();

enum ScratchSlot {
    kScratchField = 0,
    kScratchCounts,
    kScratchPlaneIter,
    kScratchPhase,
    kScratchDeX,
    kScratchDeY,
    kScratchTest1,
    kScratchTest2,
    kScratchRgb,
    kScratchLut,
    kScratchKfpSamples,
    kScratchKfpAux,
    kScratchWork,
    kScratchCount
};

struct ThreadRuntime {
    int device = -1;
    cudaStream_t stream = nullptr;
    void* scratch[kScratchCount] = {};
    std::size_t capacity[kScratchCount] = {};
    unsigned long long* stats = nullptr;  // kStatsSlots counters
    unsigned long long* stamp = nullptr;  // time-budget origin
    cudaEvent_t start = nullptr;
    cudaEvent_t stop = nullptr;
    double last_kernel_ms = 0.0;
    ~ThreadRuntime();
};

// The calling thread's runtime, created on first use (throws Failure when no
// CUDA device is usable).
ThreadRuntime& thread_runtime();
void* scratch(ThreadRuntime& rt, ScratchSlot slot, std::size_t bytes);

std::shared_ptr<DeviceTables> device_tables(ReferenceContext& ctx);
void floatexp_tables(ReferenceContext& ctx, DeviceTables& dev);

}  // namespace fgb
