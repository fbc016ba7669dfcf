// Per-thread CUDA runtime state behind the C ABI: one non-blocking stream per
// calling host thread, grow-only device scratch for the host-buffer entry
// points, the time-budget stamp slot and the stats counters.  The reference
// lets several Python threads call the ABI at once (prefetch executor, live
// view); per-thread streams keep those calls independent.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <map>
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
    kScratchDirect,
    kScratchQueue,
    kScratchTiles,
    kScratchSeries,
    kScratchAtlas,
    kScratchSurface,
    kScratchPoints,
    kScratchPlanesIn,
    kScratchPlanesOut,
    kScratchDiscard,  // planes a batch's plain kernels write but no caller asked for
    kScratchAltQueue, // claim counters of the alternate-formula queue (one per lane stream + one)
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
    // Completion of the last launch that used the scratch buffers, recorded
    // on whichever stream it ran (a caller's stream for the device entry
    // points); the next launch on another stream waits for it.
    cudaEvent_t scratch_done = nullptr;
    bool scratch_recorded = false;
    // Keyframe batches: a second stream for the direct (FP64) fields so they
    // overlap the floatexp (FP32) fields, a capture stream, fork/join events
    // and the instantiated CUDA graphs of batches seen before.
    cudaStream_t side = nullptr;
    cudaStream_t capture = nullptr;
    cudaEvent_t fork = nullptr;
    cudaEvent_t join = nullptr;
    std::map<std::string, cudaGraphExec_t> graphs;
    // Plain-form (FP64) fields of a batch are dealt over these streams, so a
    // field's long-orbit tail overlaps the next fields' launches instead of
    // holding the GPU mostly idle until it ends.
    static constexpr int kPlainLanes = 8;
    cudaStream_t lanes[kPlainLanes] = {};
    cudaEvent_t lane_join[kPlainLanes] = {};
    int last_shapes[4] = {};
    int pinned_shapes[4] = {};  // set by fractal_gb300_set_queue_shapes
    void* costnet = nullptr;    // attached tile-cost network (not owned)
    cudaStream_t tile_stream = nullptr;  // stream of the last tile-scheduled batch
    cudaStream_t batch_stream = nullptr; // stream of the last keyframe batch
    int last_tiles = 0;
    unsigned* atlas_exact_count = nullptr;  // exact-pass counter of the last atlas frame
    bool shapes_pinned = false;
    double last_kernel_ms = 0.0;
    ~ThreadRuntime();
};

// The calling thread's runtime, created on first use (throws Failure when no
// CUDA device is usable).
ThreadRuntime& thread_runtime();
void* scratch(ThreadRuntime& rt, ScratchSlot slot, std::size_t bytes);
// Order scratch use across streams of one thread: wait_scratch before the
// first launch on `stream` that touches scratch, release_scratch after the
// last one.
void wait_scratch(ThreadRuntime& rt, cudaStream_t stream);
void release_scratch(ThreadRuntime& rt, cudaStream_t stream);

std::shared_ptr<DeviceTables> device_tables(ReferenceContext& ctx);
void floatexp_tables(ReferenceContext& ctx, DeviceTables& dev);

}  // namespace fgb
