// Direct field render without any device allocation.
//
// Some callers cannot call cudaMalloc: code running inside a memory pool or
// allocator hook that must not re-enter the allocator, processes that
// pre-reserve all device memory at start-up and forbid growth afterwards,
// and real-time loops where an allocation's implicit synchronisation would
// stall the frame.  For them the direct queue kernel gets its scratch (the
// warp claim counter and the per-column/per-row coordinate tables) from a
// fixed array compiled into this library instead of the thread's grow-only
// scratch buffers, which the other entry points allocate on first use.
//
// Limits and sharing:
//   * the array holds kNoAllocScratchBytes; a field needs 256 bytes plus
//     8 bytes per column and per row, so width + height may be at most
//     (kNoAllocScratchBytes - 256) / 8 = 16352.  Larger fields are rejected
//     with an error before anything is launched.
//   * every call, from every thread, uses the same array.  The kernel zeroes
//     the claim counter and rewrites the coordinate tables at the start of
//     each call, on the call's stream, so calls ordered on one stream are
//     independent.  Calls whose kernels overlap on the GPU (different
//     streams, no ordering between them) race on the array and give wrong
//     pixels.
//   * the first call on each device looks the array's address up with
//     cudaGetSymbolAddress (with that device current) and keeps it; make
//     that first call before any stream capture begins.
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <string>

#include "device.h"

namespace fgb {
namespace {

constexpr std::size_t kNoAllocScratchBytes = 128 * 1024;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char noalloc_scratch[kNoAllocScratchBytes];

std::mutex noalloc_mutex;
void* noalloc_address[kNoAllocMaxDevices] = {};

// The array's device address on the current device, looked up once per
// device.  Returns nullptr and sets `why` on failure.
void* scratch_address(std::string& why) {
    int device = -1;
    cudaError_t status = cudaGetDevice(&device);
    if (status != cudaSuccess) {
        why = std::string("cudaGetDevice: ") + cudaGetErrorString(status);
        return nullptr;
    }
    if (device < 0 || device >= kNoAllocMaxDevices) {
        why = "device index out of range for the no-allocation scratch";
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(noalloc_mutex);
    if (!noalloc_address[device]) {
        void* address = nullptr;
        status = cudaGetSymbolAddress(&address, noalloc_scratch);
        if (status != cudaSuccess || !address) {
            why = std::string("cudaGetSymbolAddress (no-allocation scratch): ") + cudaGetErrorString(status);
            return nullptr;
        }
        noalloc_address[device] = address;
    }
    return noalloc_address[device];
}

}  // namespace

std::size_t noalloc_scratch_limit() { return kNoAllocScratchBytes; }

bool launch_direct_noalloc(const DirectParams& p, cudaStream_t stream, std::string& why) {
    const std::size_t needed = direct_scratch_bytes(&p, 1, 0);
    if (needed > kNoAllocScratchBytes) {
        why = "field needs " + std::to_string(needed) + " bytes of scratch but the no-allocation entry point has " +
              std::to_string(kNoAllocScratchBytes) + " (width + height at most " +
              std::to_string((kNoAllocScratchBytes - 256) / 8) + ")";
        return false;
    }
    void* address = scratch_address(why);
    if (!address) return false;
    const cudaError_t status = launch_direct_batch(&p, 1, address, QueueShape{}, 0, stream);
    if (status != cudaSuccess) {
        why = std::string("direct kernel launch: ") + cudaGetErrorString(status);
        return false;
    }
    return true;
}

}  // namespace fgb
