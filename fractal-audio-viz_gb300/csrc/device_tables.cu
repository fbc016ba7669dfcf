// Upload of one reference's tables to HBM, once per handle generation.
//
// A handle's tables are immutable after creation, so the device copy is made
// on the first render that needs it and shared by every later render of the
// same handle (the reference keys its OpenCL cache on the generation the
// same way, renderer.cpp:9077-9245).
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "runtime.h"

namespace fgb {

DeviceTables::~DeviceTables() {
    // Freed on the owning device; errors at process teardown are ignored.
    int current = -1;
    cudaGetDevice(&current);
    if (device >= 0 && current != device) cudaSetDevice(device);
    cudaFree(orbit);
    cudaFree(cubic);
    cudaFree(linear);
    cudaFree(deep_linear);
    cudaFree(alt);
    cudaFree(series);
    cudaFree(fe_orbit);
    cudaFree(fe_linear);
    cudaFree(fe_deep_linear);
    if (device >= 0 && current >= 0 && current != device) cudaSetDevice(current);
}

namespace {

template <typename T>
T* upload(const std::vector<T>& host) {
    if (host.empty()) return nullptr;
    T* device = nullptr;
    check_cuda(cudaMalloc(&device, host.size() * sizeof(T)), "cudaMalloc (reference tables)");
    check_cuda(cudaMemcpy(device, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice),
               "cudaMemcpy (reference tables)");
    return device;
}

template <typename T>
T* upload_levels(const std::vector<std::vector<T>>& levels, LevelIndex& index) {
    if (levels.size() > static_cast<std::size_t>(kMaxLevels)) {
        throw Failure{"BLA hierarchy has more levels than the device index holds"};
    }
    std::vector<T> flat;
    index = LevelIndex{};
    index.levels = static_cast<int>(levels.size());
    for (std::size_t level = 0; level < levels.size(); ++level) {
        index.offset[level] = static_cast<int>(flat.size());
        index.count[level] = static_cast<int>(levels[level].size());
        flat.insert(flat.end(), levels[level].begin(), levels[level].end());
    }
    return upload(flat);
}

}  // namespace

std::shared_ptr<DeviceTables> device_tables(ReferenceContext& ctx) {
    const int device = current_device();
    std::lock_guard<std::mutex> lock(ctx.device_mutex);
    if (ctx.device && ctx.device->device == device) return ctx.device;
    auto tables = std::make_shared<DeviceTables>();
    tables->device = device;
    const std::vector<OrbitRec> records = make_orbit_records(ctx);
    tables->orbit = upload(records);
    tables->orbit_size = static_cast<int>(records.size());
    tables->cubic = upload_levels(ctx.cubic, tables->cubic_index);
    tables->linear = upload_levels(ctx.linear, tables->linear_index);
    tables->deep_linear = upload_levels(ctx.deep_linear, tables->deep_linear_index);
    tables->alt = upload_levels(ctx.alt, tables->alt_index);
    tables->series = upload(ctx.series.coeff);
    tables->series_terms = static_cast<int>(ctx.series.coeff.size());
    ctx.device = tables;
    return tables;
}

}  // namespace fgb
