// Floatexp form kernels: one field per launch (the per-field entry point),
// the batched persistent queue over many fields of any formula and size, the
// tile-scheduled queue (64x64 tiles claimed in a given order, per-tile cost
// and tail timing recorded), the coarse tile probe with the cost network's
// features, and the heaviest-first ordering of tiles.  All run the same
// per-pixel code (render_fe.cuh), so scheduling never changes a pixel.
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.h"
#include "render_fe_alt.cuh"

namespace fgb {
namespace {

__global__ void __launch_bounds__(128, 8) floatexp_kernel(const FxParams p) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const long long index = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (index >= pixels) return;
    const int py = static_cast<int>(index / p.width);
    const int px = static_cast<int>(index - static_cast<long long>(py) * p.width);
    fxk::render_pixel(p, px, py);
}

// Batched persistent form: every warp claims chunks of pixels from one
// device counter over all fields of the batch (fields in the order given,
// heaviest first when the caller orders them so) and renders them with the
// per-pixel code above.  Lanes of a warp stay on neighbouring pixels, whose
// paths through the series/BLA/tail code coincide (31.5 of 32 lanes active
// per instruction on the 1920x1080 keyframes), so no lane refill is needed.
__global__ void __launch_bounds__(128, 8) floatexp_queue_kernel(const __grid_constant__ FxBatch b) {
    constexpr unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const long long total = b.first[b.count];
    int f = 0;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(b.counter, static_cast<unsigned long long>(b.chunk));
        base = __shfl_sync(kFull, base, 0);
        if (static_cast<long long>(base) >= total) break;
        const long long end = static_cast<long long>(base) + b.chunk < total ? static_cast<long long>(base) + b.chunk
                                                                              : total;
        for (long long g = static_cast<long long>(base) + lane; g < end; g += 32) {
            while (g >= b.first[f + 1]) ++f;
            const FxParams& p = b.field[f];
            const int local = static_cast<int>(g - b.first[f]);
            const int py = local / p.width;
            const int px = local - py * p.width;
            fxk::render_pixel(p, px, py);
        }
    }
}

// Series prologue: one thread per field rescales the F2e coefficients to
// the field's view (see FxSeriesScaled).
__global__ void series_prologue_kernel(const __grid_constant__ FxBatch b) {
    const int f = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (f >= b.count) return;
    const FxParams& p = b.field[f];
    FxSeriesScaled* out = p.series_scaled;
    if (!out || !p.series_on) return;
    const int scale = p.view_width.e > p.view_height.e ? p.view_width.e : p.view_height.e;
    const int terms = p.series_terms < kMaxSeriesTerms ? p.series_terms : kMaxSeriesTerms;
    int shift = -0x3fffffff;
    for (int k = 1; k < terms; ++k) {
        const f32x::F2e c = p.series[k];
        if (c.x == 0.0f && c.y == 0.0f) continue;
        const int e = c.e + k * scale;
        shift = e > shift ? e : shift;
    }
    if (shift == -0x3fffffff) shift = 0;
    out->b[0][0] = 0.0f;
    out->b[0][1] = 0.0f;
    // Trailing terms below 2^-48 of the largest are dropped from the pixels'
    // Horner loop: with |u| <= 1 each is smaller than that largest term
    // times u^k by more than float rounding can see.  (Terms inside the kept
    // range stay, however small: a small low-order coefficient still
    // dominates near the view's centre.)
    int used = 2;
    for (int k = 1; k < terms; ++k) {
        const f32x::F2e c = p.series[k];
        const long long d = static_cast<long long>(c.e) + static_cast<long long>(k) * scale - shift;
        const bool keep = d > -200 && !(c.x == 0.0f && c.y == 0.0f);
        out->b[k][0] = keep ? f32x::ldexpf_fast(c.x, static_cast<int>(d)) : 0.0f;
        out->b[k][1] = keep ? f32x::ldexpf_fast(c.y, static_cast<int>(d)) : 0.0f;
        if (keep && d > -48 && k + 1 > used) used = k + 1;
    }
    out->terms = used < terms ? used : terms;
    out->shift = shift;
    out->scale = scale;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Field of a batch tile id (binary search over the tile prefix).
__device__ __forceinline__ int tile_field(const FxBatch& b, int tile) {
    int lo = 0, hi = b.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b.tiles_first[mid] <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Tile-scheduled persistent queue: a warp claims one band (tile_rows rows)
// of a 64x64 tile at a time, tiles in `order`.
__global__ void __launch_bounds__(128, 8) floatexp_tile_kernel(const __grid_constant__ FxBatch b) {
    constexpr unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const int bands = kTileSide / b.tile_rows;
    const long long units = static_cast<long long>(b.tiles_first[b.count]) * bands;
    while (true) {
        unsigned long long unit = 0;
        if (lane == 0) unit = atomicAdd(b.counter, 1ull);
        unit = __shfl_sync(kFull, unit, 0);
        if (static_cast<long long>(unit) >= units) break;
        const long long start = clock64();
        if (b.timing && lane == 0) {
            const unsigned long long now = global_ns();
            atomicMin(&b.timing[0], now);
            atomicMax(&b.timing[1], now);
        }
        const int rank = static_cast<int>(unit / bands);
        const int band = static_cast<int>(unit - static_cast<long long>(rank) * bands);
        const int tile = b.order ? static_cast<int>(b.order[rank]) : rank;
        const int f = tile_field(b, tile);
        const FxParams& p = b.field[f];
        const int t = tile - b.tiles_first[f];
        const int ty = t / b.tiles_x[f];
        const int tx = t - ty * b.tiles_x[f];
        const int x0 = tx * kTileSide;
        const int y0 = ty * kTileSide + band * b.tile_rows;
        for (int i = static_cast<int>(lane); i < kTileSide * b.tile_rows; i += 32) {
            const int px = x0 + (i & (kTileSide - 1));
            const int py = y0 + i / kTileSide;
            if (px >= p.width || py >= p.height) continue;
            fxk::render_pixel(p, px, py);
        }
        __syncwarp();
        if (lane == 0) {
            if (b.tile_cost) atomicAdd(&b.tile_cost[tile], static_cast<unsigned long long>(clock64() - start));
            if (b.timing) atomicMax(&b.timing[2], global_ns());
        }
    }
}

// Coarse probe: 16x16 samples (every 4th pixel each way, centred in its 4x4
// block and clamped to the field) of every tile, through the same per-pixel
// code; glitched samples count 0.
__global__ void __launch_bounds__(128) tile_probe_kernel(const __grid_constant__ FxBatch b, std::uint32_t* probe) {
    const long long samples = static_cast<long long>(b.tiles_first[b.count]) * mlp::kProbe;
    for (long long s = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; s < samples;
         s += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int tile = static_cast<int>(s / mlp::kProbe);
        const int k = static_cast<int>(s - static_cast<long long>(tile) * mlp::kProbe);
        const int f = tile_field(b, tile);
        const FxParams& p = b.field[f];
        const int t = tile - b.tiles_first[f];
        const int ty = t / b.tiles_x[f];
        const int tx = t - ty * b.tiles_x[f];
        int px = tx * kTileSide + (k % mlp::kProbeSide) * kProbeStride + kProbeStride / 2;
        int py = ty * kTileSide + (k / mlp::kProbeSide) * kProbeStride + kProbeStride / 2;
        px = px < p.width ? px : p.width - 1;
        py = py < p.height ? py : p.height - 1;
        probe[s] = fxk::pixel_count(p, px, py);
    }
}

// Network features of each tile: log(1 + count) / log(1 + cap) for the 256
// probe samples, log10 zoom / 100, log10 cap / 7, zeros to 320; zero rows
// pad to `rows`.
__global__ void tile_features_kernel(const __grid_constant__ FxBatch b, const std::uint32_t* probe,
                                     __nv_bfloat16* features, int rows) {
    const long long total = static_cast<long long>(rows) * mlp::kFeatures;
    const int tiles = b.tiles_first[b.count];
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int tile = static_cast<int>(i / mlp::kFeatures);
        const int k = static_cast<int>(i - static_cast<long long>(tile) * mlp::kFeatures);
        float v = 0.0f;
        if (tile < tiles) {
            const int f = tile_field(b, tile);
            const float cap = static_cast<float>(b.field[f].max_iter);
            if (k < mlp::kProbe) {
                v = log1pf(static_cast<float>(probe[static_cast<long long>(tile) * mlp::kProbe + k])) / log1pf(cap);
            } else if (k == mlp::kProbe) {
                v = b.log_zoom[f] / 100.0f;
            } else if (k == mlp::kProbe + 1) {
                v = log10f(cap) / 7.0f;
            }
        }
        features[i] = __float2bfloat16_rn(v);
    }
}

// Heaviest-first order from predicted normalised log costs: a counting sort
// over 1024 buckets of [-8, 8) in one block (descending).
__global__ void __launch_bounds__(1024) tile_order_kernel(const float* predicted, int tiles, unsigned* order) {
    __shared__ unsigned count[1024];
    __shared__ unsigned offset[1024];
    count[threadIdx.x] = 0;
    __syncthreads();
    auto bucket = [](float v) {
        int k = static_cast<int>(floorf((v + 8.0f) * 64.0f));
        k = k < 0 ? 0 : (k > 1023 ? 1023 : k);
        return 1023 - k;  // heaviest first
    };
    for (int i = threadIdx.x; i < tiles; i += blockDim.x) {
        const float v = predicted[i];
        atomicAdd(&count[bucket(isfinite(v) ? v : 0.0f)], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned run = 0;
        for (int k = 0; k < 1024; ++k) {
            offset[k] = run;
            run += count[k];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < tiles; i += blockDim.x) {
        const float v = predicted[i];
        const unsigned slot = atomicAdd(&offset[bucket(isfinite(v) ? v : 0.0f)], 1u);
        order[slot] = static_cast<unsigned>(i);
    }
}

FxBatch make_batch(const FxParams* fields, const float* log_zoom, int count) {
    FxBatch b{};
    b.count = count;
    long long pixels = 0;
    int tiles = 0;
    for (int f = 0; f < count; ++f) {
        b.field[f] = fields[f];
        b.first[f] = pixels;
        b.tiles_first[f] = tiles;
        b.tiles_x[f] = (fields[f].width + kTileSide - 1) / kTileSide;
        b.log_zoom[f] = log_zoom ? log_zoom[f] : 0.0f;
        pixels += static_cast<long long>(fields[f].width) * fields[f].height;
        tiles += b.tiles_x[f] * ((fields[f].height + kTileSide - 1) / kTileSide);
    }
    b.first[count] = pixels;
    b.tiles_first[count] = tiles;
    return b;
}

int resident_grid(const void* kernel, int blocks_per_sm, long long needed_blocks) {
    int device = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
    if (per_sm <= 0) per_sm = 1;
    const int use = blocks_per_sm > 0 && blocks_per_sm < per_sm ? blocks_per_sm : per_sm;
    long long grid = static_cast<long long>(sms) * use;
    if (grid > needed_blocks) grid = needed_blocks;
    return grid < 1 ? 1 : static_cast<int>(grid);
}

}  // namespace

cudaError_t launch_series_prologue(const FxParams* fields, int count, cudaStream_t stream) {
    if (count < 1 || count > kMaxFxFields) return cudaErrorInvalidValue;
    const FxBatch b = make_batch(fields, nullptr, count);
    series_prologue_kernel<<<(count + 63) / 64, 64, 0, stream>>>(b);
    return cudaGetLastError();
}

cudaError_t floatexp_queue_attributes(bool tiles, cudaFuncAttributes* attributes) {
    return tiles ? cudaFuncGetAttributes(attributes, floatexp_tile_kernel)
                 : cudaFuncGetAttributes(attributes, floatexp_queue_kernel);
}

int floatexp_queue_occupancy(bool tiles) {
    int blocks = 0;
    if (tiles) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, floatexp_tile_kernel, 128, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, floatexp_queue_kernel, 128, 0);
    }
    return blocks > 0 ? blocks : 1;
}

int batch_tiles(const FxParams* fields, int count) {
    int tiles = 0;
    for (int f = 0; f < count; ++f) {
        tiles += ((fields[f].width + kTileSide - 1) / kTileSide) * ((fields[f].height + kTileSide - 1) / kTileSide);
    }
    return tiles;
}

cudaError_t launch_floatexp_tiles(const FxParams* fields, const float* log_zoom, int count,
                                  unsigned long long* counter, const QueueShape& shape, const TileSchedule& schedule,
                                  cudaStream_t stream) {
    if (count < 1 || count > kMaxFxFields || !counter) return cudaErrorInvalidValue;
    const int rows = schedule.tile_rows;
    if (rows <= 0 || rows > kTileSide || kTileSide % rows != 0) return cudaErrorInvalidValue;
    FxBatch b = make_batch(fields, log_zoom, count);
    b.counter = counter;
    b.chunk = 1;
    b.tile_rows = rows;
    b.order = schedule.order;
    b.tile_cost = schedule.tile_cost;
    b.timing = schedule.timing;
    cudaError_t status = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (status == cudaSuccess && b.tile_cost) {
        status = cudaMemsetAsync(b.tile_cost, 0, sizeof(unsigned long long) * b.tiles_first[count], stream);
    }
    if (status == cudaSuccess && b.timing) {
        status = cudaMemsetAsync(b.timing, 0xff, sizeof(unsigned long long), stream);
        if (status == cudaSuccess) status = cudaMemsetAsync(b.timing + 1, 0, 2 * sizeof(unsigned long long), stream);
    }
    if (status != cudaSuccess) return status;
    const long long units = static_cast<long long>(b.tiles_first[count]) * (kTileSide / rows);
    const int grid = resident_grid(reinterpret_cast<const void*>(floatexp_tile_kernel), shape.blocks_per_sm,
                                   (units + 3) / 4);
    floatexp_tile_kernel<<<grid, 128, 0, stream>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_tile_probe(const FxParams* fields, const float* log_zoom, int count, std::uint32_t* probe,
                              __nv_bfloat16* features, int feature_rows, cudaStream_t stream) {
    if (count < 1 || count > kMaxFxFields || !probe || !features) return cudaErrorInvalidValue;
    const FxBatch b = make_batch(fields, log_zoom, count);
    const long long samples = static_cast<long long>(b.tiles_first[count]) * mlp::kProbe;
    const int grid = resident_grid(reinterpret_cast<const void*>(tile_probe_kernel), 0, (samples + 127) / 128);
    tile_probe_kernel<<<grid, 128, 0, stream>>>(b, probe);
    cudaError_t status = cudaGetLastError();
    if (status != cudaSuccess) return status;
    const long long values = static_cast<long long>(feature_rows) * mlp::kFeatures;
    tile_features_kernel<<<static_cast<unsigned>((values + 255) / 256 < 4096 ? (values + 255) / 256 : 4096), 256, 0,
                           stream>>>(b, probe, features, feature_rows);
    return cudaGetLastError();
}

cudaError_t launch_tile_order(const float* predicted, int tiles, unsigned* order, cudaStream_t stream) {
    if (tiles < 1 || !predicted || !order) return cudaErrorInvalidValue;
    tile_order_kernel<<<1, 1024, 0, stream>>>(predicted, tiles, order);
    return cudaGetLastError();
}

cudaError_t launch_floatexp_mandelbrot(const FxParams& p, cudaStream_t stream) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    floatexp_kernel<<<static_cast<unsigned>((pixels + 127) / 128), 128, 0, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_floatexp_batch(const FxParams* fields, int count, unsigned long long* counter,
                                  const QueueShape& shape, cudaStream_t stream) {
    if (count < 1 || count > kMaxFxFields || !counter) return cudaErrorInvalidValue;
    static_assert(sizeof(FxBatch) <= 32000, "kernel parameter limit");
    FxBatch b{};
    b.count = count;
    b.chunk = shape.chunk > 0 ? shape.chunk : 256;
    b.counter = counter;
    long long pixels = 0;
    for (int f = 0; f < count; ++f) {
        b.field[f] = fields[f];
        b.first[f] = pixels;
        pixels += static_cast<long long>(fields[f].width) * fields[f].height;
    }
    b.first[count] = pixels;
    static int per_sm = 0;
    if (per_sm == 0) {
        int blocks = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, floatexp_queue_kernel, 128, 0);
        per_sm = blocks > 0 ? blocks : 1;
    }
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int use = shape.blocks_per_sm > 0 && shape.blocks_per_sm < per_sm ? shape.blocks_per_sm : per_sm;
    long long grid = static_cast<long long>(sms) * use;
    const long long needed = (pixels + 127) / 128;
    if (grid > needed) grid = needed;
    if (grid < 1) grid = 1;
    cudaError_t status = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
    if (status != cudaSuccess) return status;
    floatexp_queue_kernel<<<static_cast<unsigned>(grid), 128, 0, stream>>>(b);
    return cudaGetLastError();
}
}  // namespace fgb
