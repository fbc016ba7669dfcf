// The extern "C" boundary: renderer.h v10 hot subset plus GB300 extensions.
//
// Validation, error strings and the 0/1/NULL conventions follow the
// reference's exported API (renderer.cpp:15870-20535, render entry points at
// :19568-20013 and :20280-20474).  Every render and colour call runs on the
// GPU; no C++ exception crosses the boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "device.h"
#include "mlp.h"
#include "fractal_gb300.h"
#include "reference.h"
#include "runtime.h"

namespace fgb {

thread_local std::string last_error;
// Whether this thread has made its runtime (streams, scratch), and whether
// its last direct launch was a no-allocation one (whose counters live in
// the shared no-allocation array, not in the thread's scratch).
thread_local bool runtime_made = false;
thread_local bool last_direct_noalloc = false;

void set_error(const std::string& message) { last_error = message; }

void check_cuda(cudaError_t status, const char* what) {
    if (status != cudaSuccess) {
        throw Failure{std::string(what) + ": " + cudaGetErrorString(status)};
    }
}

int current_device() {
    int device = -1;
    check_cuda(cudaGetDevice(&device), "cudaGetDevice");
    return device;
}

ThreadRuntime::~ThreadRuntime() {
    for (void* p : scratch) cudaFree(p);
    cudaFree(stats);
    cudaFree(stamp);
    if (start) cudaEventDestroy(start);
    if (stop) cudaEventDestroy(stop);
    if (scratch_done) cudaEventDestroy(scratch_done);
    for (auto& entry : graphs) cudaGraphExecDestroy(entry.second);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    for (int l = 0; l < kPlainLanes; ++l) {
        if (lane_join[l]) cudaEventDestroy(lane_join[l]);
        if (lanes[l]) cudaStreamDestroy(lanes[l]);
    }
    if (side) cudaStreamDestroy(side);
    if (capture) cudaStreamDestroy(capture);
    if (stream) cudaStreamDestroy(stream);
}

ThreadRuntime& thread_runtime() {
    thread_local ThreadRuntime rt;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        throw Failure{"no CUDA device is available; this library renders on the GPU only"};
    }
    const int device = current_device();
    if (rt.stream == nullptr || rt.device != device) {
        rt.~ThreadRuntime();
        new (&rt) ThreadRuntime();
        runtime_made = true;
        rt.device = device;
        check_cuda(cudaStreamCreateWithFlags(&rt.stream, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(cudaMalloc(&rt.stats, sizeof(unsigned long long) * kStatsSlots), "cudaMalloc (stats)");
        check_cuda(cudaMalloc(&rt.stamp, sizeof(unsigned long long)), "cudaMalloc (stamp)");
        check_cuda(cudaEventCreate(&rt.start), "cudaEventCreate");
        check_cuda(cudaEventCreate(&rt.stop), "cudaEventCreate");
        check_cuda(cudaEventCreateWithFlags(&rt.scratch_done, cudaEventDisableTiming), "cudaEventCreate");
        // The FP64 direct queue's stream has the highest priority: when both
        // persistent queues are launched, its blocks are placed first, and
        // FP32-queue blocks beyond what fits beside them start as its blocks
        // finish (see the autotuner's over-subscribed candidates).
        int least = 0, greatest = 0;
        check_cuda(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
        check_cuda(cudaStreamCreateWithPriority(&rt.side, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
        check_cuda(cudaStreamCreateWithFlags(&rt.capture, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(cudaEventCreateWithFlags(&rt.fork, cudaEventDisableTiming), "cudaEventCreate");
        check_cuda(cudaEventCreateWithFlags(&rt.join, cudaEventDisableTiming), "cudaEventCreate");
        for (int l = 0; l < ThreadRuntime::kPlainLanes; ++l) {
            check_cuda(cudaStreamCreateWithFlags(&rt.lanes[l], cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaEventCreateWithFlags(&rt.lane_join[l], cudaEventDisableTiming), "cudaEventCreate");
        }
    }
    return rt;
}

void* scratch(ThreadRuntime& rt, ScratchSlot slot, std::size_t bytes) {
    if (bytes == 0) bytes = 1;
    if (rt.capacity[slot] < bytes) {
        // A stream may still use the old buffer.
        check_cuda(cudaStreamSynchronize(rt.stream), "cudaStreamSynchronize");
        if (rt.scratch_recorded) check_cuda(cudaEventSynchronize(rt.scratch_done), "cudaEventSynchronize");
        cudaFree(rt.scratch[slot]);
        rt.scratch[slot] = nullptr;
        rt.capacity[slot] = 0;
        check_cuda(cudaMalloc(&rt.scratch[slot], bytes), "cudaMalloc (scratch)");
        // Zeroed once: the direct queue's spill entries carry a generation
        // mark that must not match by accident.
        check_cuda(cudaMemset(rt.scratch[slot], 0, bytes), "cudaMemset (scratch)");
        rt.capacity[slot] = bytes;
    }
    return rt.scratch[slot];
}

void wait_scratch(ThreadRuntime& rt, cudaStream_t stream) {
    if (rt.scratch_recorded && stream != rt.stream) {
        check_cuda(cudaStreamWaitEvent(stream, rt.scratch_done, 0), "cudaStreamWaitEvent");
    } else if (rt.scratch_recorded) {
        check_cuda(cudaStreamWaitEvent(rt.stream, rt.scratch_done, 0), "cudaStreamWaitEvent");
    }
}

void release_scratch(ThreadRuntime& rt, cudaStream_t stream) {
    check_cuda(cudaEventRecord(rt.scratch_done, stream), "cudaEventRecord");
    rt.scratch_recorded = true;
}

namespace {

constexpr int kMaxIterations = 10'000'000;
constexpr int kMaxThreads = 4096;
constexpr long long kMaxPixels = 100'000'000;
constexpr int kStatsFields = 16;

// ----------------------------------------------------------------- stats
std::atomic<bool> stats_enabled{false};
std::mutex stats_mutex;
std::array<unsigned long long, kStatsSlots> last_stats{};

void publish_stats(const std::array<unsigned long long, kStatsSlots>& values) {
    std::lock_guard<std::mutex> lock(stats_mutex);
    last_stats = values;
}

// ------------------------------------------------------------ validation
bool valid_dims(int width, int height) {
    if (width <= 0 || height <= 0) return false;
    return static_cast<unsigned long long>(width)
        <= static_cast<unsigned long long>(kMaxPixels) / static_cast<unsigned long long>(height);
}
bool valid_iterations(int value) { return value > 0 && value <= kMaxIterations; }
bool valid_threads(int value) { return value >= 0 && value <= kMaxThreads; }
bool valid_precision(int value) { return value >= 128 && value <= 131072; }
bool valid_series(int order, int block) { return order >= 1 && order <= 32 && block >= 2 && block <= 4096; }
bool valid_formula(int formula) { return formula >= 0 && formula <= 3; }

bool valid_planes(const FractalRenderPlanes* planes, int width, int height) {
    if (!planes || !valid_dims(width, height)) return false;
    return planes->struct_size >= sizeof(FractalRenderPlanes) && planes->version == 1
        && planes->orbit_iteration && planes->phase && planes->de_x && planes->de_y && planes->test1
        && planes->test2;
}

FractalRenderOptions default_options() {
    FractalRenderOptions o{};
    o.struct_size = sizeof(FractalRenderOptions);
    o.version = FRACTAL_RENDER_OPTIONS_VERSION;
    o.strict = 1;
    o.allow_recovery = 0;
    o.time_budget_ms = 0;
    o.disable_bla = 0;
    o.disable_cycle = 0;
    o.strict_cycle = 0;
    o.series_min_terms = 8;
    o.series_max_terms = 32;
    o.max_bla_length = kMaxSafeBlaLength;
    o.max_linear_bla_length = kMaxSafeLinearBlaLength;
    o.backend = 0;
    o.escape_radius_mode = 0;
    o.coordinate_mode = 0;
    o.output_bias = 0.0;
    return o;
}

// checked_render_options (renderer.cpp:4729-4765).
FractalRenderOptions checked_options(const FractalRenderOptions* supplied) {
    FractalRenderOptions o = default_options();
    if (!supplied) return o;
    if (supplied->struct_size < sizeof(FractalRenderOptions) || supplied->version != FRACTAL_RENDER_OPTIONS_VERSION) {
        throw Failure{"unsupported FractalRenderOptions version or size"};
    }
    o = *supplied;
    auto flag = [](std::int32_t value, const char* label) {
        if (value != 0 && value != 1) throw Failure{std::string(label) + " must be 0 or 1"};
    };
    flag(o.strict, "strict render flag");
    flag(o.allow_recovery, "recovery flag");
    flag(o.disable_bla, "disable-BLA flag");
    flag(o.disable_cycle, "disable-cycle flag");
    flag(o.strict_cycle, "strict-cycle flag");
    if (o.escape_radius_mode != 0 && o.escape_radius_mode != 1) throw Failure{"unknown escape-radius mode"};
    if (o.coordinate_mode != 0 && o.coordinate_mode != 1) throw Failure{"unknown coordinate mode"};
    o.series_min_terms = std::clamp(o.series_min_terms, 1, 32);
    o.series_max_terms = std::clamp(o.series_max_terms, o.series_min_terms, 32);
    o.max_bla_length = std::clamp(o.max_bla_length, 1, kMaxSafeBlaLength);
    o.max_linear_bla_length = std::clamp(o.max_linear_bla_length, 1, kMaxSafeLinearBlaLength);
    if (o.time_budget_ms < 0) throw Failure{"render time budget cannot be negative"};
    if (!std::isfinite(o.output_bias) || o.output_bias < 0.0) {
        throw Failure{"render output bias must be finite and non-negative"};
    }
    return o;
}

void check_backend(const FractalRenderOptions& o) {
    if (o.backend == 0 || o.backend == FRACTAL_BACKEND_CUDA) return;
    if (o.backend == 1) throw Failure{"AVX2 backend requested but this build has no AVX2 support"};
    if (o.backend == 2) throw Failure{"OpenCL backend is not available in this build"};
    throw Failure{"unknown native render backend"};
}

// ------------------------------------------------------------ render core

long double fe_log10(const fx::Fe& v) {
    const long double log_two = 0.693147180559945309417232121458176568L;
    return (std::log(std::fabs(static_cast<long double>(v.m))) + static_cast<long double>(v.e) * log_two)
        / std::log(10.0L);
}

// Per-render geometry shared by the deep kernels (renderer.cpp:12690-12762).
struct DeepGeometry {
    fx::Fe view_height;
    fx::Fe view_width;
    fx::Fe pixel_spacing;
    fx::Fe current_input_radius;
};

DeepGeometry deep_geometry(const fx::Fe& zoom, int width, int height, int coordinate_mode) {
    DeepGeometry g;
    const fx::Fe inverse_zoom = fx::fe_div(fx::fe_from(1.0, 0), zoom);
    const double factor = viewport_height_factor(coordinate_mode);
    g.view_height = fx::fe_mul(inverse_zoom, factor);
    g.view_width = fx::fe_mul(g.view_height, static_cast<double>(width) / static_cast<double>(height));
    g.pixel_spacing = fx::fe_div(g.view_height, fx::fe_from(static_cast<double>(height), 0));
    g.current_input_radius = fx::fe_mul(inverse_zoom, factor);
    return g;
}

// A point render's inputs (fractal_render_points_impl, renderer.cpp:
// 20019-20186): device dc list, the largest |dc| (it replaces the view
// radius in the BLA and series decisions) and the exact-repair flags.
struct PointInput {
    const fx::Sc* points = nullptr;
    fx::Fe radius = {0.0, 0};
    std::uint8_t* exact_flags = nullptr;
};

void launch_deep_mandelbrot(ReferenceContext& ctx, DeviceTables& dev, const Outputs& out, int width, int height,
                            const fx::Fe& zoom, int max_iter, int series_order, int series_block,
                            const FractalRenderOptions& o, bool collect_stats, ThreadRuntime& rt,
                            cudaStream_t stream, const PointInput* points = nullptr) {
    DeepGeometry g = deep_geometry(zoom, width, height, o.coordinate_mode);
    if (points) g.current_input_radius = points->radius;
    const bool covers = fx::fe_cmp(g.current_input_radius, ctx.input_radius) <= 0;
    const bool disable_bla = !covers || o.disable_bla != 0;
    const bool cycle = o.disable_cycle == 0 && (o.strict == 0 || o.strict_cycle != 0);
    const bool use_deep = fx::fe_cmp(g.current_input_radius, ctx.deep_input_radius) <= 0;
    const fx::Fe ultra = fx::fe_mul(ctx.input_radius, 1.0e-40);
    const bool use_ultra = fx::fe_cmp(g.current_input_radius, ultra) <= 0;
    PlainParams p{};
    p.orbit = dev.orbit;
    p.orbit_size = dev.orbit_size;
    p.cubic = dev.cubic;
    p.cubic_index = dev.cubic_index;
    p.linear = use_deep ? dev.deep_linear : dev.linear;
    p.linear_index = use_deep ? dev.deep_linear_index : dev.linear_index;
    p.series = dev.series;
    p.series_terms = dev.series_terms;
    p.series_iteration = ctx.series.iteration;
    p.series_on = ctx.series.enabled && ctx.series.order >= o.series_min_terms
        && ctx.series.order <= o.series_max_terms
        && fx::fe_cmp(g.current_input_radius, fx::fe_sqrt(ctx.series.r2)) <= 0
        && ctx.series.iteration < max_iter && dev.series_terms > 1;
    p.series_r2 = fx::nrm_make(ctx.series.r2.m, ctx.series.r2.e);
    p.view_width = g.view_width;
    p.view_height = g.view_height;
    p.coordinate_mode = o.coordinate_mode;
    p.width = width;
    p.height = height;
    p.max_iter = max_iter;
    p.map_end = ctx.map_end;
    p.disable_bla = disable_bla;
    p.strict = o.strict;
    p.allow_recovery = o.allow_recovery;
    p.strict_cycle = o.strict_cycle;
    p.cycle = cycle ? 1 : 0;
    p.escape_mode = o.escape_radius_mode;
    p.max_bla_len = std::clamp(std::min(series_block, static_cast<int>(o.max_bla_length)), 2, kMaxSafeBlaLength);
    p.max_lin_len = std::clamp(std::min(series_block, static_cast<int>(o.max_linear_bla_length)), 2,
                               use_ultra ? kMaxSafeLinearBlaLength
                                         : (use_deep ? kMaxSafeDeepLinearBlaLength : kMaxSafeBlaLength));
    p.approx_order = std::clamp(series_order, 1, 3);
    p.output_bias = o.output_bias;
    p.pixel_spacing = g.pixel_spacing;
    p.out = out.field;
    p.counts = out.counts;
    p.p_iter = out.p_iter;
    p.p_phase = out.p_phase;
    p.p_dex = out.p_dex;
    p.p_dey = out.p_dey;
    p.p_t1 = out.p_t1;
    p.p_t2 = out.p_t2;
    if (o.time_budget_ms > 0) {
        check_cuda(launch_stamp_time(rt.stamp, stream), "time stamp launch");
        p.deadline_base = rt.stamp;
        p.budget_ns = static_cast<unsigned long long>(o.time_budget_ms) * 1000000ull;
    }
    p.stats = collect_stats ? rt.stats : nullptr;
    p.points = points ? points->points : nullptr;
    p.exact_flags = points ? points->exact_flags : nullptr;
    check_cuda(launch_plain_mandelbrot(p, out.p_iter != nullptr, collect_stats, stream),
               "plain Mandelbrot kernel launch");
}

// Claim counters of the alternate-formula queue: one 256-byte slot per lane
// stream of a batch, and one (the last) for single renders.
constexpr int kAltQueueSlots = ThreadRuntime::kPlainLanes + 1;
constexpr std::size_t kAltQueueStride = 256 / sizeof(unsigned long long);

unsigned long long* alt_queue_counters(ThreadRuntime& rt) {
    return static_cast<unsigned long long*>(scratch(rt, kScratchAltQueue, kAltQueueSlots * 256));
}

// `queue_counter`: the claim counter of the lane-refill queue (a batch
// passes its lane's slot); NULL takes the single-render slot, and point
// lists always run one thread per point.
void launch_deep_alternate(ReferenceContext& ctx, DeviceTables& dev, const Outputs& out, int width, int height,
                           const fx::Fe& zoom, int max_iter, const FractalRenderOptions& o, bool collect_stats,
                           ThreadRuntime& rt, cudaStream_t stream, const PointInput* points = nullptr,
                           unsigned long long* queue_counter = nullptr) {
    const DeepGeometry g = deep_geometry(zoom, width, height, o.coordinate_mode);
    AltParams p{};
    p.orbit = dev.orbit;
    p.orbit_size = dev.orbit_size;
    p.alt = dev.alt;
    p.alt_index = dev.alt_index;
    p.alt_start = ctx.alt_start;
    p.alt_input_radius2 = ctx.alt_input_radius2;
    p.series = dev.series;
    p.series_terms = dev.series_terms;
    p.series_iteration = ctx.series.iteration;
    p.series_r2 = fx::nrm_make(ctx.series.r2.m, ctx.series.r2.e);
    p.view_width = g.view_width;
    p.view_height = g.view_height;
    p.coordinate_mode = o.coordinate_mode;
    p.width = width;
    p.height = height;
    p.max_iter = max_iter;
    p.map_end = ctx.map_end;
    p.formula = ctx.formula;
    p.strict = o.strict;
    p.allow_recovery = o.allow_recovery;
    p.escape_mode = o.escape_radius_mode;
    p.output_bias = o.output_bias;
    p.pixel_spacing = g.pixel_spacing;
    p.parameter = ctx.parameter;
    p.current_input_radius2 = fx::fe_sqr(g.current_input_radius);
    p.out = out.field;
    p.counts = out.counts;
    p.p_iter = out.p_iter;
    p.p_phase = out.p_phase;
    p.p_dex = out.p_dex;
    p.p_dey = out.p_dey;
    p.p_t1 = out.p_t1;
    p.p_t2 = out.p_t2;
    // Alternate-formula policy (render_alternate_reference_impl,
    // renderer.cpp:12116-12137): the block table is used whenever it exists
    // (each block checks the pixel's parameter radius itself), the series
    // only for Julia, and cycle detection only for non-strict renders.
    p.disable_bla = o.disable_bla != 0 ? 1 : 0;
    p.max_lin_len = std::clamp(static_cast<int>(o.max_linear_bla_length), 2, kMaxSafeLinearBlaLength);
    p.series_on = ctx.formula == kFormulaJulia && ctx.series.enabled && ctx.series.iteration < max_iter
        && dev.series_terms > 1
        && (points == nullptr || fx::fe_cmp(points->radius, fx::fe_sqrt(ctx.series.r2)) <= 0);
    p.points = points ? points->points : nullptr;
    p.cycle = (o.disable_cycle == 0 && (o.strict == 0 || o.strict_cycle != 0)) ? 1 : 0;
    if (o.time_budget_ms > 0) {
        check_cuda(launch_stamp_time(rt.stamp, stream), "time stamp launch");
        p.deadline_base = rt.stamp;
        p.budget_ns = static_cast<unsigned long long>(o.time_budget_ms) * 1000000ull;
    }
    p.stats = collect_stats ? rt.stats : nullptr;
    if (points == nullptr && queue_counter == nullptr) {
        queue_counter = alt_queue_counters(rt) + (kAltQueueSlots - 1) * kAltQueueStride;
    }
    check_cuda(launch_plain_alternate(p, out.p_iter != nullptr, collect_stats, points ? nullptr : queue_counter,
                                      stream),
               "plain alternate-formula kernel launch");
}

// Spill-list entries for a direct batch of `pixels` pixels: enough for the
// long-running pixels of interior-heavy views (a full list only costs speed).
long long spill_entries(long long pixels) { return std::min<long long>(pixels, 1ll << 20); }

DirectParams make_direct_params(const Outputs& out, int width, int height, long double zoom, long double x_center,
                                long double y_center, int max_iter, int formula, double julia_re, double julia_im,
                                const FractalRenderOptions& o) {
    const double zoom_value = static_cast<double>(zoom);
    const double center_re = static_cast<double>(x_center);
    const double center_im = static_cast<double>(y_center);
    if (!std::isfinite(zoom_value) || zoom_value <= 0.0 || !std::isfinite(center_re) || !std::isfinite(center_im)) {
        throw Failure{"direct native coordinates or zoom exceed double range"};
    }
    const double height_span = viewport_height_factor(o.coordinate_mode) / zoom_value;
    const double width_span = height_span * static_cast<double>(width) / static_cast<double>(height);
    if (!std::isfinite(height_span) || !std::isfinite(width_span)) {
        throw Failure{"direct native viewport is outside double range"};
    }
    DirectParams p;
    std::memset(static_cast<void*>(&p), 0, sizeof p);  // padding too: the bytes key the graph cache
    p.center_re = center_re;
    p.center_im = center_im;
    p.width_span = width_span;
    p.height_span = height_span;
    p.coordinate_mode = o.coordinate_mode;
    p.width = width;
    p.height = height;
    p.max_iter = max_iter;
    p.formula = formula;
    p.julia_re = julia_re;
    p.julia_im = julia_im;
    p.output_bias = o.output_bias;
    p.escape_mode = o.escape_radius_mode;
    p.out = out.field;
    p.counts = out.counts;
    p.p_iter = out.p_iter;
    p.p_phase = out.p_phase;
    p.p_dex = out.p_dex;
    p.p_dey = out.p_dey;
    p.p_t1 = out.p_t1;
    p.p_t2 = out.p_t2;
    const std::uint32_t hints = static_cast<std::uint32_t>(o.reserved[0]);
    p.need_phase = (hints & FRACTAL_RENDER_HINT_SKIP_PHASE) == 0;
    p.need_de = (hints & FRACTAL_RENDER_HINT_SKIP_ANALYTIC_DE) == 0;
    p.pixel_spacing = height_span / static_cast<double>(height);
    return p;
}

void launch_direct_render(const Outputs& out, int width, int height, long double zoom, long double x_center,
                          long double y_center, int max_iter, int formula, double julia_re, double julia_im,
                          const FractalRenderOptions& o, cudaStream_t stream) {
    const DirectParams p = make_direct_params(out, width, height, zoom, x_center, y_center, max_iter, formula,
                                              julia_re, julia_im, o);
    ThreadRuntime& rt = thread_runtime();
    const long long spill = spill_entries(static_cast<long long>(width) * height);
    void* work = scratch(rt, kScratchDirect, direct_scratch_bytes(&p, 1, spill));
    check_cuda(launch_direct_batch(&p, 1, work, QueueShape{}, spill, stream), "direct kernel launch");
    last_direct_noalloc = false;
}

// Dispatch of a reference render by zoom depth and formula
// (renderer.cpp:19868-19950): >= 1e6 deep paths, else the direct path.
void render_from_reference(ReferenceContext& ctx, const Outputs& out, int width, int height,
                           const char* zoom_text, int max_iter, int series_order, int series_block,
                           const FractalRenderOptions& o, bool collect_stats, ThreadRuntime& rt,
                           cudaStream_t stream) {
    const fx::Fe zoom = parse_zoom_fe(zoom_text, ctx.precision_bits);
    const long double zoom_log10 = fe_log10(zoom);
    if (zoom_log10 >= 6.0L) {
        std::shared_ptr<DeviceTables> dev = device_tables(ctx);
        if (ctx.formula != kFormulaMandelbrot) {
            launch_deep_alternate(ctx, *dev, out, width, height, zoom, max_iter, o, collect_stats, rt, stream);
        } else {
            launch_deep_mandelbrot(ctx, *dev, out, width, height, zoom, max_iter, series_order, series_block, o,
                                   collect_stats, rt, stream);
        }
        return;
    }
    const long double zoom_direct = parse_zoom_direct(zoom_text);
    launch_direct_render(out, width, height, zoom_direct, ctx.x_center, ctx.y_center, max_iter, ctx.formula,
                         ctx.julia_re, ctx.julia_im, o, stream);
}

}  // namespace

// Floatexp form of a reference render.  It covers strict deep Mandelbrot
// fields (the production atlas path); shallow fields, the other formulas,
// non-strict cycle detection and time budgets use the plain form.
namespace {

// Zoom below which the reference pipeline renders a field on the direct
// path (visualizer.py:6152); the floatexp form renders such fields in its
// shallow mode (FxParams::shallow).
constexpr long double kShallowLog10Zoom = 12.0L;

// Floatexp kernel parameters of one field, or false when the field is not
// one the floatexp form covers (non-strict cycle detection, time budget,
// render planes other than the derivative pair; the other formulas unless
// `fp32_alternates`, and then from 1e6): those render in the plain form.
// The other formulas stay FP64 by default because their deep views hold
// long post-linear orbits (Julia near its parabolic-like points, burning
// ship's folds) that FP32 deltas cannot follow: against a direct mpmath
// iteration the FP64 form is right where the FP32 form is not.  Mandelbrot fields below 1e12 take
// the shallow mode: plain FP32 perturbation against the handle's orbit with
// unlimited rebasing, no series and no BLA.
bool make_floatexp_params(ReferenceContext& ctx, const Outputs& out, int width, int height, const char* zoom_text,
                          int max_iter, int series_order, int series_block, const FractalRenderOptions& o,
                          FxParams& p, bool fp32_alternates = false) {
    const fx::Fe zoom = parse_zoom_fe(zoom_text, ctx.precision_bits);
    const bool cycle = o.disable_cycle == 0 && (o.strict == 0 || o.strict_cycle != 0);
    if (cycle || o.time_budget_ms > 0 || out.p_iter || out.p_phase || out.p_t1 || out.p_t2) return false;
    if ((out.p_dex == nullptr) != (out.p_dey == nullptr)) return false;
    if (ctx.formula != kFormulaMandelbrot && (!fp32_alternates || fe_log10(zoom) < 6.0L)) return false;
    std::shared_ptr<DeviceTables> dev = device_tables(ctx);
    floatexp_tables(ctx, *dev);
    const DeepGeometry g = deep_geometry(zoom, width, height, o.coordinate_mode);
    std::memset(static_cast<void*>(&p), 0, sizeof p);  // padding too: the bytes key the graph cache
    p.formula = ctx.formula;
    p.de_x = out.p_dex;
    p.de_y = out.p_dey;
    p.pixel_spacing = f32x::n_norm(static_cast<float>(g.pixel_spacing.m), g.pixel_spacing.e);
    if (ctx.formula != kFormulaMandelbrot) {
        // Alternate-formula policy (render_alternate_reference_impl,
        // renderer.cpp:12116-12137): the 2x2 table whenever it exists, the
        // series only for Julia.
        p.orbit = dev->fx_orbit;
        p.orbit_size = dev->orbit_size;
        p.alt = dev->fx_alt;
        p.linear_index = dev->fx_index + 3;
        p.alt_start = ctx.alt_start;
        p.alt_input_radius2 = f32x::n_norm(static_cast<float>(ctx.alt_input_radius2.m), ctx.alt_input_radius2.e);
        p.parameter = f32x::norm(static_cast<float>(ctx.parameter.re), static_cast<float>(ctx.parameter.im),
                                 ctx.parameter.e);
        p.series = dev->fx_series;
        p.series_terms = dev->series_terms;
        p.series_iteration = ctx.series.iteration;
        p.series_on = ctx.formula == kFormulaJulia && ctx.series.enabled && ctx.series.iteration < max_iter
            && dev->series_terms > 1;
        p.series_r2 = f32x::n_norm(static_cast<float>(ctx.series.r2.m), ctx.series.r2.e);
        p.view_width = f32x::norm(static_cast<float>(g.view_width.m), 0.0f, g.view_width.e);
        p.view_height = f32x::norm(static_cast<float>(g.view_height.m), 0.0f, g.view_height.e);
        p.coordinate_mode = o.coordinate_mode;
        p.width = width;
        p.height = height;
        p.max_iter = max_iter;
        p.map_end = ctx.map_end;
        p.disable_bla = o.disable_bla != 0 || !p.alt ? 1 : 0;
        p.strict = o.strict;
        p.allow_recovery = o.allow_recovery;
        p.escape_mode = o.escape_radius_mode;
        p.max_lin_len = std::clamp(static_cast<int>(o.max_linear_bla_length), 2, kMaxSafeLinearBlaLength);
        p.output_bias = static_cast<float>(o.output_bias);
        p.out = out.field;
        p.counts = out.counts;
        return true;
    }
    if (fe_log10(zoom) < kShallowLog10Zoom) {
        if (dev->orbit_size < 2) return false;
        const double half_h = 0.5 * fx::scale2(g.view_height.m, g.view_height.e) + 0.05;
        const double half_w = 0.5 * fx::scale2(g.view_width.m, g.view_width.e) + 0.05;
        const double x = static_cast<double>(ctx.x_center), y = static_cast<double>(ctx.y_center);
        const bool cardioid = x + half_w >= -0.80 && x - half_w <= 0.40 && y + half_h >= -0.70 && y - half_h <= 0.70;
        const bool bulb = x + half_w >= -1.30 && x - half_w <= -0.70 && y + half_h >= -0.30 && y - half_h <= 0.30;
        p.orbit = dev->fx_orbit;
        p.orbit_size = dev->orbit_size;
        p.view_width = f32x::norm(static_cast<float>(g.view_width.m), 0.0f, g.view_width.e);
        p.view_height = f32x::norm(static_cast<float>(g.view_height.m), 0.0f, g.view_height.e);
        p.coordinate_mode = o.coordinate_mode;
        p.width = width;
        p.height = height;
        p.max_iter = max_iter;
        p.map_end = ctx.map_end;
        p.disable_bla = 1;
        p.strict = o.strict;
        p.escape_mode = o.escape_radius_mode;
        p.output_bias = static_cast<float>(o.output_bias);
        p.out = out.field;
        p.counts = out.counts;
        p.shallow = 1;
        p.interior_test = cardioid || bulb ? 1 : 0;
        p.centre_re = static_cast<float>(x);
        p.centre_im = static_cast<float>(y);
        return true;
    }
    const bool covers = fx::fe_cmp(g.current_input_radius, ctx.input_radius) <= 0;
    const bool use_deep = fx::fe_cmp(g.current_input_radius, ctx.deep_input_radius) <= 0;
    const bool use_ultra = fx::fe_cmp(g.current_input_radius, fx::fe_mul(ctx.input_radius, 1.0e-40)) <= 0;
    p.orbit = dev->fx_orbit;
    p.orbit_size = dev->orbit_size;
    p.cubic = dev->fx_cubic;
    p.cubic_index = dev->fx_index;
    p.linear = use_deep ? dev->fx_deep_linear : dev->fx_linear;
    p.linear_index = dev->fx_index + (use_deep ? 2 : 1);
    p.series = dev->fx_series;
    p.series_terms = dev->series_terms;
    p.series_iteration = ctx.series.iteration;
    p.series_on = ctx.series.enabled && ctx.series.order >= o.series_min_terms
        && ctx.series.order <= o.series_max_terms
        && fx::fe_cmp(g.current_input_radius, fx::fe_sqrt(ctx.series.r2)) <= 0
        && ctx.series.iteration < max_iter && dev->series_terms > 1;
    p.series_r2 = f32x::n_norm(static_cast<float>(ctx.series.r2.m), ctx.series.r2.e);
    p.view_width = f32x::norm(static_cast<float>(g.view_width.m), 0.0f, g.view_width.e);
    p.view_height = f32x::norm(static_cast<float>(g.view_height.m), 0.0f, g.view_height.e);
    p.coordinate_mode = o.coordinate_mode;
    p.width = width;
    p.height = height;
    p.max_iter = max_iter;
    p.map_end = ctx.map_end;
    p.disable_bla = (!covers || o.disable_bla != 0) ? 1 : 0;
    p.strict = o.strict;
    p.allow_recovery = o.allow_recovery;
    p.escape_mode = o.escape_radius_mode;
    p.max_bla_len = std::clamp(std::min(series_block, static_cast<int>(o.max_bla_length)), 2, kMaxSafeBlaLength);
    p.max_lin_len = std::clamp(std::min(series_block, static_cast<int>(o.max_linear_bla_length)), 2,
                               use_ultra ? kMaxSafeLinearBlaLength
                                         : (use_deep ? kMaxSafeDeepLinearBlaLength : kMaxSafeBlaLength));
    p.approx_order = std::clamp(series_order, 1, 3);
    p.output_bias = static_cast<float>(o.output_bias);
    p.out = out.field;
    p.counts = out.counts;
    return true;
}

}  // namespace

void render_floatexp_from_reference(ReferenceContext& ctx, const Outputs& out, int width, int height,
                                    const char* zoom_text, int max_iter, int series_order, int series_block,
                                    const FractalRenderOptions& o, ThreadRuntime& rt, cudaStream_t stream) {
    FxParams p;
    if (!make_floatexp_params(ctx, out, width, height, zoom_text, max_iter, series_order, series_block, o, p)) {
        render_from_reference(ctx, out, width, height, zoom_text, max_iter, series_order, series_block, o, false, rt,
                              stream);
        return;
    }
    p.series_scaled = static_cast<FxSeriesScaled*>(scratch(rt, kScratchSeries, sizeof(FxSeriesScaled)));
    check_cuda(launch_series_prologue(&p, 1, stream), "series prologue launch");
    check_cuda(launch_floatexp_mandelbrot(p, stream), "floatexp kernel launch");
}

namespace {

// Host-buffer wrapper: device scratch, kernel, copies back, stats.
void render_to_host(float* output, FractalRenderPlanes* planes, int width, int height,
                    const std::function<void(const Outputs&, bool, ThreadRuntime&, cudaStream_t)>& launch) {
    ThreadRuntime& rt = thread_runtime();
    wait_scratch(rt, rt.stream);
    const auto started = std::chrono::steady_clock::now();
    const std::size_t pixels = static_cast<std::size_t>(width) * static_cast<std::size_t>(height);
    Outputs out;
    out.field = static_cast<float*>(scratch(rt, kScratchField, pixels * sizeof(float)));
    if (planes) {
        out.p_iter = static_cast<std::int64_t*>(scratch(rt, kScratchPlaneIter, pixels * sizeof(std::int64_t)));
        out.p_phase = static_cast<double*>(scratch(rt, kScratchPhase, pixels * sizeof(double)));
        out.p_dex = static_cast<double*>(scratch(rt, kScratchDeX, pixels * sizeof(double)));
        out.p_dey = static_cast<double*>(scratch(rt, kScratchDeY, pixels * sizeof(double)));
        out.p_t1 = static_cast<double*>(scratch(rt, kScratchTest1, pixels * sizeof(double)));
        out.p_t2 = static_cast<double*>(scratch(rt, kScratchTest2, pixels * sizeof(double)));
    }
    const bool collect = stats_enabled.load(std::memory_order_relaxed);
    if (collect) check_cuda(cudaMemsetAsync(rt.stats, 0, sizeof(unsigned long long) * kStatsSlots, rt.stream), "stats reset");
    check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
    launch(out, collect, rt, rt.stream);
    check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
    check_cuda(cudaMemcpyAsync(output, out.field, pixels * sizeof(float), cudaMemcpyDeviceToHost, rt.stream),
               "copy field to host");
    if (planes) {
        check_cuda(cudaMemcpyAsync(planes->orbit_iteration, out.p_iter, pixels * sizeof(std::int64_t),
                                   cudaMemcpyDeviceToHost, rt.stream), "copy planes");
        check_cuda(cudaMemcpyAsync(planes->phase, out.p_phase, pixels * sizeof(double), cudaMemcpyDeviceToHost,
                                   rt.stream), "copy planes");
        check_cuda(cudaMemcpyAsync(planes->de_x, out.p_dex, pixels * sizeof(double), cudaMemcpyDeviceToHost,
                                   rt.stream), "copy planes");
        check_cuda(cudaMemcpyAsync(planes->de_y, out.p_dey, pixels * sizeof(double), cudaMemcpyDeviceToHost,
                                   rt.stream), "copy planes");
        check_cuda(cudaMemcpyAsync(planes->test1, out.p_t1, pixels * sizeof(double), cudaMemcpyDeviceToHost,
                                   rt.stream), "copy planes");
        check_cuda(cudaMemcpyAsync(planes->test2, out.p_t2, pixels * sizeof(double), cudaMemcpyDeviceToHost,
                                   rt.stream), "copy planes");
    }
    std::array<unsigned long long, kStatsSlots> stats{};
    if (collect) {
        check_cuda(cudaMemcpyAsync(stats.data(), rt.stats, sizeof(unsigned long long) * kStatsSlots,
                                   cudaMemcpyDeviceToHost, rt.stream), "copy stats");
    }
    check_cuda(cudaStreamSynchronize(rt.stream), "render");
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    if (collect) {
        stats[22] = static_cast<unsigned long long>(  // render_ns
            std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - started).count());
        publish_stats(stats);
    }
}

std::string julia_text(double value) {
    char buffer[64];
    if (std::snprintf(buffer, sizeof buffer, "%.17g", value) < 0) throw Failure{"failed to format the Julia constant"};
    return buffer;
}

template <typename F>
int guarded(const char* unknown, F&& body) {
    try {
        body();
        set_error("");
        return 0;
    } catch (const Failure& failure) {
        set_error(failure.message);
        return 1;
    } catch (const std::exception& error) {
        set_error(error.what());
        return 1;
    } catch (...) {
        set_error(unknown);
        return 1;
    }
}

template <typename F>
void* guarded_handle(const char* unknown, F&& body) {
    try {
        void* handle = body();
        set_error("");
        return handle;
    } catch (const Failure& failure) {
        set_error(failure.message);
    } catch (const std::exception& error) {
        set_error(error.what());
    } catch (...) {
        set_error(unknown);
    }
    return nullptr;
}

void* create_handle(const char* x, const char* y, const char* zoom, int max_iter, int precision_bits,
                    int series_order, bool retain, int formula, const char* jr, const char* ji,
                    const FractalRenderOptions* supplied, const char* invalid_message) {
    if (!x || !y || !zoom || !jr || !ji || !valid_iterations(max_iter) || !valid_precision(precision_bits)
        || !valid_series(series_order, 2) || !valid_formula(formula)) {
        throw Failure{invalid_message};
    }
    const FractalRenderOptions o = checked_options(supplied);
    auto context = create_reference_context(x, y, zoom, max_iter, precision_bits, series_order, retain, formula,
                                            jr, ji, o.escape_radius_mode, o.coordinate_mode);
    return register_reference(std::move(context));
}

}  // namespace

// ---------------------------------------------------------- aurora palette
// aurora_palette_for / colour_basis_for (renderer.cpp:4788-4923), built on
// the host exactly as the reference does and cached per thread.
namespace {

struct AuroraCache {
    int max_iter = -1;
    double phase = 0, vocal = 0, pitch = 0;
    bool accented = false;
    std::array<std::uint8_t, 9> accents{};
    std::vector<std::uint8_t> rgb;
    int device = -1;
    std::uint8_t* device_lut = nullptr;
    std::size_t device_capacity = 0;
};

std::uint8_t colour_byte(double value) { return static_cast<std::uint8_t>(std::clamp(value, 0.0, 255.0)); }

// aurora_palette_for (renderer.cpp:4841-4923); with `accents` (three RGB
// triples) the three waves are projected through the accents before the hue
// rotation.
void build_aurora(AuroraCache& cache, int max_iter, double phase, double vocal, double pitch,
                  const std::uint8_t* accents) {
    const int size = std::min(65536, std::max(4096, max_iter * 4));
    std::vector<float> cosine(static_cast<std::size_t>(size)), sine(static_cast<std::size_t>(size));
    const double denominator = std::max(1, size - 1);
    for (int i = 0; i < size; ++i) {
        const double angle = 0.15 * static_cast<double>(max_iter) * static_cast<double>(i) / denominator;
        cosine[static_cast<std::size_t>(i)] = static_cast<float>(std::cos(angle));
        sine[static_cast<std::size_t>(i)] = static_cast<float>(std::sin(angle));
    }
    const double mix = std::clamp(vocal, 0.0, 1.0);
    const double split = 5.0 * mix * mix;
    const double rc = std::cos(phase), rs = std::sin(phase);
    const double gc = std::cos(phase + split * 0.4), gs = std::sin(phase + split * 0.4);
    const double bc = std::cos(phase + split), bs = std::sin(phase + split);
    const double two_pi = 6.283185307179586476925286766559005768;
    const double signed_pitch = std::clamp(2.0 * (pitch - 0.5), -1.0, 1.0);
    const double hue = signed_pitch * 0.16 * two_pi;
    const bool rotate = std::abs(hue) > 1.0e-15;
    const double hcos = rotate ? std::cos(hue) : 1.0;
    const double hsin = rotate ? std::sin(hue) : 0.0;
    cache.rgb.resize(static_cast<std::size_t>(size) * 3);
    for (int i = 0; i < size; ++i) {
        const double c = cosine[static_cast<std::size_t>(i)];
        const double s = sine[static_cast<std::size_t>(i)];
        double r = (0.5 - 0.5 * (c * rc + s * rs)) * 140.0;
        double g = (0.5 - 0.5 * (c * gc + s * gs)) * 140.0;
        double b = (0.5 - 0.5 * (c * bc + s * bs)) * 140.0;
        if (accents != nullptr) {
            const double wr = std::clamp(static_cast<double>(colour_byte(r)) / 140.0, 0.0, 1.0);
            const double wg = std::clamp(static_cast<double>(colour_byte(g)) / 140.0, 0.0, 1.0);
            const double wb = std::clamp(static_cast<double>(colour_byte(b)) / 140.0, 0.0, 1.0);
            const double ar = (wr * static_cast<double>(accents[0]) + wg * static_cast<double>(accents[3])
                               + wb * static_cast<double>(accents[6])) / 1.8;
            const double ag = (wr * static_cast<double>(accents[1]) + wg * static_cast<double>(accents[4])
                               + wb * static_cast<double>(accents[7])) / 1.8;
            const double ab = (wr * static_cast<double>(accents[2]) + wg * static_cast<double>(accents[5])
                               + wb * static_cast<double>(accents[8])) / 1.8;
            r = ar;
            g = ag;
            b = ab;
        }
        if (rotate) {
            // Chroma rotation in YIQ (renderer.cpp:4815-4833).
            const double y = 0.299 * r + 0.587 * g + 0.114 * b;
            const double ii = 0.596 * r - 0.275 * g - 0.321 * b;
            const double q = 0.212 * r - 0.523 * g + 0.311 * b;
            const double ri = ii * hcos - q * hsin;
            const double rq = ii * hsin + q * hcos;
            const double nr = y + 0.956 * ri + 0.621 * rq;
            const double ng = y - 0.272 * ri - 0.647 * rq;
            const double nb = y - 1.106 * ri + 1.703 * rq;
            r = nr;
            g = ng;
            b = nb;
        }
        cache.rgb[3 * static_cast<std::size_t>(i)] = colour_byte(r);
        cache.rgb[3 * static_cast<std::size_t>(i) + 1] = colour_byte(g);
        cache.rgb[3 * static_cast<std::size_t>(i) + 2] = colour_byte(b);
    }
    cache.max_iter = max_iter;
    cache.phase = phase;
    cache.vocal = vocal;
    cache.pitch = pitch;
    cache.accented = accents != nullptr;
    if (accents != nullptr) std::copy(accents, accents + 9, cache.accents.begin());
}

// Returns the device LUT for the parameters; uploads when they change.
const std::uint8_t* aurora_lut(ThreadRuntime& rt, int max_iter, double phase, double vocal, double pitch,
                               int& size, const std::uint8_t* accents = nullptr) {
    thread_local AuroraCache cache;
    const bool same = cache.max_iter == max_iter && cache.phase == phase && cache.vocal == vocal
        && cache.pitch == pitch && !cache.rgb.empty() && cache.accented == (accents != nullptr)
        && (accents == nullptr || std::equal(accents, accents + 9, cache.accents.begin()));
    if (!same) build_aurora(cache, max_iter, phase, vocal, pitch, accents);
    size = static_cast<int>(cache.rgb.size() / 3);
    if (!same || cache.device != rt.device || cache.device_lut == nullptr) {
        std::uint8_t* lut = static_cast<std::uint8_t*>(scratch(rt, kScratchLut, cache.rgb.size()));
        check_cuda(cudaMemcpyAsync(lut, cache.rgb.data(), cache.rgb.size(), cudaMemcpyHostToDevice, rt.stream),
                   "upload aurora LUT");
        check_cuda(cudaStreamSynchronize(rt.stream), "upload aurora LUT");
        cache.device_lut = lut;
        cache.device = rt.device;
    }
    return cache.device_lut;
}

bool valid_colour_controls(double a, double b, double c, double d) {
    return std::isfinite(a) && std::isfinite(b) && std::isfinite(c) && std::isfinite(d);
}

}  // namespace

// ------------------------------------------------------------------ KFP
namespace {

// valid_kfp_options (renderer.cpp:7396-7454).
bool valid_kfp(const FractalKfpOptions* o, int lut_size) {
    const std::uint32_t legacy = static_cast<std::uint32_t>(offsetof(FractalKfpOptions, show_glitches));
    if (!o || o->struct_size < legacy || o->version != FRACTAL_KFP_OPTIONS_VERSION || lut_size < 2 || lut_size > 65536
        || !std::isfinite(o->iter_div) || o->iter_div <= 0.0 || !std::isfinite(o->color_offset)
        || !std::isfinite(o->ratio) || o->color_method < 0 || o->color_method > 11 || o->smooth_method < 0
        || o->smooth_method > 2 || o->smooth < 0 || o->smooth > 1 || o->flat < 0 || o->flat > 1
        || o->inverse_transition < 0 || o->inverse_transition > 1 || !std::isfinite(o->phase_color_strength)
        || o->multi_color < 0 || o->multi_color > 1 || o->blend_multi_color < 0 || o->blend_multi_color > 1
        || o->multi_color_count > FRACTAL_KFP_MAX_MULTI_COLORS || !std::isfinite(o->power) || o->power <= 0.0
        || o->slopes < 0 || o->slopes > 1 || !std::isfinite(o->slope_power) || o->slope_power < 0.0
        || !std::isfinite(o->slope_ratio) || o->slope_ratio < 0.0 || !std::isfinite(o->slope_angle)
        || o->differences < 0 || o->differences > 7 || !std::isfinite(o->field_bias) || o->field_bias < 0.0
        || o->bailout_radius_preset < 0 || o->bailout_radius_preset > 3 || !std::isfinite(o->bailout_radius_custom)
        || o->bailout_radius_custom <= 0.0 || o->bailout_norm_preset < 0 || o->bailout_norm_preset > 3
        || !std::isfinite(o->bailout_norm_custom) || o->bailout_norm_custom <= 0.0 || o->texture_enabled < 0
        || o->texture_enabled > 1 || !std::isfinite(o->texture_merge) || !std::isfinite(o->texture_power)
        || !std::isfinite(o->texture_ratio) || o->texture_resize < 0 || o->texture_resize > 1 || o->use_opengl < 0
        || o->use_opengl > 1 || o->use_srgb < 0 || o->use_srgb > 1) {
        return false;
    }
    if (o->struct_size >= legacy + sizeof(o->show_glitches) && (o->show_glitches < 0 || o->show_glitches > 1)) {
        return false;
    }
    for (std::uint32_t i = 0; i < o->multi_color_count; ++i) {
        if (!std::isfinite(o->multi_color_period[i]) || o->multi_color_period[i] == 0.0
            || o->multi_color_type[i] < 0 || o->multi_color_type[i] > 2) {
            return false;
        }
    }
    for (int c = 0; c < 3; ++c) {
        if (o->interior_color[c] < 0 || o->interior_color[c] > 255) return false;
    }
    return true;
}

// kfp_smooth_offset (renderer.cpp:5398-5421).
double kfp_smooth_offset(const FractalKfpOptions& o) {
    if (o.smooth_method != 0 || !std::isfinite(o.power) || o.power <= 0.0 || std::abs(o.power - 1.0) < 1.0e-12) {
        return 0.0;
    }
    double radius = 10000.0;
    switch (o.bailout_radius_preset) {
        case 0: radius = 10000.0; break;
        case 1: radius = 2.0; break;
        case 2: radius = std::pow(2.0, 1.0 / (o.power - 1.0)); break;
        case 3: radius = o.bailout_radius_custom; break;
        default: return 0.0;
    }
    if (!std::isfinite(radius) || radius <= 1.0) return 0.0;
    return std::log(std::log(radius)) / std::log(o.power);
}

struct KfpDeviceInputs {
    const std::uint8_t* lut = nullptr;
    const double* period = nullptr;
    const int* type = nullptr;
};

// Uploads the LUT and multi-colour waves into the thread's scratch.  The
// upload is skipped when the same waves (and, for a host LUT, the same LUT
// bytes) already sit in the same scratch buffer; `uploaded` reports whether
// copies were enqueued on the thread stream.
KfpDeviceInputs kfp_inputs(ThreadRuntime& rt, const FractalKfpOptions& o, const std::uint8_t* lut, int lut_size,
                           bool lut_on_device, bool* uploaded = nullptr) {
    struct Cached {
        const void* base = nullptr;
        std::vector<double> period;
        std::vector<int> type;
        std::vector<std::uint8_t> lut;
        bool host_lut = false;
    };
    thread_local Cached cached;
    KfpDeviceInputs in;
    // Layout: [LUT padded to 16 B][256 wave periods][256 wave types].
    const std::size_t lut_bytes = static_cast<std::size_t>(lut_size) * 3;
    const std::size_t lut_padded = (lut_bytes + 15) / 16 * 16;
    const std::size_t waves = o.multi_color_count;
    char* base = static_cast<char*>(scratch(rt, kScratchKfpAux,
                                            lut_padded + FRACTAL_KFP_MAX_MULTI_COLORS * (sizeof(double) + sizeof(int))));
    std::uint8_t* lut_copy = reinterpret_cast<std::uint8_t*>(base);
    double* period = reinterpret_cast<double*>(base + lut_padded);
    int* type = reinterpret_cast<int*>(base + lut_padded + FRACTAL_KFP_MAX_MULTI_COLORS * sizeof(double));
    const bool same_waves = cached.base == base && cached.period.size() == waves
        && std::equal(o.multi_color_period, o.multi_color_period + waves, cached.period.begin())
        && std::equal(o.multi_color_type, o.multi_color_type + waves, cached.type.begin());
    const bool same_lut = lut_on_device
        || (cached.base == base && cached.host_lut && cached.lut.size() == lut_bytes
            && std::equal(lut, lut + lut_bytes, cached.lut.begin()));
    bool copied = false;
    if (!same_waves) {
        if (waves > 0) {
            check_cuda(cudaMemcpyAsync(period, o.multi_color_period, waves * sizeof(double), cudaMemcpyHostToDevice,
                                       rt.stream), "upload KFP waves");
            check_cuda(cudaMemcpyAsync(type, o.multi_color_type, waves * sizeof(int), cudaMemcpyHostToDevice,
                                       rt.stream), "upload KFP waves");
            copied = true;
        }
        cached.period.assign(o.multi_color_period, o.multi_color_period + waves);
        cached.type.assign(o.multi_color_type, o.multi_color_type + waves);
    }
    if (lut_on_device) {
        in.lut = lut;
    } else {
        if (!same_lut) {
            check_cuda(cudaMemcpyAsync(lut_copy, lut, lut_bytes, cudaMemcpyHostToDevice, rt.stream),
                       "upload KFP LUT");
            cached.lut.assign(lut, lut + lut_bytes);
            cached.host_lut = true;
            copied = true;
        }
        in.lut = lut_copy;
    }
    if (lut_on_device) cached.host_lut = cached.host_lut && same_lut;
    cached.base = base;
    in.period = period;
    in.type = type;
    if (uploaded) *uploaded = copied;
    return in;
}

// The per-pass constants of write_kfp_pixel for a width x height field.
KfpLaunch kfp_constants(const FractalKfpOptions& o, int width, int height, int max_iter, int lut_size) {
    KfpLaunch k{};
    k.width = width;
    k.height = height;
    k.max_iter = max_iter;
    k.field_bias = o.field_bias;
    k.smooth_offset = kfp_smooth_offset(o);
    k.color_method = o.color_method;
    k.differences = o.differences;
    k.smooth = o.smooth;
    k.flat = o.flat;
    k.inverse_transition = o.inverse_transition;
    k.needs_difference = o.color_method >= 5 && o.color_method <= 8;
    k.needs_slopes = o.slopes && o.slope_power > 0.0 && o.slope_ratio > 0.0;
    k.iter_div = o.iter_div;
    k.color_offset = o.color_offset;
    k.transfer_min = 0.0;
    k.transfer_max = 1.0;
    k.multi_color = o.multi_color;
    k.blend_multi_color = o.blend_multi_color;
    k.multi_count = static_cast<int>(o.multi_color_count);
    if (o.slopes) {
        const double angle = o.slope_angle * 3.14159265358979323846 / 180.0;
        k.slope_cos = std::cos(angle);
        k.slope_sin = std::sin(angle);
    } else {
        k.slope_cos = 1.0;
        k.slope_sin = 0.0;
    }
    k.slope_power = o.slope_power;
    k.slope_ratio = o.slope_ratio;
    for (int c = 0; c < 3; ++c) k.interior[c] = o.interior_color[c];
    k.lut_size = lut_size;
    return k;
}

// ColorMethod 4's transfer bounds (kfp_transfer_bounds, renderer.cpp:
// 7296-7393) of a scalar field or of plane samples, read back to the host;
// (0, 1) when no pixel qualifies.
void kfp_transfer_bounds(ThreadRuntime& rt, const float* d_field, long long pixels, int max_iter,
                         const FractalKfpOptions& o, double smooth_offset, cudaStream_t stream, double& minimum,
                         double& maximum, const void* samples = nullptr, const std::uint8_t* flags = nullptr) {
    unsigned long long* bounds = static_cast<unsigned long long*>(scratch(rt, kScratchWork, 16));
    if (samples != nullptr) {
        check_cuda(launch_kfp_plane_bounds(samples, flags, pixels, max_iter, bounds, stream), "KFP plane bounds launch");
    } else {
        check_cuda(launch_kfp_bounds(d_field, pixels, max_iter, o.field_bias, smooth_offset, bounds, stream),
                   "KFP bounds launch");
    }
    unsigned long long host[2];
    check_cuda(cudaMemcpyAsync(host, bounds, sizeof host, cudaMemcpyDeviceToHost, stream), "KFP bounds");
    check_cuda(cudaStreamSynchronize(stream), "KFP bounds");
    auto unorder = [](unsigned long long v) {
        const unsigned long long bits = (v & 0x8000000000000000ull) ? (v & 0x7fffffffffffffffull) : ~v;
        double d;
        std::memcpy(&d, &bits, sizeof d);
        return d;
    };
    minimum = 0.0;
    maximum = 1.0;
    if (host[0] != ~0ull && host[1] != 0ull) {
        minimum = unorder(host[0]);
        maximum = unorder(host[1]);
    }
}

// Resolves the per-pass constants and launches (write_kfp_pixel inputs).
void kfp_colour(const float* d_field, std::uint8_t* d_rgb, int width, int height, int max_iter,
                const FractalKfpOptions& o, const KfpDeviceInputs& in, int lut_size, ThreadRuntime& rt,
                cudaStream_t stream, const KfpPlanesLaunch* planes = nullptr, const void* samples = nullptr,
                const std::uint8_t* flags = nullptr) {
    KfpLaunch k = kfp_constants(o, width, height, max_iter, lut_size);
    if (o.color_method == 4) {
        const bool plane_samples = planes != nullptr && planes->has_iteration;
        kfp_transfer_bounds(rt, d_field, static_cast<long long>(width) * height, max_iter, o, k.smooth_offset, stream,
                            k.transfer_min, k.transfer_max, plane_samples ? samples : nullptr,
                            plane_samples ? flags : nullptr);
    }
    check_cuda(launch_kfp(d_field, d_rgb, k, in.lut, in.period, in.type, stream, planes, samples, flags),
               "KFP kernel launch");
}

// kfp_selected_bailout_radius / _norm (renderer.cpp:5672-5716).
double kfp_bailout_radius(const FractalKfpOptions& o) {
    double radius = 10000.0;
    switch (o.bailout_radius_preset) {
        case 0: radius = 10000.0; break;
        case 1: radius = 2.0; break;
        case 2:
            if (o.power > 1.0 && std::isfinite(o.power)) {
                radius = std::pow(2.0, 1.0 / (o.power - 1.0));
            } else {
                return 0.0;
            }
            break;
        case 3: radius = o.bailout_radius_custom; break;
        default: return 0.0;
    }
    return std::isfinite(radius) && radius > 1.0 ? radius : 0.0;
}

double kfp_bailout_norm(const FractalKfpOptions& o) {
    switch (o.bailout_norm_preset) {
        case 0: return 1.0;
        case 1: return 2.0;
        case 2: return std::numeric_limits<double>::infinity();
        case 3: return std::isfinite(o.bailout_norm_custom) && o.bailout_norm_custom > 0.0 ? o.bailout_norm_custom : 0.0;
        default: return 0.0;
    }
}


int kfp_host(const float* field, uint8_t* output, int width, int height, int max_iter, double phase, double vocal,
             double instrumental, double pitch, const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
             int threads) {
    return guarded("native KFP colouriser failed with an unknown exception", [&] {
        if (!field || !output || !valid_dims(width, height) || !valid_iterations(max_iter) || !valid_threads(threads)
            || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut || !valid_kfp(options, lut_size)) {
            throw Failure{"invalid native KFP colour dimensions or controls"};
        }
        if (options->field_bias > static_cast<double>(max_iter)) {
            throw Failure{"native KFP field bias exceeds iteration cap"};
        }
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        const std::size_t pixels = static_cast<std::size_t>(width) * static_cast<std::size_t>(height);
        float* d_field = static_cast<float*>(scratch(rt, kScratchField, pixels * sizeof(float)));
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, *options, lut, lut_size, false);
        check_cuda(cudaMemcpyAsync(d_field, field, pixels * sizeof(float), cudaMemcpyHostToDevice, rt.stream),
                   "copy field to device");
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        kfp_colour(d_field, d_rgb, width, height, max_iter, *options, in, lut_size, rt, rt.stream);
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream), "copy RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "KFP colour");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

// kfp_pixel_context (renderer.cpp:5723-5763) for planes whose device
// pointers are already in `pl`.
void plane_context(KfpPlanesLaunch& pl, const FractalKfpOptions& o) {
    pl.has_iteration = pl.orbit_iteration != nullptr || pl.iteration != nullptr;
    const std::uint32_t glitch_field = static_cast<std::uint32_t>(offsetof(FractalKfpOptions, show_glitches));
    pl.show_glitches = o.struct_size < glitch_field + sizeof(o.show_glitches) ? 1 : (o.show_glitches != 0);
    pl.analytic = o.differences == 7 && pl.de_x != nullptr && pl.de_y != nullptr;
    pl.smooth_method = o.smooth_method;
    pl.has_constant_bailout = pl.bailout == nullptr;
    pl.smooth_bailout_radius = kfp_bailout_radius(o);
    pl.power = o.power;
    if (std::isfinite(o.power) && o.power > 1.0) {
        pl.smooth_power_log = std::log(o.power);
        pl.has_smooth_power_log = std::isfinite(pl.smooth_power_log) && pl.smooth_power_log != 0.0;
    }
    if (pl.has_constant_bailout && pl.smooth_bailout_radius > 1.0 && std::isfinite(pl.smooth_bailout_radius)) {
        pl.smooth_bailout_log = std::log(pl.smooth_bailout_radius);
        pl.has_smooth_bailout_log = std::isfinite(pl.smooth_bailout_log) && pl.smooth_bailout_log != 0.0;
    }
    const double norm = kfp_bailout_norm(o);
    if (norm > 0.0 && std::isfinite(norm)) {
        pl.smooth_norm_exponent = 1.0 / norm;
        pl.has_smooth_norm_exponent = 1;
    } else if (std::isinf(norm) && norm > 0.0) {
        pl.smooth_norm_exponent = 1.0;
        pl.has_smooth_norm_exponent = 1;
    }
    pl.phase_scale = o.phase_color_strength / 100.0 * 1024.0;
    pl.smooth_power_ok = std::isfinite(o.power) && o.power > 1.0;
    pl.smooth_power_log_f = static_cast<float>(pl.has_smooth_power_log ? pl.smooth_power_log : 0.0);
    pl.smooth_radius_ok = std::isfinite(pl.smooth_bailout_radius) && pl.smooth_bailout_radius > 1.0;
    pl.smooth_radius_log_f = static_cast<float>(pl.smooth_radius_ok ? std::log(pl.smooth_bailout_radius) : 0.0);
}

// Bytes of a texture the merge can address: (height - 1) strides plus one row.
std::size_t texture_bytes(const FractalKfpPlanes& planes) {
    return static_cast<std::size_t>(planes.texture_height - 1) * static_cast<std::size_t>(planes.texture_stride)
        + static_cast<std::size_t>(planes.texture_width) * 3;
}

// SetTexture's constants (renderer.cpp:7191-7226) for a texture on the device.
void attach_texture(KfpPlanesLaunch& pl, const FractalKfpPlanes& planes, const FractalKfpOptions& o,
                    const void* d_texture) {
    pl.texture = static_cast<const std::uint8_t*>(d_texture);
    pl.texture_active = 1;
    pl.texture_width = planes.texture_width;
    pl.texture_height = planes.texture_height;
    pl.texture_stride = planes.texture_stride;
    pl.texture_power = o.texture_power;
    pl.texture_ratio = o.texture_ratio;
    pl.texture_merge = o.texture_merge;
    pl.image_offset = std::isfinite(o.texture_power)
        ? static_cast<int>(std::clamp(o.texture_power / 64.0, static_cast<double>(std::numeric_limits<int>::min()),
                                      static_cast<double>(std::numeric_limits<int>::max())))
        : 0;
}

// valid_kfp_planes (renderer.cpp:7467-7491).
bool valid_kfp_planes(const FractalKfpPlanes* planes, int width, int height) {
    if (planes == nullptr) return true;
    if (planes->struct_size < sizeof(FractalKfpPlanes) || planes->version != FRACTAL_KFP_PLANES_VERSION) return false;
    if (planes->texture_rgb == nullptr) {
        return planes->texture_width == 0 && planes->texture_height == 0 && planes->texture_stride == 0;
    }
    if (planes->texture_width <= 0 || planes->texture_height <= 0
        || static_cast<long long>(planes->texture_stride) < static_cast<long long>(planes->texture_width) * 3) {
        return false;
    }
    const unsigned long long bytes = static_cast<unsigned long long>(planes->texture_stride)
        * static_cast<unsigned long long>(planes->texture_height);
    return bytes <= static_cast<unsigned long long>(kMaxPixels) * 3ull && valid_dims(width, height);
}

// fractal_colourise_kfp_planes (renderer.cpp:16729-16748 through
// fractal_colourise_kfp_impl, 16314-16545): the planes copied to the device,
// the pixel context resolved here, one samples pass, then the KFP pass.
int kfp_planes_host(const float* field, uint8_t* output, int width, int height, int max_iter, double phase,
                    double vocal, double instrumental, double pitch, const FractalKfpOptions* options,
                    const FractalKfpPlanes* planes, const uint8_t* lut, int lut_size, int threads) {
    return guarded("native KFP colouriser failed with an unknown exception", [&] {
        const bool planes_ok = valid_kfp_planes(planes, width, height);
        if (!field || !output || !valid_dims(width, height) || !valid_iterations(max_iter) || !valid_threads(threads)
            || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut || !valid_kfp(options, lut_size)
            || !planes_ok) {
            throw Failure{"invalid native KFP colour dimensions or controls"};
        }
        if (options->field_bias > static_cast<double>(max_iter)) {
            throw Failure{"native KFP field bias exceeds iteration cap"};
        }
        const FractalKfpOptions& o = *options;
        if (planes == nullptr) {
            if (kfp_host(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, options, lut,
                         lut_size, threads) != 0) {
                throw Failure{last_error};
            }
            return;
        }
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        const std::size_t pixels = static_cast<std::size_t>(width) * static_cast<std::size_t>(height);
        // Device layout: field, then each present plane, then samples and flags.
        const void* host_arrays[9] = {planes->orbit_iteration, planes->bailout, planes->iteration, planes->transition,
                                      planes->phase, planes->de_x, planes->de_y, planes->test1, planes->test2};
        auto up = [](std::size_t v) { return (v + 255) / 256 * 256; };
        const bool texture = planes->texture_rgb != nullptr && o.texture_enabled != 0;
        const std::size_t texture_size = texture ? texture_bytes(*planes) : 0;
        std::size_t total = up(pixels * sizeof(float)) + up(pixels * 8) + up(pixels) + up(texture_size);
        for (const void* a : host_arrays) total += a ? up(pixels * 8) : 0;
        char* base = static_cast<char*>(scratch(rt, kScratchPlanesIn, total));
        std::size_t at = 0;
        auto put = [&](const void* data, std::size_t bytes) -> void* {
            void* dst = base + at;
            if (data) check_cuda(cudaMemcpyAsync(dst, data, bytes, cudaMemcpyHostToDevice, rt.stream), "upload planes");
            at += up(bytes);
            return dst;
        };
        float* d_field = static_cast<float*>(put(field, pixels * sizeof(float)));
        const void* d_arrays[9];
        for (int a = 0; a < 9; ++a) d_arrays[a] = host_arrays[a] ? put(host_arrays[a], pixels * 8) : nullptr;
        void* samples = put(nullptr, pixels * 8);
        std::uint8_t* flags = static_cast<std::uint8_t*>(put(nullptr, pixels));
        const void* d_texture = texture ? put(planes->texture_rgb, texture_size) : nullptr;
        KfpPlanesLaunch pl{};
        if (texture) attach_texture(pl, *planes, o, d_texture);
        pl.orbit_iteration = static_cast<const long long*>(d_arrays[0]);
        pl.bailout = static_cast<const double*>(d_arrays[1]);
        pl.iteration = static_cast<const long long*>(d_arrays[2]);
        pl.transition = static_cast<const double*>(d_arrays[3]);
        pl.phase = static_cast<const double*>(d_arrays[4]);
        pl.de_x = static_cast<const double*>(d_arrays[5]);
        pl.de_y = static_cast<const double*>(d_arrays[6]);
        pl.test1 = static_cast<const double*>(d_arrays[7]);
        pl.test2 = static_cast<const double*>(d_arrays[8]);
        plane_context(pl, o);
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, o, lut, lut_size, false);
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        if (pl.has_iteration) {
            check_cuda(launch_kfp_plane_samples(pl, max_iter, static_cast<long long>(pixels), samples, flags,
                                                rt.stream), "KFP plane samples launch");
        }
        kfp_colour(d_field, d_rgb, width, height, max_iter, o, in, lut_size, rt, rt.stream, &pl, samples, flags);
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream), "copy RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "KFP plane colour");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

}  // namespace

}  // namespace fgb

using namespace fgb;


// ------------------------------------------------------------ atlas frames
namespace {

// launch_atlas, remembering the frame's exact-pass counter for
// fractal_gb300_atlas_last_exact_pixels.
cudaError_t run_atlas(ThreadRuntime& rt, AtlasLaunch& a, void* tables, cudaStream_t stream) {
    const cudaError_t status = launch_atlas(a, tables, stream);
    rt.atlas_exact_count = a.exact_count;
    return status;
}

// Validated arguments of one atlas frame: geometry and numbers for
// launch_atlas, sources and outputs left to the caller.
struct AtlasRequest {
    int parent_width, parent_height, parent_max_iter;
    int child_width, child_height, child_max_iter;
    bool has_child;
    int out_width, out_height;
    double parent_zoom, child_fraction;
    int palette_max_iter;
};

AtlasLaunch atlas_geometry(const AtlasRequest& r) {
    AtlasLaunch a{};
    a.parent_width = r.parent_width;
    a.parent_height = r.parent_height;
    a.parent_max_iter = r.parent_max_iter;
    a.parent_zoom = r.parent_zoom;
    a.child_width = r.child_width;
    a.child_height = r.child_height;
    a.child_max_iter = r.child_max_iter;
    a.child_zoom = 1.0;
    a.out_width = r.out_width;
    a.out_height = r.out_height;
    const bool use_child = r.has_child && r.child_fraction > 0.0;
    a.use_child = use_child;
    a.full_child = use_child && r.child_fraction >= 0.999999;
    if (use_child) {
        a.child_visible_width = std::max(1, static_cast<int>(std::lround(static_cast<double>(r.out_width)
                                                                         * r.child_fraction)));
        a.child_visible_height = std::max(1, static_cast<int>(std::lround(static_cast<double>(r.out_height)
                                                                          * r.child_fraction)));
    }
    a.child_left = (r.out_width - a.child_visible_width) / 2;
    a.child_top = (r.out_height - a.child_visible_height) / 2;
    return a;
}

void check_atlas_common(const AtlasRequest& r) {
    if (!valid_dims(r.parent_width, r.parent_height) || !valid_dims(r.out_width, r.out_height)
        || !valid_iterations(r.parent_max_iter) || !std::isfinite(r.parent_zoom) || r.parent_zoom <= 0.0
        || !std::isfinite(r.child_fraction) || r.child_fraction < 0.0 || r.child_fraction > 1.0) {
        throw Failure{""};
    }
}

// fractal_atlas_field_ex's checks and frame constants (renderer.cpp:
// 18720-18770).
AtlasLaunch atlas_field_launch(const AtlasRequest& r, double child_zoom, double parent_bias, double child_bias,
                               double output_bias, int feather) {
    const char* invalid = "invalid native scalar atlas dimensions";
    try {
        check_atlas_common(r);
    } catch (const Failure&) {
        throw Failure{invalid};
    }
    if (!std::isfinite(child_zoom) || child_zoom <= 0.0 || !std::isfinite(parent_bias) || parent_bias < 0.0
        || parent_bias > static_cast<double>(r.parent_max_iter) || !std::isfinite(child_bias) || child_bias < 0.0
        || !std::isfinite(output_bias) || output_bias < 0.0 || feather < 0 || !valid_iterations(r.palette_max_iter)) {
        throw Failure{invalid};
    }
    AtlasLaunch a = atlas_geometry(r);
    a.mode = kAtlasField;
    if (a.use_child && (!valid_dims(r.child_width, r.child_height) || !valid_iterations(r.child_max_iter)
                        || child_bias > static_cast<double>(r.child_max_iter))) {
        throw Failure{"invalid native scalar atlas child tile"};
    }
    const int effective = std::max(r.palette_max_iter, std::max(r.parent_max_iter, a.use_child ? r.child_max_iter : 0));
    if (!valid_iterations(effective) || output_bias > static_cast<double>(effective)) {
        throw Failure{"invalid native scalar atlas iteration cap"};
    }
    a.parent_bias = parent_bias;
    a.child_bias = child_bias;
    a.child_zoom = std::max(child_zoom, 1.0);
    a.output_bias = output_bias;
    a.effective_iter = effective;
    a.feather = a.use_child && !a.full_child
        ? std::min(feather, std::min(a.child_visible_width / 2, a.child_visible_height / 2)) : 0;
    return a;
}

// atlas_colourise_impl's checks and frame constants (renderer.cpp:
// 19162-19215); the aurora table is uploaded by the caller.
AtlasLaunch atlas_colour_launch(const AtlasRequest& r, double phase, double vocal, double instrumental, double pitch,
                                const int* interior_color) {
    const char* invalid = "invalid native atlas dimensions or controls";
    try {
        check_atlas_common(r);
    } catch (const Failure&) {
        throw Failure{invalid};
    }
    if (r.palette_max_iter < 0 || r.palette_max_iter > kMaxIterations
        || !valid_colour_controls(phase, vocal, instrumental, pitch)
        || (interior_color != nullptr
            && (interior_color[0] < 0 || interior_color[0] > 255 || interior_color[1] < 0 || interior_color[1] > 255
                || interior_color[2] < 0 || interior_color[2] > 255))) {
        throw Failure{invalid};
    }
    AtlasLaunch a = atlas_geometry(r);
    a.mode = kAtlasAurora;
    if (a.use_child && (!valid_dims(r.child_width, r.child_height) || !valid_iterations(r.child_max_iter))) {
        throw Failure{"invalid native atlas child tile"};
    }
    a.palette_iter = std::max(1, std::max(r.palette_max_iter,
                                          std::max(r.parent_max_iter, a.use_child ? r.child_max_iter : 0)));
    a.feather = a.use_child && !a.full_child
        ? std::min(48, std::min(a.child_visible_width / 8, a.child_visible_height / 8)) : 0;
    for (int c = 0; c < 3; ++c) a.interior[c] = interior_color ? interior_color[c] : 0;
    return a;
}

void attach_aurora(ThreadRuntime& rt, AtlasLaunch& a, double phase, double vocal, double pitch,
                   const std::uint8_t* accents) {
    int lut_size = 0;
    a.lut = aurora_lut(rt, a.palette_iter, phase, vocal, pitch, lut_size, accents);
    a.lut_size = lut_size;
    a.index_scale = static_cast<float>(lut_size - 1) / static_cast<float>(a.palette_iter);
}

// Copies host sources (float fields, or RGB8 for kAtlasRgb) into the atlas
// scratch and points `a` at them; returns the table space that follows.
void* stage_atlas_sources(ThreadRuntime& rt, AtlasLaunch& a, const void* parent, const void* child) {
    auto up = [](std::size_t v) { return (v + 255) / 256 * 256; };
    const std::size_t unit = a.mode == kAtlasRgb ? 3 : 4;
    const std::size_t parent_bytes = a.full_child ? 0 : static_cast<std::size_t>(a.parent_width) * a.parent_height * unit;
    const std::size_t child_bytes = a.use_child ? static_cast<std::size_t>(a.child_width) * a.child_height * unit : 0;
    char* base = static_cast<char*>(scratch(rt, kScratchAtlas, up(parent_bytes) + up(child_bytes)
                                                                   + atlas_table_bytes(a)));
    if (parent_bytes) {
        check_cuda(cudaMemcpyAsync(base, parent, parent_bytes, cudaMemcpyHostToDevice, rt.stream), "atlas parent");
    }
    if (child_bytes) {
        check_cuda(cudaMemcpyAsync(base + up(parent_bytes), child, child_bytes, cudaMemcpyHostToDevice, rt.stream),
                   "atlas child");
    }
    if (a.mode == kAtlasRgb) {
        a.parent_rgb = reinterpret_cast<const std::uint8_t*>(base);
        a.child_rgb = reinterpret_cast<const std::uint8_t*>(base + up(parent_bytes));
    } else {
        a.parent = reinterpret_cast<const float*>(base);
        a.child = reinterpret_cast<const float*>(base + up(parent_bytes));
    }
    return base + up(parent_bytes) + up(child_bytes);
}

// Copies host sources into the atlas scratch, composes, copies the frame
// back; `output` is float[W*H] (field) or uint8[W*H*3] (aurora).
void atlas_from_host(ThreadRuntime& rt, AtlasLaunch& a, const void* parent, const void* child, void* output,
                     bool field) {
    void* tables = stage_atlas_sources(rt, a, parent, child);
    const std::size_t pixels = static_cast<std::size_t>(a.out_width) * a.out_height;
    const std::size_t out_bytes = field ? pixels * sizeof(float) : pixels * 3;
    void* device_out = scratch(rt, field ? kScratchField : kScratchRgb, out_bytes);
    if (field) {
        a.field_out = static_cast<float*>(device_out);
    } else {
        a.rgb = static_cast<std::uint8_t*>(device_out);
    }
    check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
    check_cuda(run_atlas(rt, a, tables, rt.stream), "atlas kernel launch");
    check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
    check_cuda(cudaMemcpyAsync(output, device_out, out_bytes, cudaMemcpyDeviceToHost, rt.stream),
               "copy atlas frame to host");
    check_cuda(cudaStreamSynchronize(rt.stream), "atlas frame");
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
}

// kfp_atlas_seam_feather (renderer.cpp:99-112).
int kfp_seam_feather(int width, int height) {
    const int minimum = std::min(width, height);
    if (minimum <= 0) return 0;
    const int requested = std::max(2, std::min(64, minimum / 2));
    return std::min(requested, std::max(0, (minimum - 1) / 2));
}

// fractal_atlas_colourise_kfp_raw's child checks and surface constants
// (renderer.cpp:18010-18068); `field_bias` is the KFP field bias.
AtlasLaunch kfp_surface_launch(const AtlasRequest& r, double child_zoom, int max_iter, double field_bias) {
    const bool use_child = r.has_child && r.child_fraction > 0.0;
    if (use_child && (!valid_dims(r.child_width, r.child_height) || !valid_iterations(r.child_max_iter))) {
        throw Failure{"invalid native raw KFP atlas child tile"};
    }
    if (!use_child && r.has_child) throw Failure{"raw KFP atlas child needs a positive visible fraction"};
    if (!use_child && (r.child_width != 0 || r.child_height != 0 || r.child_max_iter != 0)) {
        throw Failure{"invalid native raw KFP atlas child absence"};
    }
    if (field_bias > static_cast<double>(max_iter)) throw Failure{"native KFP field bias exceeds iteration cap"};
    AtlasLaunch a = atlas_geometry(r);
    a.mode = kAtlasKfpSurface;
    a.full_child = 0;  // the parent is sampled everywhere; the seam runs to the frame edge
    a.parent_zoom = std::max(r.parent_zoom, 1.0);
    a.child_zoom = std::max(child_zoom, 1.0);
    const bool centred = field_bias > 0.0;
    a.parent_bias = centred ? static_cast<double>(r.parent_max_iter) : 0.0;
    a.child_bias = centred ? static_cast<double>(r.child_max_iter) : 0.0;
    a.output_bias = field_bias;
    a.effective_iter = max_iter;
    a.feather = use_child ? kfp_seam_feather(a.child_visible_width, a.child_visible_height) : 0;
    return a;
}

// The argument checks of fractal_atlas_colourise_kfp_raw (renderer.cpp:
// 17994-18009), then the surface constants.
AtlasLaunch kfp_raw_launch(const AtlasRequest& r, double child_zoom, int max_iter, double phase, double vocal,
                           double instrumental, double pitch, const FractalKfpOptions* options, const uint8_t* lut,
                           int lut_size) {
    const char* invalid = "invalid native raw KFP atlas dimensions or controls";
    try {
        check_atlas_common(r);
    } catch (const Failure&) {
        throw Failure{invalid};
    }
    if (!valid_iterations(max_iter) || !std::isfinite(child_zoom) || child_zoom <= 0.0
        || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut || !valid_kfp(options, lut_size)) {
        throw Failure{invalid};
    }
    return kfp_surface_launch(r, child_zoom, max_iter, options->field_bias);
}

}  // namespace

// ------------------------------------------------------- keyframe batches
namespace {

struct BatchShapes {
    QueueShape direct{64, 8};
    QueueShape floatexp{256, 0};
};

std::mutex tuned_mutex;
std::map<std::string, BatchShapes> tuned_shapes;  // by batch class

// Everything one batch enqueues, resolved on the host first (tables
// uploaded, zooms parsed) so the enqueue itself can be captured in a graph.
struct BatchPlan {
    std::map<int, std::vector<DirectParams>> direct;  // by formula, | 0x100 for fields with planes
    std::vector<FxParams> floatexp;
    std::vector<float> log_zoom;       // per floatexp field (tile features)
    unsigned tile_flags = 0;           // FRACTAL_GB300_BATCH_TILES / _LEARNED / _PROBE
    bool fast_smooth = false;          // floatexp form: direct frames' smooth value in FP32
    mlp::CostNet* net = nullptr;
    int tiles = 0;
    int feature_rows = 0;
    // Plain-form launches: (stream, the alternate queue's claim counter for
    // that stream).
    std::vector<std::function<void(cudaStream_t, unsigned long long*)>> plain;
    // A time budget stamps its origin per launch in one per-thread word, so
    // budgeted plain launches stay one after another on one stream.
    bool serial_plain = false;
    std::vector<std::shared_ptr<ReferenceContext>> contexts;
    std::string key;
    std::size_t direct_bytes = 0;
};

template <typename T>
void append_bytes(std::string& key, const T& value) {
    key.append(reinterpret_cast<const char*>(&value), sizeof value);
}

// Tile-mode buffers in one scratch region: per-tile cost, timing, probe,
// features, predictions, order.
struct TileBuffers {
    unsigned long long* cost;
    unsigned long long* timing;
    std::uint32_t* probe;
    __nv_bfloat16* features;
    float* predicted;
    unsigned* order;
    std::size_t bytes;
};

TileBuffers tile_buffers(char* base, int tiles, int rows) {
    auto up = [](std::size_t v) { return (v + 255) / 256 * 256; };
    TileBuffers t{};
    std::size_t at = 0;
    t.cost = reinterpret_cast<unsigned long long*>(base + at);
    at += up(sizeof(unsigned long long) * tiles);
    t.timing = reinterpret_cast<unsigned long long*>(base + at);
    at += 256;
    t.probe = reinterpret_cast<std::uint32_t*>(base + at);
    at += up(sizeof(std::uint32_t) * static_cast<std::size_t>(tiles) * mlp::kProbe);
    t.features = reinterpret_cast<__nv_bfloat16*>(base + at);
    at += up(sizeof(__nv_bfloat16) * static_cast<std::size_t>(rows) * mlp::kFeatures);
    t.predicted = reinterpret_cast<float*>(base + at);
    at += up(sizeof(float) * rows);
    t.order = reinterpret_cast<unsigned*>(base + at);
    at += up(sizeof(unsigned) * tiles);
    t.bytes = at;
    return t;
}

void enqueue_batch(const BatchPlan& plan, const BatchShapes& shapes, ThreadRuntime& rt, cudaStream_t main,
                   void* direct_scratch, unsigned long long* counter, unsigned long long* alt_counters) {
    // The direct queue runs on the second stream beside the other launches;
    // with an FP32 queue in the batch a single plain-form (FP64) launch joins
    // it there, so the FP64 and FP32 pipes work at once.  Two or more
    // plain-form launches are dealt over the lane streams instead (all forked
    // from and joined back to the caller's stream), so their tails overlap.
    // Fields that asked for derivative planes only share one discard region
    // for the planes nobody reads; concurrent lanes may write it in any order.
    const int lanes = plan.plain.size() > 1 && !plan.serial_plain
        ? static_cast<int>(std::min<std::size_t>(ThreadRuntime::kPlainLanes, plan.plain.size())) : 0;
    const bool fork = (!plan.direct.empty() && (!plan.floatexp.empty() || !plan.plain.empty()))
        || (!plan.plain.empty() && !plan.floatexp.empty());
    cudaStream_t plain_stream = fork && !plan.floatexp.empty() ? rt.side : main;
    cudaStream_t direct_stream = fork ? rt.side : main;
    if (fork || lanes > 0) check_cuda(cudaEventRecord(rt.fork, main), "cudaEventRecord (fork)");
    if (fork) check_cuda(cudaStreamWaitEvent(rt.side, rt.fork, 0), "cudaStreamWaitEvent (fork)");
    for (int l = 0; l < lanes; ++l) {
        check_cuda(cudaStreamWaitEvent(rt.lanes[l], rt.fork, 0), "cudaStreamWaitEvent (lane fork)");
    }
    for (const auto& group : plan.direct) {
        const std::vector<DirectParams>& fields = group.second;
        for (std::size_t i = 0; i < fields.size(); i += kMaxDirectFields) {
            const int n = static_cast<int>(std::min<std::size_t>(kMaxDirectFields, fields.size() - i));
            long long pixels = 0;
            for (int f = 0; f < n; ++f) pixels += static_cast<long long>(fields[i + f].width) * fields[i + f].height;
            last_direct_noalloc = false;
            check_cuda(launch_direct_batch(fields.data() + i, n, direct_scratch, shapes.direct, spill_entries(pixels),
                                           direct_stream, plan.fast_smooth),
                       "direct batch launch");
        }
    }
    for (std::size_t i = 0; i < plan.floatexp.size(); i += kMaxFxFields) {
        const int n = static_cast<int>(std::min<std::size_t>(kMaxFxFields, plan.floatexp.size() - i));
        check_cuda(launch_series_prologue(plan.floatexp.data() + i, n, main), "series prologue launch");
    }
    if (plan.tile_flags != 0 && !plan.floatexp.empty()) {
        const TileBuffers t = tile_buffers(static_cast<char*>(scratch(rt, kScratchTiles, 1)), plan.tiles,
                                           plan.feature_rows);
        const int n = static_cast<int>(plan.floatexp.size());
        TileSchedule schedule;
        schedule.tile_rows = shapes.floatexp.chunk >= 64 && shapes.floatexp.chunk <= 4096
            ? std::max(1, std::min(64, shapes.floatexp.chunk / 64)) : 8;
        while (64 % schedule.tile_rows != 0) --schedule.tile_rows;
        schedule.tile_cost = t.cost;
        schedule.timing = t.timing;
        if (plan.tile_flags & (FRACTAL_GB300_BATCH_LEARNED | FRACTAL_GB300_BATCH_PROBE)) {
            check_cuda(launch_tile_probe(plan.floatexp.data(), plan.log_zoom.data(), n, t.probe, t.features,
                                         plan.feature_rows, main),
                       "tile probe launch");
        }
        if (plan.tile_flags & FRACTAL_GB300_BATCH_LEARNED) {
            std::string why;
            if (!mlp::predict_async(plan.net, t.features, plan.feature_rows, t.predicted, main, why)) {
                throw Failure{why};
            }
            check_cuda(launch_tile_order(t.predicted, plan.tiles, t.order, main), "tile order launch");
            schedule.order = t.order;
        }
        check_cuda(launch_floatexp_tiles(plan.floatexp.data(), plan.log_zoom.data(), n, counter, shapes.floatexp,
                                         schedule, main),
                   "floatexp tile queue launch");
    } else {
        for (std::size_t i = 0; i < plan.floatexp.size(); i += kMaxFxFields) {
            const int n = static_cast<int>(std::min<std::size_t>(kMaxFxFields, plan.floatexp.size() - i));
            check_cuda(launch_floatexp_batch(plan.floatexp.data() + i, n, counter, shapes.floatexp, main),
                       "floatexp batch launch");
        }
    }
    if (lanes > 0) {
        for (std::size_t i = 0; i < plan.plain.size(); ++i) {
            plan.plain[i](rt.lanes[i % lanes], alt_counters + (i % lanes) * kAltQueueStride);
        }
        for (int l = 0; l < lanes; ++l) {
            check_cuda(cudaEventRecord(rt.lane_join[l], rt.lanes[l]), "cudaEventRecord (lane join)");
            check_cuda(cudaStreamWaitEvent(main, rt.lane_join[l], 0), "cudaStreamWaitEvent (lane join)");
        }
    } else {
        for (const auto& launch : plan.plain) launch(plain_stream, alt_counters);
    }
    if (fork) {
        check_cuda(cudaEventRecord(rt.join, rt.side), "cudaEventRecord (join)");
        check_cuda(cudaStreamWaitEvent(main, rt.join, 0), "cudaStreamWaitEvent (join)");
    }
}

void launch_plan(const BatchPlan& plan, const BatchShapes& shapes, ThreadRuntime& rt, cudaStream_t stream,
                 bool graph) {
    void* direct_scratch = plan.direct.empty() ? nullptr : scratch(rt, kScratchDirect, plan.direct_bytes);
    auto* counter = static_cast<unsigned long long*>(scratch(rt, kScratchQueue, 256));
    unsigned long long* alt_counters = plan.plain.empty() ? nullptr : alt_queue_counters(rt);
    if (!graph) {
        enqueue_batch(plan, shapes, rt, stream, direct_scratch, counter, alt_counters);
        return;
    }
    std::string key = plan.key;
    append_bytes(key, shapes);
    append_bytes(key, direct_scratch);
    append_bytes(key, counter);
    append_bytes(key, alt_counters);
    auto found = rt.graphs.find(key);
    if (found == rt.graphs.end()) {
        if (rt.graphs.size() >= 16) {
            check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize (graph cache)");
            for (auto& entry : rt.graphs) cudaGraphExecDestroy(entry.second);
            rt.graphs.clear();
        }
        check_cuda(cudaStreamBeginCapture(rt.capture, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
        try {
            enqueue_batch(plan, shapes, rt, rt.capture, direct_scratch, counter, alt_counters);
        } catch (...) {
            cudaGraph_t broken = nullptr;
            cudaStreamEndCapture(rt.capture, &broken);
            if (broken) cudaGraphDestroy(broken);
            throw;
        }
        cudaGraph_t g = nullptr;
        check_cuda(cudaStreamEndCapture(rt.capture, &g), "cudaStreamEndCapture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t made = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        check_cuda(made, "cudaGraphInstantiate");
        found = rt.graphs.emplace(key, exec).first;
    }
    check_cuda(cudaGraphLaunch(found->second, stream), "cudaGraphLaunch");
}

// FP32-queue blocks that stay resident on an SM beside `direct_blocks`
// blocks of the FP64 direct queue: the registers (allocated per warp in
// units of 256) and shared memory (plus the 1 KB each block reserves) left
// over, within the FP32 queue's own occupancy and the SM's thread limit.
int floatexp_blocks_beside(int direct_blocks, bool tiles) {
    const int alone = floatexp_queue_occupancy(tiles);
    cudaFuncAttributes fd{}, ff{};
    int device = 0, sm_regs = 0, sm_smem = 0, sm_threads = 0;
    if (direct_queue_attributes(&fd) != cudaSuccess || floatexp_queue_attributes(tiles, &ff) != cudaSuccess
        || cudaGetDevice(&device) != cudaSuccess
        || cudaDeviceGetAttribute(&sm_regs, cudaDevAttrMaxRegistersPerMultiprocessor, device) != cudaSuccess
        || cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device) != cudaSuccess
        || cudaDeviceGetAttribute(&sm_threads, cudaDevAttrMaxThreadsPerMultiProcessor, device) != cudaSuccess) {
        cudaGetLastError();
        return std::max(1, std::min(direct_queue_occupancy(), alone) - direct_blocks);
    }
    auto block_regs = [](const cudaFuncAttributes& a) {
        return 4 * ((a.numRegs * 32 + 255) / 256 * 256);  // four warps of 128-thread blocks
    };
    const int regs_left = sm_regs - direct_blocks * block_regs(fd);
    const int smem_left = sm_smem - direct_blocks * (static_cast<int>(fd.sharedSizeBytes) + 1024);
    int blocks = std::min(alone, regs_left / std::max(1, block_regs(ff)));
    blocks = std::min(blocks, smem_left / (static_cast<int>(ff.sharedSizeBytes) + 1024));
    blocks = std::min(blocks, (sm_threads - 128 * direct_blocks) / 128);
    return std::max(1, blocks);
}

// Coordinate descent over the launch shapes, each candidate timed (median of
// three, or one run for batches of a second or more; CUDA events) on the
// batch itself and through the same launch path (graph replay or direct
// enqueue) the batch will use.  When the batch has both queues, their
// blocks per SM are chosen together: splits where both stay resident (the
// FP64 direct queue and the FP32 queue then share every SM instead of
// waiting on each other), and the FP32 queue at its full occupancy, whose
// extra blocks start as the direct queue's (placed first: its stream has the
// highest priority) finish.  Shapes change only the schedule, never a pixel.
BatchShapes autotune(const BatchPlan& plan, ThreadRuntime& rt, cudaStream_t stream, bool graph) {
    BatchShapes best;
    const bool both = !plan.direct.empty() && !plan.floatexp.empty();
    const bool tiles = plan.tile_flags != 0;
    const int capacity = std::min(direct_queue_occupancy(), floatexp_queue_occupancy(tiles));
    if (both) {
        best.direct.blocks_per_sm = std::max(1, capacity / 2);
        best.floatexp.blocks_per_sm = floatexp_blocks_beside(best.direct.blocks_per_sm, tiles);
    }
    cudaEvent_t a = nullptr, b = nullptr;
    check_cuda(cudaEventCreate(&a), "cudaEventCreate");
    check_cuda(cudaEventCreate(&b), "cudaEventCreate");
    int repeats = 3;  // median of three; one run each for batches of a second or more
    auto time = [&](const BatchShapes& shapes) {
        float runs[3];
        for (int r = 0; r < repeats; ++r) {
            check_cuda(cudaEventRecord(a, stream), "cudaEventRecord");
            launch_plan(plan, shapes, rt, stream, graph);
            check_cuda(cudaEventRecord(b, stream), "cudaEventRecord");
            check_cuda(cudaEventSynchronize(b), "cudaEventSynchronize");
            check_cuda(cudaEventElapsedTime(&runs[r], a, b), "cudaEventElapsedTime");
        }
        std::sort(runs, runs + repeats);
        return runs[repeats / 2];
    };
    try {
        if (time(best) >= 1000.0f) repeats = 1;  // warm-up (occupancy queries, graph capture, caches)
        float best_ms = time(best);
        auto sweep = [&](const std::vector<BatchShapes>& candidates) {
            for (const BatchShapes& c : candidates) {
                const float ms = time(c);
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
        };
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<BatchShapes> c;
            if (!plan.direct.empty()) {
                for (int chunk : {32, 64, 128}) {
                    if (chunk == best.direct.chunk) continue;
                    BatchShapes s = best;
                    s.direct.chunk = chunk;
                    c.push_back(s);
                }
                for (int steps : {1, 2, 4}) {
                    if (steps == (best.direct.steps > 0 ? best.direct.steps : 2)) continue;
                    BatchShapes s = best;
                    s.direct.steps = steps;
                    c.push_back(s);
                }
            }
            if (both) {
                // Co-resident splits, and the FP32 queue at its full
                // occupancy: the blocks that do not fit beside the direct
                // queue's start when its blocks finish.
                const int full = floatexp_queue_occupancy(tiles);
                for (int d = 1; d < capacity; ++d) {
                    // Full occupancy is tried with every direct share, or for
                    // batches of a second or more with the best one so far.
                    const bool try_full = repeats > 1 || d == best.direct.blocks_per_sm;
                    for (int f : {floatexp_blocks_beside(d, tiles), try_full ? full : 0}) {
                        if (f == 0 || (d == best.direct.blocks_per_sm && f == best.floatexp.blocks_per_sm)) continue;
                        BatchShapes s = best;
                        s.direct.blocks_per_sm = d;
                        s.floatexp.blocks_per_sm = f;
                        c.push_back(s);
                    }
                }
            } else if (!plan.direct.empty()) {
                for (int d : {2, 4, 6, 0}) {
                    if (d == best.direct.blocks_per_sm) continue;
                    BatchShapes s = best;
                    s.direct.blocks_per_sm = d;
                    c.push_back(s);
                }
            } else if (!plan.floatexp.empty()) {
                for (int f : {4, 6, 0}) {
                    if (f == best.floatexp.blocks_per_sm) continue;
                    BatchShapes s = best;
                    s.floatexp.blocks_per_sm = f;
                    c.push_back(s);
                }
            }
            if (!plan.floatexp.empty()) {
                for (int chunk : {128, 256, 512}) {
                    if (chunk == best.floatexp.chunk) continue;
                    BatchShapes s = best;
                    s.floatexp.chunk = chunk;
                    c.push_back(s);
                }
            }
            sweep(c);
        }
    } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}

// Zoom (log10) from which a direct-path frame keeps the FP64 direct iteration
// in the floatexp form: there FP64's 2^-53 resolution leaves fewer than about
// ten bits below a 1080-row pixel, so the FP64 counts are decided by FP64
// rounding and only FP64 reproduces them.
constexpr long double kShallowFp64Log10Zoom = 10.0L;

// Whether the floatexp form renders a direct-path frame (FRACTAL_GB300_
// KEYFRAME_SHALLOW) by FP32 perturbation: Mandelbrot only, below 1e10, and
// only where a 16:9 view does not reach the main cardioid's or period-2
// bulb's bounding box (near those parabolic boundaries a 1e-4-pixel error in
// c moves many escape counts).  atlas.shallow_perturbation is the same rule.
bool shallow_perturbs(const ReferenceContext& ctx, const char* zoom_text, const FractalRenderOptions& o) {
    if (ctx.formula != kFormulaMandelbrot) return false;
    const long double zoom = parse_zoom_direct(zoom_text);
    if (!(zoom > 0.0L) || std::log10(zoom) >= kShallowFp64Log10Zoom) return false;
    const double span = viewport_height_factor(o.coordinate_mode) / static_cast<double>(zoom);
    const double half_h = 0.5 * span + 0.05;
    const double half_w = 0.5 * span * (16.0 / 9.0) + 0.05;
    const double x = static_cast<double>(ctx.x_center), y = static_cast<double>(ctx.y_center);
    const bool cardioid = x + half_w >= -0.80 && x - half_w <= 0.40 && y + half_h >= -0.70 && y - half_h <= 0.70;
    const bool bulb = x + half_w >= -1.30 && x - half_w <= -0.70 && y + half_h >= -0.30 && y - half_h <= 0.30;
    return !(cardioid || bulb);
}

// One field of a batch: device outputs (derivative planes optional), its
// view and the reference handle it renders from.
struct FieldRequest {
    Outputs out;
    const char* zoom_text = nullptr;
    void* reference = nullptr;
    int width = 0;
    int height = 0;
    int max_iter = 0;
    int flags = 0;
};

// The batch behind fractal_gb300_render_keyframes_device and
// fractal_gb300_render_fields_device: every field resolved on the host
// (zooms parsed, tables uploaded), then one enqueue -- the direct fields in
// the FP64 lane-refill queue on the second stream (one launch per formula and
// plane set), the floatexp fields of every formula and size in one
// persistent FP32 queue, plain-form deep fields one launch each -- optionally
// captured into a CUDA graph and autotuned.
void render_field_batch(const std::vector<FieldRequest>& fields, const char* x_center, const char* y_center,
                        int series_order, int series_block, const FractalRenderOptions* supplied, int form,
                        unsigned flags, void* stream_handle) {
    if (fields.empty() || !valid_series(series_order, series_block) || (form != 0 && form != 1)) {
        throw Failure{"invalid native keyframe batch"};
    }
    const FractalRenderOptions o = checked_options(supplied);
    check_backend(o);
    ThreadRuntime& rt = thread_runtime();
    cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
    BatchPlan plan;
    plan.fast_smooth = form == 1;
    plan.serial_plain = o.time_budget_ms > 0;
    append_bytes(plan.key, form);
    std::size_t direct_doubles = 0;
    bool centre_parsed = false;
    long double cx = 0.0L, cy = 0.0L;
    // Planes no caller asked for but the plain kernels write (they take all
    // six or none): one shared discard region sized for the largest field.
    long long plane_pixels = 0;
    for (std::size_t i = 0; i < fields.size(); ++i) {
        const FieldRequest& f = fields[i];
        if (!f.out.field || !f.zoom_text || !valid_iterations(f.max_iter) || !valid_dims(f.width, f.height)) {
            throw Failure{"invalid native keyframe " + std::to_string(i)};
        }
        if ((f.flags & ~FRACTAL_GB300_KEYFRAME_SHALLOW) != 0) {
            throw Failure{"invalid native keyframe " + std::to_string(i) + " flags"};
        }
        if (f.out.p_dex) plane_pixels = std::max(plane_pixels, static_cast<long long>(f.width) * f.height);
    }
    Outputs discard;
    if (plane_pixels > 0) {
        auto* base = static_cast<char*>(scratch(rt, kScratchDiscard, static_cast<std::size_t>(plane_pixels) * 32));
        discard.p_iter = reinterpret_cast<std::int64_t*>(base);
        discard.p_phase = reinterpret_cast<double*>(base + plane_pixels * 8);
        discard.p_t1 = reinterpret_cast<double*>(base + plane_pixels * 16);
        discard.p_t2 = reinterpret_cast<double*>(base + plane_pixels * 24);
    }
    // All six planes for the plain kernels: the caller's derivative planes,
    // the rest into the discard region.
    auto plain_outputs = [&](const Outputs& out) {
        Outputs full = out;
        if (out.p_dex) {
            full.p_iter = discard.p_iter;
            full.p_phase = discard.p_phase;
            full.p_t1 = discard.p_t1;
            full.p_t2 = discard.p_t2;
        }
        return full;
    };
    auto direct_group = [](int formula, const Outputs& out) { return formula | (out.p_dex ? 0x100 : 0); };
    for (std::size_t i = 0; i < fields.size(); ++i) {
        const FieldRequest& frame = fields[i];
        const int width = frame.width, height = frame.height;
        const bool shallow = (frame.flags & FRACTAL_GB300_KEYFRAME_SHALLOW) != 0;
        if (!frame.reference) {
            if (!centre_parsed) {
                if (!x_center || !y_center) throw Failure{"keyframe batch without a centre for direct frames"};
                cx = parse_coordinate(x_center, "real");
                cy = parse_coordinate(y_center, "imaginary");
                centre_parsed = true;
            }
            const Outputs out = plain_outputs(frame.out);
            auto& group = plan.direct[direct_group(kFormulaMandelbrot, out)];
            group.push_back(make_direct_params(out, width, height, parse_zoom_direct(frame.zoom_text), cx, cy,
                                               frame.max_iter, kFormulaMandelbrot, 0.0, 0.0, o));
            direct_doubles += static_cast<std::size_t>(width) + height;
            append_bytes(plan.key, group.back());
            continue;
        }
        std::shared_ptr<ReferenceContext> ctx = acquire_reference(frame.reference);
        if (!ctx) throw Failure{"invalid or already-destroyed reference handle"};
        if (ctx->escape_mode != o.escape_radius_mode) {
            throw Failure{"reference escape-radius mode does not match render options"};
        }
        if (frame.max_iter > ctx->requested_max_iter) {
            throw Failure{"render iteration count exceeds prepared reference"};
        }
        plan.contexts.push_back(ctx);
        // A shallow frame stays on the FP64 direct path (at its reference's
        // centre) in form 0, and in form 1 wherever the shallow mode would
        // not reproduce the FP64 counts within the floatexp budget.
        const bool direct_path = shallow && (form == 0 || !shallow_perturbs(*ctx, frame.zoom_text, o));
        FxParams fx;
        if (form == 1 && !direct_path
            && make_floatexp_params(*ctx, frame.out, width, height, frame.zoom_text, frame.max_iter, series_order,
                                    series_block, o, fx, (flags & FRACTAL_GB300_BATCH_FP32_ALTERNATES) != 0)) {
            plan.floatexp.push_back(fx);
            plan.log_zoom.push_back(static_cast<float>(fe_log10(parse_zoom_fe(frame.zoom_text,
                                                                              ctx->precision_bits))));
            append_bytes(plan.key, fx);
            continue;
        }
        const fx::Fe zoom = parse_zoom_fe(frame.zoom_text, ctx->precision_bits);
        const Outputs out = plain_outputs(frame.out);
        if (fe_log10(zoom) < 6.0L || direct_path) {
            auto& group = plan.direct[direct_group(ctx->formula, out)];
            group.push_back(make_direct_params(out, width, height, parse_zoom_direct(frame.zoom_text), ctx->x_center,
                                               ctx->y_center, frame.max_iter, ctx->formula, ctx->julia_re,
                                               ctx->julia_im, o));
            direct_doubles += static_cast<std::size_t>(width) + height;
            append_bytes(plan.key, group.back());
            continue;
        }
        std::shared_ptr<DeviceTables> dev = device_tables(*ctx);
        ReferenceContext* raw = ctx.get();
        const int max_iter = frame.max_iter;
        plan.plain.push_back([raw, dev, out, width, height, zoom, max_iter, series_order, series_block, o,
                              &rt](cudaStream_t s, unsigned long long* queue_counter) {
            if (raw->formula != kFormulaMandelbrot) {
                launch_deep_alternate(*raw, *dev, out, width, height, zoom, max_iter, o, false, rt, s, nullptr,
                                      queue_counter);
            } else {
                launch_deep_mandelbrot(*raw, *dev, out, width, height, zoom, max_iter, series_order,
                                       series_block, o, false, rt, s);
            }
        });
        append_bytes(plan.key, raw);
        append_bytes(plan.key, raw->generation);
        append_bytes(plan.key, out);
        append_bytes(plan.key, zoom);
        append_bytes(plan.key, max_iter);
        append_bytes(plan.key, width);
        append_bytes(plan.key, height);
        append_bytes(plan.key, series_order);
        append_bytes(plan.key, series_block);
        append_bytes(plan.key, o);
    }
    for (const auto& group : plan.direct) {
        const std::vector<DirectParams>& direct = group.second;
        for (std::size_t i = 0; i < direct.size(); i += kMaxDirectFields) {
            const int n = static_cast<int>(std::min<std::size_t>(kMaxDirectFields, direct.size() - i));
            long long pixels = 0;
            for (int f = 0; f < n; ++f) pixels += static_cast<long long>(direct[i + f].width) * direct[i + f].height;
            plan.direct_bytes = std::max(plan.direct_bytes,
                                         direct_scratch_bytes(direct.data() + i, n, spill_entries(pixels)));
        }
    }
    if (!plan.floatexp.empty()) {
        auto* slots = static_cast<FxSeriesScaled*>(
            scratch(rt, kScratchSeries, sizeof(FxSeriesScaled) * plan.floatexp.size()));
        for (std::size_t f = 0; f < plan.floatexp.size(); ++f) plan.floatexp[f].series_scaled = slots + f;
        append_bytes(plan.key, slots);
    }
    plan.tile_flags = flags & (FRACTAL_GB300_BATCH_TILES | FRACTAL_GB300_BATCH_LEARNED | FRACTAL_GB300_BATCH_PROBE);
    if (plan.tile_flags != 0 && !plan.floatexp.empty()) {
        if (plan.floatexp.size() > static_cast<std::size_t>(kMaxFxFields)) {
            throw Failure{"tile-scheduled batches take at most 64 floatexp keyframes"};
        }
        plan.tiles = batch_tiles(plan.floatexp.data(), static_cast<int>(plan.floatexp.size()));
        plan.feature_rows = (plan.tiles + 127) / 128 * 128;
        if (plan.tile_flags & FRACTAL_GB300_BATCH_LEARNED) {
            if (!rt.costnet) throw Failure{"learned tile order requested but no cost network is attached"};
            plan.net = static_cast<mlp::CostNet*>(rt.costnet);
            std::string why;
            if (!mlp::reserve_rows(plan.net, plan.feature_rows, why)) throw Failure{why};
            append_bytes(plan.key, plan.net);
        }
        scratch(rt, kScratchTiles, tile_buffers(nullptr, plan.tiles, plan.feature_rows).bytes);
        append_bytes(plan.key, plan.tile_flags);
        rt.tile_stream = stream;
        rt.last_tiles = plan.tiles;
    }
    long long total_pixels = 0;
    for (const FieldRequest& f : fields) total_pixels += static_cast<long long>(f.width) * f.height;
    std::string shape_key;
    append_bytes(shape_key, plan.tile_flags);
    append_bytes(shape_key, total_pixels);
    append_bytes(shape_key, form);
    append_bytes(shape_key, static_cast<int>(plan.floatexp.size()));
    append_bytes(shape_key, static_cast<int>(plan.plain.size()));
    append_bytes(shape_key, static_cast<int>(direct_doubles));
    BatchShapes shapes;
    bool tuned = false;
    {
        std::lock_guard<std::mutex> lock(tuned_mutex);
        auto known = tuned_shapes.find(shape_key);
        if (known != tuned_shapes.end()) {
            shapes = known->second;
            tuned = true;
        }
    }
    if (!tuned && !plan.direct.empty() && !plan.floatexp.empty()) {
        // Both queues resident at once: split the SM between them.
        const int capacity = std::min(direct_queue_occupancy(), floatexp_queue_occupancy(plan.tile_flags != 0));
        shapes.direct.blocks_per_sm = std::max(1, capacity / 2);
        shapes.floatexp.blocks_per_sm = floatexp_blocks_beside(shapes.direct.blocks_per_sm, plan.tile_flags != 0);
    }
    if (rt.shapes_pinned) {
        if (rt.pinned_shapes[0] > 0) shapes.direct.chunk = rt.pinned_shapes[0];
        shapes.direct.blocks_per_sm = rt.pinned_shapes[1];
        if (rt.pinned_shapes[2] > 0) shapes.floatexp.chunk = rt.pinned_shapes[2];
        shapes.floatexp.blocks_per_sm = rt.pinned_shapes[3];
    }
    wait_scratch(rt, stream);
    if ((flags & FRACTAL_GB300_BATCH_AUTOTUNE) && !rt.shapes_pinned) {
        shapes = autotune(plan, rt, stream, (flags & FRACTAL_GB300_BATCH_GRAPH) != 0);
        std::lock_guard<std::mutex> lock(tuned_mutex);
        tuned_shapes[shape_key] = shapes;
    }
    rt.batch_stream = stream;
    rt.last_shapes[0] = shapes.direct.chunk;
    rt.last_shapes[1] = shapes.direct.blocks_per_sm;
    rt.last_shapes[2] = shapes.floatexp.chunk;
    rt.last_shapes[3] = shapes.floatexp.blocks_per_sm;
    launch_plan(plan, shapes, rt, stream, (flags & FRACTAL_GB300_BATCH_GRAPH) != 0);
    release_scratch(rt, stream);
}

}  // namespace

extern "C" {

int fractal_abi_version(void) { return FRACTAL_ABI_VERSION; }

int fractal_render_options_version(void) { return FRACTAL_RENDER_OPTIONS_VERSION; }
void fractal_render_options_default(FractalRenderOptions* options) {
    if (options) *options = default_options();
}

int fractal_backend_capabilities(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        set_error("no CUDA device is available");
        return 0;
    }
    set_error("");
    return FRACTAL_CAPABILITY_CUDA;
}

const char* fractal_last_error(void) { return last_error.c_str(); }

void fractal_set_stats_enabled(int enabled) { stats_enabled.store(enabled != 0, std::memory_order_relaxed); }

int fractal_get_last_stats(uint64_t* values, int capacity) {
    if (!values || capacity < kStatsFields) return -1;
    std::lock_guard<std::mutex> lock(stats_mutex);
    for (int i = 0; i < kStatsFields; ++i) values[i] = last_stats[static_cast<std::size_t>(i)];
    return kStatsFields;
}

int fractal_get_last_stats_ex(uint64_t* values, int capacity) {
    if (!values || capacity < kStatsSlots) return -1;
    std::lock_guard<std::mutex> lock(stats_mutex);
    for (int i = 0; i < kStatsSlots; ++i) values[i] = last_stats[static_cast<std::size_t>(i)];
    return kStatsSlots;
}

void* fractal_create_reference(const char* x, const char* y, const char* zoom, int max_iter, int precision_bits,
                               int series_order) {
    return guarded_handle("native reference creation failed with an unknown exception", [&] {
        return create_handle(x, y, zoom, max_iter, precision_bits, series_order, false, kFormulaMandelbrot, "0", "0",
                             nullptr, "invalid reference configuration");
    });
}

void* fractal_create_reference_reusable(const char* x, const char* y, const char* zoom, int max_iter,
                                        int precision_bits, int series_order) {
    return guarded_handle("native reusable reference creation failed with an unknown exception", [&] {
        return create_handle(x, y, zoom, max_iter, precision_bits, series_order, true, kFormulaMandelbrot, "0", "0",
                             nullptr, "invalid reusable reference configuration");
    });
}

void* fractal_create_reference_reusable_options(const char* x, const char* y, const char* zoom, int max_iter,
                                                int precision_bits, int series_order,
                                                const FractalRenderOptions* options) {
    return guarded_handle("native reusable reference creation failed with an unknown exception", [&] {
        return create_handle(x, y, zoom, max_iter, precision_bits, series_order, true, kFormulaMandelbrot, "0", "0",
                             options, "invalid reusable reference configuration");
    });
}

void* fractal_create_reference_ex(const char* x, const char* y, const char* zoom, int max_iter, int precision_bits,
                                  int series_order, int formula, const char* jr, const char* ji) {
    return guarded_handle("formula-aware reference creation failed with an unknown exception", [&] {
        return create_handle(x, y, zoom, max_iter, precision_bits, series_order, formula != kFormulaMandelbrot,
                             formula, jr, ji, nullptr, "invalid formula-aware reference configuration");
    });
}

void* fractal_create_reference_ex_options(const char* x, const char* y, const char* zoom, int max_iter,
                                          int precision_bits, int series_order, int formula, const char* jr,
                                          const char* ji, const FractalRenderOptions* options) {
    return guarded_handle("formula-aware reference creation failed with an unknown exception", [&] {
        return create_handle(x, y, zoom, max_iter, precision_bits, series_order, formula != kFormulaMandelbrot,
                             formula, jr, ji, options, "invalid formula-aware reference configuration");
    });
}

void* fractal_clone_reference(void* source_handle, const char* zoom) {
    return guarded_handle("native reference clone failed with an unknown exception", [&] {
        if (!source_handle || !zoom) throw Failure{"invalid reference tier clone configuration"};
        const auto source = acquire_reference(source_handle);
        if (!source) throw Failure{"invalid or already-destroyed reference handle"};
        return register_reference(clone_reference_context(*source, zoom));
    });
}

void fractal_destroy_reference(void* handle) {
    try {
        if (!handle) {
            set_error("");
            return;
        }
        const auto context = remove_reference(handle);
        if (!context) {
            set_error("invalid or already-destroyed reference handle");
            return;
        }
        set_error("");
    } catch (...) {
        set_error("native reference destruction failed with an unknown exception");
    }
}

int fractal_get_reference_stats(void* handle, uint64_t* values, int capacity) {
    try {
        if (!values || capacity < 5) {
            set_error("reference statistics buffer is too small or null");
            return -1;
        }
        const auto ctx = acquire_reference(handle);
        if (!ctx) {
            set_error("invalid or already-destroyed reference handle");
            return -1;
        }
        values[0] = ctx->reference_build_ns;
        values[1] = ctx->series_build_ns;
        values[2] = ctx->bla_build_ns;
        values[3] = ctx->series.enabled ? static_cast<uint64_t>(ctx->series.iteration) : 0;
        values[4] = ctx->series.enabled ? static_cast<uint64_t>(ctx->series.order) : 0;
        set_error("");
        return 5;
    } catch (...) {
        set_error("reference statistics lookup failed with an unknown exception");
        return -1;
    }
}

int fractal_render_reference_ex_planes(float* output, int width, int height, const char* zoom_text, void* handle,
                                       int max_iter, int threads, int series_order, int series_block,
                                       const FractalRenderOptions* supplied, FractalRenderPlanes* planes) {
    return guarded("native reference render failed with an unknown exception", [&] {
        if (!output || !zoom_text || !handle || !valid_dims(width, height) || !valid_iterations(max_iter)
            || !valid_threads(threads) || !valid_series(series_order, series_block)
            || (planes != nullptr && !valid_planes(planes, width, height))) {
            throw Failure{"invalid native render dimensions or handle"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        const auto ctx = acquire_reference(handle);
        if (!ctx) throw Failure{"invalid or already-destroyed reference handle"};
        if (ctx->escape_mode != o.escape_radius_mode) {
            throw Failure{"reference escape-radius mode does not match render options"};
        }
        if (max_iter > ctx->requested_max_iter) throw Failure{"render iteration count exceeds prepared reference"};
        render_to_host(output, planes, width, height, [&](const Outputs& out, bool collect, ThreadRuntime& rt,
                                                          cudaStream_t stream) {
            // Backend 4 selects the floatexp form for field-only renders;
            // backend 0 (the default) is the plain, reference-identical form.
            if (o.backend == FRACTAL_BACKEND_CUDA && planes == nullptr && !collect) {
                render_floatexp_from_reference(*ctx, out, width, height, zoom_text, max_iter, series_order,
                                               series_block, o, rt, stream);
            } else {
                render_from_reference(*ctx, out, width, height, zoom_text, max_iter, series_order, series_block, o,
                                      collect, rt, stream);
            }
        });
    });
}

}  // extern "C"

namespace {

constexpr int kMaxPoints = 100'000'000;          // MAX_NATIVE_POINTS (renderer.cpp:92)
constexpr int kMaxExactRepairPoints = 8192;      // MAX_EXACT_POINT_REPAIR_PIXELS (renderer.cpp:76)

// fractal_render_points_impl (renderer.cpp:20019-20186): an arbitrary list of
// scaled offsets from the reference centre rendered by the deep kernels.
// Strict Mandelbrot lists of at most 8192 points repair their glitch pixels
// exactly: the kernel flags them, the host iterates each in MPFR (as the
// reference does) on `threads` workers, and any the repair declines are
// rendered again without the flag (rebase or NaN per the options).
int render_points(float* output, int count, const char* zoom_text, const double* real, const double* imag,
                  const std::int32_t* exponents, void* handle, int max_iter, int threads, int series_order,
                  int series_block, const FractalRenderOptions* supplied, FractalRenderPlanes* planes) {
    return guarded("native point render failed with an unknown exception", [&] {
        if (!output || count <= 0 || count > kMaxPoints || !zoom_text || !real || !imag || !exponents || !handle
            || (planes != nullptr && !valid_planes(planes, count, 1))) {
            throw Failure{"invalid native point-render arguments"};
        }
        if (!valid_iterations(max_iter) || !valid_threads(threads) || !valid_series(series_order, series_block)) {
            throw Failure{"invalid native point-render limits"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        const auto ctx = acquire_reference(handle);
        if (!ctx) throw Failure{"invalid or already-destroyed reference handle"};
        if (max_iter > ctx->requested_max_iter) throw Failure{"point render iteration count exceeds prepared reference"};
        const fx::Fe zoom = parse_zoom_fe(zoom_text, ctx->precision_bits);
        std::vector<fx::Sc> points(static_cast<std::size_t>(count));
        fx::Nrm largest = fx::nrm_make(0.0, 0);
        for (int i = 0; i < count; ++i) {
            fx::Sc point = fx::sc_make(real[i], imag[i], exponents[i]);
            if (!fx::sc_finite(point)) throw Failure{"non-finite point offset"};
            fx::sc_normalize(point);
            points[static_cast<std::size_t>(i)] = point;
            const fx::Nrm radius = fx::sc_norm2(point);
            if (fx::nrm_cmp(radius, largest) > 0) largest = radius;
        }
        const fx::Fe point_radius = fx::fe_sqrt(fx::fe_make(largest.m, largest.e));
        const bool repair = ctx->formula == kFormulaMandelbrot && o.strict != 0 && count <= kMaxExactRepairPoints;
        std::vector<std::uint8_t> flags(repair ? static_cast<std::size_t>(count) : 0);

        auto render_list = [&](const std::vector<fx::Sc>& list, float* out_field, FractalRenderPlanes* out_planes,
                               std::uint8_t* host_flags) {
            const int n = static_cast<int>(list.size());
            render_to_host(out_field, out_planes, n, 1, [&](const Outputs& out, bool collect, ThreadRuntime& rt,
                                                            cudaStream_t stream) {
                const std::size_t point_bytes = list.size() * sizeof(fx::Sc);
                const std::size_t flag_offset = (point_bytes + 255) / 256 * 256;
                char* base = static_cast<char*>(scratch(rt, kScratchPoints, flag_offset + list.size()));
                check_cuda(cudaMemcpyAsync(base, list.data(), point_bytes, cudaMemcpyHostToDevice, stream),
                           "upload points");
                PointInput input;
                input.points = reinterpret_cast<const fx::Sc*>(base);
                input.radius = point_radius;
                if (host_flags) {
                    input.exact_flags = reinterpret_cast<std::uint8_t*>(base + flag_offset);
                    check_cuda(cudaMemsetAsync(input.exact_flags, 0, list.size(), stream), "clear repair flags");
                }
                std::shared_ptr<DeviceTables> dev = device_tables(*ctx);
                check_cuda(cudaEventRecord(rt.start, stream), "cudaEventRecord");
                if (ctx->formula != kFormulaMandelbrot) {
                    launch_deep_alternate(*ctx, *dev, out, n, 1, zoom, max_iter, o, collect, rt, stream, &input);
                } else {
                    launch_deep_mandelbrot(*ctx, *dev, out, n, 1, zoom, max_iter, series_order, series_block, o,
                                           collect, rt, stream, &input);
                }
                check_cuda(cudaEventRecord(rt.stop, stream), "cudaEventRecord");
                if (host_flags) {
                    check_cuda(cudaMemcpyAsync(host_flags, input.exact_flags, list.size(), cudaMemcpyDeviceToHost,
                                               stream), "copy repair flags");
                }
            });
        };
        render_list(points, output, planes, repair ? flags.data() : nullptr);
        ThreadRuntime& timing = thread_runtime();
        float kernel_ms = 0.0f;
        if (cudaEventElapsedTime(&kernel_ms, timing.start, timing.stop) == cudaSuccess) {
            timing.last_kernel_ms = kernel_ms;
        }
        if (!repair) return;

        std::vector<int> flagged;
        for (int i = 0; i < count; ++i) {
            if (flags[static_cast<std::size_t>(i)]) flagged.push_back(i);
        }
        if (flagged.empty()) return;
        const fx::Fe spacing = deep_geometry(zoom, count, 1, o.coordinate_mode).pixel_spacing;
        std::vector<std::uint8_t> repaired(flagged.size(), 0);
        std::vector<ExactPlanes> repair_planes(flagged.size());
        std::vector<float> repair_values(flagged.size());
        const unsigned hardware = std::max(1u, std::thread::hardware_concurrency());
        const unsigned workers = std::min<unsigned>(threads > 0 ? static_cast<unsigned>(threads) : hardware,
                                                    static_cast<unsigned>(flagged.size()));
        std::atomic<std::size_t> next{0};
        auto work = [&] {
            for (std::size_t k = next.fetch_add(1); k < flagged.size(); k = next.fetch_add(1)) {
                const std::size_t i = static_cast<std::size_t>(flagged[k]);
                repaired[k] = exact_mandelbrot_pixel(*ctx, points[i], max_iter, o.output_bias, o.escape_radius_mode,
                                                     spacing, repair_values[k],
                                                     planes ? &repair_planes[k] : nullptr) ? 1 : 0;
            }
        };
        std::vector<std::thread> pool;
        for (unsigned w = 1; w < workers; ++w) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
        std::vector<fx::Sc> retry;
        std::vector<int> retry_index;
        for (std::size_t k = 0; k < flagged.size(); ++k) {
            const std::size_t i = static_cast<std::size_t>(flagged[k]);
            if (!repaired[k]) {
                retry.push_back(points[i]);
                retry_index.push_back(static_cast<int>(i));
                continue;
            }
            output[i] = repair_values[k];
            if (planes) {
                planes->orbit_iteration[i] = repair_planes[k].iteration;
                planes->phase[i] = repair_planes[k].phase;
                planes->de_x[i] = repair_planes[k].de_x;
                planes->de_y[i] = repair_planes[k].de_y;
                planes->test1[i] = repair_planes[k].test1;
                planes->test2[i] = repair_planes[k].test2;
            }
        }
        if (retry.empty()) return;
        // Points the exact repair declined: the kernel's own glitch handling.
        const std::size_t n = retry.size();
        std::vector<float> field(n);
        std::vector<std::int64_t> iters(planes ? n : 0);
        std::vector<double> phase(planes ? n : 0), dex(planes ? n : 0), dey(planes ? n : 0), t1(planes ? n : 0),
            t2(planes ? n : 0);
        FractalRenderPlanes sub{};
        if (planes) {
            sub = *planes;
            sub.orbit_iteration = iters.data();
            sub.phase = phase.data();
            sub.de_x = dex.data();
            sub.de_y = dey.data();
            sub.test1 = t1.data();
            sub.test2 = t2.data();
        }
        render_list(retry, field.data(), planes ? &sub : nullptr, nullptr);
        for (std::size_t k = 0; k < n; ++k) {
            const std::size_t i = static_cast<std::size_t>(retry_index[k]);
            output[i] = field[k];
            if (planes) {
                planes->orbit_iteration[i] = iters[k];
                planes->phase[i] = phase[k];
                planes->de_x[i] = dex[k];
                planes->de_y[i] = dey[k];
                planes->test1[i] = t1[k];
                planes->test2[i] = t2[k];
            }
        }
    });
}

}  // namespace

extern "C" {

// fractal_render_points (renderer.h:287-300).
int fractal_render_points(float* output, int point_count, const char* zoom_text, const double* real_mantissa,
                          const double* imag_mantissa, const int32_t* exponents, void* handle, int max_iter,
                          int threads, int series_order, int series_block, const FractalRenderOptions* options) {
    return render_points(output, point_count, zoom_text, real_mantissa, imag_mantissa, exponents, handle, max_iter,
                         threads, series_order, series_block, options, nullptr);
}

// fractal_render_points_ex_planes (renderer.h:302-320).
int fractal_render_points_ex_planes(float* output, int point_count, const char* zoom_text,
                                    const double* real_mantissa, const double* imag_mantissa,
                                    const int32_t* exponents, void* handle, int max_iter, int threads,
                                    int series_order, int series_block, const FractalRenderOptions* options,
                                    FractalRenderPlanes* planes) {
    return render_points(output, point_count, zoom_text, real_mantissa, imag_mantissa, exponents, handle, max_iter,
                         threads, series_order, series_block, options, planes);
}

int fractal_render_reference_ex(float* output, int width, int height, const char* zoom_text, void* handle,
                                int max_iter, int threads, int series_order, int series_block,
                                const FractalRenderOptions* options) {
    return fractal_render_reference_ex_planes(output, width, height, zoom_text, handle, max_iter, threads,
                                              series_order, series_block, options, nullptr);
}

int fractal_render_mandelbrot_reference_ex(float* output, int width, int height, const char* zoom_text,
                                           void* handle, int max_iter, int threads, int series_order,
                                           int series_block, const FractalRenderOptions* options) {
    return fractal_render_reference_ex(output, width, height, zoom_text, handle, max_iter, threads, series_order,
                                       series_block, options);
}

int render_mandelbrot_reference(float* output, int width, int height, const char* zoom_text, void* handle,
                                int max_iter, int threads, int series_order, int series_block) {
    return fractal_render_reference_ex(output, width, height, zoom_text, handle, max_iter, threads, series_order,
                                       series_block, nullptr);
}

int render_fractal_ex_planes(float* output, int width, int height, const char* zoom_text, const char* x_center,
                             const char* y_center, int max_iter, int precision_bits, int use_perturbation,
                             int threads, int formula, double julia_real, double julia_imag,
                             const FractalRenderOptions* supplied, FractalRenderPlanes* planes) {
    return guarded("native render failed with an unknown exception", [&] {
        if (!output || !zoom_text || !x_center || !y_center || !valid_dims(width, height)
            || (planes != nullptr && !valid_planes(planes, width, height)) || !valid_iterations(max_iter)
            || !valid_precision(precision_bits) || use_perturbation < 0 || use_perturbation > 1
            || !valid_threads(threads) || !valid_formula(formula) || !std::isfinite(julia_real)
            || !std::isfinite(julia_imag)) {
            throw Failure{"invalid native render dimensions, formula, or argument"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        if (!use_perturbation) {
            const long double zoom = parse_zoom_direct(zoom_text);
            const long double cx = parse_coordinate(x_center, "real");
            const long double cy = parse_coordinate(y_center, "imaginary");
            render_to_host(output, planes, width, height, [&](const Outputs& out, bool, ThreadRuntime&,
                                                              cudaStream_t stream) {
                launch_direct_render(out, width, height, zoom, cx, cy, max_iter, formula, julia_real, julia_imag, o,
                                     stream);
            });
            return;
        }
        // One-shot deep render: series order 8 and block 32 as the
        // reference's render_fractal_ex does (renderer.cpp:20340-20354).
        const std::string jr = julia_text(julia_real);
        const std::string ji = julia_text(julia_imag);
        void* handle = fractal_create_reference_ex_options(x_center, y_center, zoom_text, max_iter, precision_bits,
                                                           8, formula, jr.c_str(), ji.c_str(), &o);
        if (!handle) throw Failure{last_error};
        const int status = fractal_render_reference_ex_planes(output, width, height, zoom_text, handle, max_iter,
                                                              threads, 8, 32, &o, planes);
        const std::string render_error = last_error;
        fractal_destroy_reference(handle);
        if (status != 0) throw Failure{render_error};
    });
}

int render_fractal_ex(float* output, int width, int height, const char* zoom_text, const char* x_center,
                      const char* y_center, int max_iter, int precision_bits, int use_perturbation, int threads,
                      int formula, double julia_real, double julia_imag, const FractalRenderOptions* options) {
    return render_fractal_ex_planes(output, width, height, zoom_text, x_center, y_center, max_iter, precision_bits,
                                    use_perturbation, threads, formula, julia_real, julia_imag, options, nullptr);
}

int render_mandelbrot_ex(float* output, int width, int height, const char* zoom_text, const char* x_center,
                         const char* y_center, int max_iter, int precision_bits, int use_perturbation, int threads,
                         const FractalRenderOptions* options) {
    return render_fractal_ex(output, width, height, zoom_text, x_center, y_center, max_iter, precision_bits,
                             use_perturbation, threads, kFormulaMandelbrot, 0.0, 0.0, options);
}

int render_mandelbrot(float* output, int width, int height, const char* zoom_text, const char* x_center,
                      const char* y_center, int max_iter, int precision_bits, int use_perturbation, int threads) {
    return render_mandelbrot_ex(output, width, height, zoom_text, x_center, y_center, max_iter, precision_bits,
                                use_perturbation, threads, nullptr);
}

}  // extern "C"

namespace {

// colourise_field_impl (renderer.cpp:13771-13826): aurora palette, optional
// interior colour and accents.
int colourise_field(const float* field, uint8_t* output, int width, int height, int max_iter, double phase,
                    double vocal, double instrumental, double pitch, int threads, const int* interior_color,
                    const std::uint8_t* accents) {
    return guarded("native colouriser failed with an unknown exception", [&] {
        if (!field || !output || !valid_dims(width, height) || !valid_iterations(max_iter) || !valid_threads(threads)
            || !valid_colour_controls(phase, vocal, instrumental, pitch)
            || (interior_color != nullptr
                && (interior_color[0] < 0 || interior_color[0] > 255 || interior_color[1] < 0
                    || interior_color[1] > 255 || interior_color[2] < 0 || interior_color[2] > 255))) {
            throw Failure{"invalid native colour dimensions or palette"};
        }
        const std::uint32_t interior = interior_color == nullptr
            ? 0u
            : static_cast<std::uint32_t>(interior_color[0]) | (static_cast<std::uint32_t>(interior_color[1]) << 8)
                | (static_cast<std::uint32_t>(interior_color[2]) << 16);
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        const std::size_t pixels = static_cast<std::size_t>(width) * static_cast<std::size_t>(height);
        int lut_size = 0;
        const std::uint8_t* lut = aurora_lut(rt, max_iter, phase, vocal, pitch, lut_size, accents);
        float* d_field = static_cast<float*>(scratch(rt, kScratchField, pixels * sizeof(float)));
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        check_cuda(cudaMemcpyAsync(d_field, field, pixels * sizeof(float), cudaMemcpyHostToDevice, rt.stream),
                   "copy field to device");
        const float scale = static_cast<float>(lut_size - 1) / static_cast<float>(max_iter);
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        check_cuda(launch_aurora(d_field, d_rgb, static_cast<long long>(pixels), lut, lut_size, scale, max_iter,
                                 rt.stream, interior), "aurora kernel launch");
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream), "copy RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "aurora colour");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

}  // namespace

extern "C" {

int fractal_colourise(const float* field, uint8_t* output, int width, int height, int max_iter, double phase,
                      double vocal, double instrumental, double pitch, int threads) {
    return colourise_field(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, threads,
                           nullptr, nullptr);
}

// fractal_colourise_accents (renderer.cpp:16210-16248): accent palette with
// an interior colour.
int fractal_colourise_accents(const float* field, uint8_t* output, int width, int height, int max_iter,
                              double phase, double vocal, double instrumental, double pitch,
                              const uint8_t* accents, int interior_red, int interior_green, int interior_blue,
                              int threads) {
    if (accents == nullptr) {
        set_error("ordinary palette accents are required");
        return 1;
    }
    const int interior[3] = {interior_red, interior_green, interior_blue};
    return colourise_field(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, threads,
                           interior, accents);
}

int fractal_colourise_kfp(const float* field, uint8_t* output, int width, int height, int max_iter, double phase,
                          double vocal, double instrumental, double pitch, const FractalKfpOptions* options,
                          const uint8_t* lut, int lut_size, int threads) {
    return kfp_host(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, options, lut, lut_size,
                    threads);
}

int fractal_colourise_kfp_planes(const float* field, uint8_t* output, int width, int height, int max_iter,
                                 double phase, double vocal, double instrumental, double pitch,
                                 const FractalKfpOptions* options, const FractalKfpPlanes* planes, const uint8_t* lut,
                                 int lut_size, int threads) {
    return kfp_planes_host(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, options, planes,
                           lut, lut_size, threads);
}

int fractal_colourise_kfp_precise(const float* field, uint8_t* output, int width, int height, int max_iter,
                                  double phase, double vocal, double instrumental, double pitch,
                                  const FractalKfpOptions* options, const uint8_t* lut, int lut_size, int threads) {
    return kfp_host(field, output, width, height, max_iter, phase, vocal, instrumental, pitch, options, lut, lut_size,
                    threads);
}

// ------------------------------------------------------------ extensions
int fractal_gb300_colourise_kfp_device(const float* field, uint8_t* rgb, int width, int height, int max_iter,
                                       const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                       void* stream_handle) {
    return guarded("device KFP colour failed with an unknown exception", [&] {
        if (!field || !rgb || !lut || !valid_dims(width, height) || !valid_iterations(max_iter)
            || !valid_kfp(options, lut_size)) {
            throw Failure{"invalid native KFP colour dimensions or controls"};
        }
        if (options->field_bias > static_cast<double>(max_iter)) {
            throw Failure{"native KFP field bias exceeds iteration cap"};
        }
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        wait_scratch(rt, rt.stream);
        bool uploaded = false;
        const KfpDeviceInputs in = kfp_inputs(rt, *options, lut, lut_size, true, &uploaded);
        if (uploaded) check_cuda(cudaStreamSynchronize(rt.stream), "KFP inputs");
        kfp_colour(field, rgb, width, height, max_iter, *options, in, lut_size, rt, stream);
        release_scratch(rt, stream);
    });
}

void fractal_gb300_set_table_builder(int on_device) { set_device_table_builder(on_device != 0); }

int fractal_gb300_device_count(void) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count;
}

// Self-check of the colour pass's division by a constant: the number of
// float inputs (of all 2^32) whose quotient differs from IEEE division.
int fractal_gb300_check_division(float divisor, unsigned long long* mismatches) {
    return guarded("division check failed with an unknown exception", [&] {
        if (!mismatches || !std::isfinite(divisor) || divisor == 0.0f) throw Failure{"invalid division check"};
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        auto* counter = static_cast<unsigned long long*>(scratch(rt, kScratchWork, sizeof(unsigned long long)));
        check_cuda(launch_division_check(divisor, counter, rt.stream), "division check launch");
        check_cuda(cudaMemcpyAsync(mismatches, counter, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                   rt.stream), "division check");
        check_cuda(cudaStreamSynchronize(rt.stream), "division check");
    });
}

double fractal_gb300_last_kernel_ms(void) {
    try {
        return thread_runtime().last_kernel_ms;
    } catch (...) {
        return 0.0;
    }
}

int fractal_gb300_render_reference_device(float* field, uint32_t* counts, int width, int height,
                                          const char* zoom_text, void* handle, int max_iter, int series_order,
                                          int series_block, const FractalRenderOptions* supplied, int form,
                                          void* stream_handle) {
    return guarded("device render failed with an unknown exception", [&] {
        if (!field || !zoom_text || !handle || !valid_dims(width, height) || !valid_iterations(max_iter)
            || !valid_series(series_order, series_block) || (form != 0 && form != 1)) {
            throw Failure{"invalid native render dimensions or handle"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        const auto ctx = acquire_reference(handle);
        if (!ctx) throw Failure{"invalid or already-destroyed reference handle"};
        if (ctx->escape_mode != o.escape_radius_mode) {
            throw Failure{"reference escape-radius mode does not match render options"};
        }
        if (max_iter > ctx->requested_max_iter) throw Failure{"render iteration count exceeds prepared reference"};
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        Outputs out;
        out.field = field;
        out.counts = counts;
        wait_scratch(rt, stream);
        if (form == 1) {
            render_floatexp_from_reference(*ctx, out, width, height, zoom_text, max_iter, series_order, series_block,
                                           o, rt, stream);
        } else {
            render_from_reference(*ctx, out, width, height, zoom_text, max_iter, series_order, series_block, o, false,
                                  rt, stream);
        }
        release_scratch(rt, stream);
    });
}

int fractal_gb300_render_direct_device(float* field, uint32_t* counts, int width, int height, const char* zoom_text,
                                       const char* x_center, const char* y_center, int max_iter, int formula,
                                       double julia_real, double julia_imag, const FractalRenderOptions* supplied,
                                       void* stream_handle) {
    return guarded("device direct render failed with an unknown exception", [&] {
        if (!field || !zoom_text || !x_center || !y_center || !valid_dims(width, height)
            || !valid_iterations(max_iter) || !valid_formula(formula) || !std::isfinite(julia_real)
            || !std::isfinite(julia_imag)) {
            throw Failure{"invalid native render dimensions, formula, or argument"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        Outputs out;
        out.field = field;
        out.counts = counts;
        wait_scratch(rt, stream);
        launch_direct_render(out, width, height, parse_zoom_direct(zoom_text), parse_coordinate(x_center, "real"),
                             parse_coordinate(y_center, "imaginary"), max_iter, formula, julia_real, julia_imag, o,
                             stream);
        release_scratch(rt, stream);
    });
}

int fractal_gb300_colourise_device(const float* field, uint8_t* rgb, int width, int height, int max_iter,
                                   double phase, double vocal, double instrumental, double pitch,
                                   void* stream_handle) {
    return guarded("device colour failed with an unknown exception", [&] {
        if (!field || !rgb || !valid_dims(width, height) || !valid_iterations(max_iter)
            || !valid_colour_controls(phase, vocal, instrumental, pitch)) {
            throw Failure{"invalid native colour dimensions or palette"};
        }
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        int lut_size = 0;
        wait_scratch(rt, rt.stream);
        const std::uint8_t* lut = aurora_lut(rt, max_iter, phase, vocal, pitch, lut_size);
        const float scale = static_cast<float>(lut_size - 1) / static_cast<float>(max_iter);
        check_cuda(cudaStreamSynchronize(rt.stream), "aurora palette");
        check_cuda(launch_aurora(field, rgb, static_cast<long long>(width) * height, lut, lut_size, scale, max_iter,
                                 stream), "aurora kernel launch");
        release_scratch(rt, stream);
    });
}

int fractal_gb300_render_keyframes_device(const FractalGb300Keyframe* frames, int count, int width, int height,
                                          const char* x_center, const char* y_center, int series_order,
                                          int series_block, const FractalRenderOptions* supplied, int form,
                                          unsigned flags, void* stream_handle) {
    return guarded("keyframe batch render failed with an unknown exception", [&] {
        if (!frames || count <= 0 || !valid_dims(width, height)) throw Failure{"invalid native keyframe batch"};
        std::vector<FieldRequest> fields(static_cast<std::size_t>(count));
        for (int i = 0; i < count; ++i) {
            FieldRequest& f = fields[static_cast<std::size_t>(i)];
            f.out.field = frames[i].field;
            f.out.counts = frames[i].counts;
            f.zoom_text = frames[i].zoom_text;
            f.reference = frames[i].reference;
            f.width = width;
            f.height = height;
            f.max_iter = frames[i].max_iter;
            f.flags = frames[i].flags;
        }
        render_field_batch(fields, x_center, y_center, series_order, series_block, supplied, form, flags,
                           stream_handle);
    });
}

int fractal_gb300_render_fields_device(const FractalGb300Field* frames, int count, const char* x_center,
                                       const char* y_center, int series_order, int series_block,
                                       const FractalRenderOptions* supplied, int form, unsigned flags,
                                       void* stream_handle) {
    return guarded("field batch render failed with an unknown exception", [&] {
        if (!frames || count <= 0) throw Failure{"invalid native field batch"};
        std::vector<FieldRequest> fields(static_cast<std::size_t>(count));
        for (int i = 0; i < count; ++i) {
            FieldRequest& f = fields[static_cast<std::size_t>(i)];
            if ((frames[i].de_x == nullptr) != (frames[i].de_y == nullptr)) {
                throw Failure{"native field " + std::to_string(i) + " names one derivative plane without the other"};
            }
            f.out.field = frames[i].field;
            f.out.counts = frames[i].counts;
            f.out.p_dex = frames[i].de_x;
            f.out.p_dey = frames[i].de_y;
            f.zoom_text = frames[i].zoom_text;
            f.reference = frames[i].reference;
            f.width = frames[i].width;
            f.height = frames[i].height;
            f.max_iter = frames[i].max_iter;
            f.flags = frames[i].flags;
        }
        render_field_batch(fields, x_center, y_center, series_order, series_block, supplied, form, flags,
                           stream_handle);
    });
}

int fractal_gb300_set_queue_shapes(const int* values, int count) {
    return guarded("queue shape setting failed", [&] {
        ThreadRuntime& rt = thread_runtime();
        if (!values || count <= 0) {
            rt.shapes_pinned = false;
            return;
        }
        if (count < 4) throw Failure{"queue shapes need four values"};
        for (int i = 0; i < 4; ++i) {
            if (values[i] < 0 || values[i] > (i % 2 == 0 ? 1 << 20 : 64)) throw Failure{"queue shape out of range"};
            rt.pinned_shapes[i] = values[i];
        }
        rt.shapes_pinned = true;
    });
}

int fractal_gb300_set_cost_network(void* net) {
    return guarded("attaching the cost network failed", [&] { thread_runtime().costnet = net; });
}

int fractal_gb300_last_tiles(int* tiles, float* cost, uint16_t* features, int capacity, double* timing_ms) {
    return guarded("reading the last tile schedule failed", [&] {
        ThreadRuntime& rt = thread_runtime();
        if (rt.last_tiles <= 0) throw Failure{"no tile-scheduled batch has run on this thread"};
        if (tiles) *tiles = rt.last_tiles;
        if ((cost || features) && capacity < rt.last_tiles) throw Failure{"tile buffer too small"};
        check_cuda(cudaStreamSynchronize(rt.tile_stream ? rt.tile_stream : rt.stream), "tile batch");
        const int rows = (rt.last_tiles + 127) / 128 * 128;
        const TileBuffers t = tile_buffers(static_cast<char*>(scratch(rt, kScratchTiles, 1)), rt.last_tiles, rows);
        if (cost) {
            std::vector<unsigned long long> cycles(rt.last_tiles);
            check_cuda(cudaMemcpy(cycles.data(), t.cost, cycles.size() * sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost), "tile costs");
            for (int i = 0; i < rt.last_tiles; ++i) cost[i] = static_cast<float>(cycles[i]);
        }
        if (features) {
            check_cuda(cudaMemcpy(features, t.features,
                                  sizeof(std::uint16_t) * static_cast<std::size_t>(rt.last_tiles) * mlp::kFeatures,
                                  cudaMemcpyDeviceToHost), "tile features");
        }
        if (timing_ms) {
            unsigned long long ns[3];
            check_cuda(cudaMemcpy(ns, t.timing, sizeof ns, cudaMemcpyDeviceToHost), "tile timing");
            timing_ms[0] = static_cast<double>(ns[2] - ns[0]) * 1e-6;
            timing_ms[1] = static_cast<double>(ns[2] - ns[1]) * 1e-6;
        }
    });
}

int fractal_gb300_last_direct_steps(unsigned long long* steps) {
    return guarded("reading the direct queue's step count failed", [&] {
        if (!steps) throw Failure{"null step counter"};
        if (!runtime_made) throw Failure{"no direct batch has run on this thread"};
        if (last_direct_noalloc) {
            throw Failure{"the calling thread's last direct launch was a no-allocation render, whose counters "
                          "are not kept"};
        }
        ThreadRuntime& rt = thread_runtime();
        if (!rt.scratch[kScratchDirect]) throw Failure{"no direct batch has run on this thread"};
        check_cuda(cudaStreamSynchronize(rt.batch_stream ? rt.batch_stream : rt.stream), "keyframe batch");
        check_cuda(cudaStreamSynchronize(rt.side), "keyframe batch");
        const auto* counters = static_cast<const unsigned long long*>(rt.scratch[kScratchDirect]);
        check_cuda(cudaMemcpy(steps, counters + kStepsExecuted, sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost), "direct step count");
        unsigned long long error = 0;
        check_cuda(cudaMemcpy(&error, counters + kQueueError, sizeof error, cudaMemcpyDeviceToHost),
                   "direct queue status");
        if (error) throw Failure{"direct queue: a spilled pixel was never published (render incomplete)"};
    });
}

int fractal_gb300_set_direct_fault_injection(int spin_limit, int withhold_publish) {
    return guarded("setting the direct queue's fault injection failed", [&] {
        if (spin_limit < 0 || spin_limit > (1 << 22) || (withhold_publish != 0 && withhold_publish != 1)) {
            throw Failure{"direct queue fault injection out of range"};
        }
        set_direct_fault_injection(spin_limit, withhold_publish);
    });
}

int fractal_gb300_queue_shapes(int* values, int capacity) {
    return guarded("queue shape query failed", [&] {
        if (!values || capacity < 4) throw Failure{"queue shape buffer too small"};
        ThreadRuntime& rt = thread_runtime();
        for (int i = 0; i < 4; ++i) values[i] = rt.last_shapes[i];
    });
}

int fractal_gb300_render_direct_device_noalloc(float* field, uint32_t* counts, int width, int height,
                                               const char* zoom_text, const char* x_center, const char* y_center,
                                               int max_iter, int formula, double julia_real, double julia_imag,
                                               const FractalRenderOptions* supplied, void* stream_handle) {
    return guarded("no-allocation direct render failed with an unknown exception", [&] {
        if (!field || !zoom_text || !x_center || !y_center || !valid_dims(width, height)
            || !valid_iterations(max_iter) || !valid_formula(formula) || !std::isfinite(julia_real)
            || !std::isfinite(julia_imag)) {
            throw Failure{"invalid native render dimensions, formula, or argument"};
        }
        const FractalRenderOptions o = checked_options(supplied);
        check_backend(o);
        Outputs out;
        out.field = field;
        out.counts = counts;
        const DirectParams p = make_direct_params(out, width, height, parse_zoom_direct(zoom_text),
                                                  parse_coordinate(x_center, "real"),
                                                  parse_coordinate(y_center, "imaginary"), max_iter, formula,
                                                  julia_real, julia_imag, o);
        std::string why;
        if (!launch_direct_noalloc(p, static_cast<cudaStream_t>(stream_handle), why)) throw Failure{why};
        last_direct_noalloc = true;
    });
}

// ------------------------------------------------------ tile-cost network

void* fractal_gb300_costnet_create(unsigned seed) {
    return guarded_handle("cost network creation failed", [&]() -> void* {
        thread_runtime();
        std::string why;
        mlp::CostNet* net = mlp::create(seed, why);
        if (!net) throw Failure{why};
        return net;
    });
}

void fractal_gb300_costnet_destroy(void* net) { mlp::destroy(static_cast<mlp::CostNet*>(net)); }

int fractal_gb300_costnet_parameter_count(void) { return static_cast<int>(mlp::parameter_count()); }

int fractal_gb300_costnet_parameters(void* net, float* values, int count, int write) {
    return guarded("cost network parameter access failed", [&] {
        if (!net || !values || count != static_cast<int>(mlp::parameter_count())) {
            throw Failure{"cost network parameter buffer must hold exactly the parameter count"};
        }
        std::string why;
        auto* n = static_cast<mlp::CostNet*>(net);
        if (write) {
            if (!mlp::set_parameters(n, values, static_cast<std::size_t>(count), why)) throw Failure{why};
        } else {
            std::vector<float> host;
            if (!mlp::get_parameters(n, host, why)) throw Failure{why};
            std::memcpy(values, host.data(), host.size() * sizeof(float));
        }
    });
}

int fractal_gb300_costnet_train_step(void* net, const void* features, const float* targets, int batch,
                                     float learning_rate, int update, float* loss, float* gradients,
                                     void* stream_handle) {
    return guarded("cost network training step failed", [&] {
        if (!net || !features || !targets) throw Failure{"invalid cost network training arguments"};
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        std::string why;
        std::vector<float> grads;
        float host_loss = 0.0f;
        if (!mlp::train_step(static_cast<mlp::CostNet*>(net), static_cast<const __nv_bfloat16*>(features), targets,
                             batch, learning_rate, update != 0, &host_loss, gradients ? &grads : nullptr, stream,
                             why)) {
            throw Failure{why};
        }
        if (loss) *loss = host_loss;
        if (gradients) std::memcpy(gradients, grads.data(), grads.size() * sizeof(float));
    });
}

int fractal_gb300_costnet_predict(void* net, const void* features, int rows, float* out, void* stream_handle) {
    return guarded("cost network prediction failed", [&] {
        if (!net || !features || !out) throw Failure{"invalid cost network prediction arguments"};
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        std::string why;
        if (!mlp::predict(static_cast<mlp::CostNet*>(net), static_cast<const __nv_bfloat16*>(features), rows, out,
                          stream, why)) {
            throw Failure{why};
        }
    });
}

int fractal_gb300_gemm_bf16(const void* a, const void* b, float* c, int m, int n, int k, int b_rows,
                            void* stream_handle) {
    return guarded("tensor-core GEMM failed", [&] {
        if (!a || !b || !c) throw Failure{"invalid GEMM arguments"};
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        int* error = static_cast<int*>(scratch(rt, kScratchWork, 256));
        check_cuda(cudaMemsetAsync(error, 0, sizeof(int), stream), "cudaMemsetAsync");
        mlp::Epilogue e;
        std::memset(&e, 0, sizeof e);
        e.out_f32 = c;
        e.ld_out = n;
        e.rows = m;
        e.cols = n;
        std::string why;
        if (!mlp::gemm(mlp::GemmShape{a, b, m, n, k, b_rows}, e, error, stream, why)) throw Failure{why};
        int flag = 0;
        check_cuda(cudaMemcpyAsync(&flag, error, sizeof flag, cudaMemcpyDeviceToHost, stream), "GEMM status");
        check_cuda(cudaStreamSynchronize(stream), "GEMM");
        if (flag) throw Failure{"tensor-core GEMM gave up waiting on its barrier"};
    });
}

// fractal_atlas_field_ex (renderer.h:815-836, renderer.cpp:18697-18888).
int fractal_atlas_field_ex(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                           const float* child, int child_width, int child_height, int child_max_iter, float* output,
                           int output_width, int output_height, double parent_zoom, double child_fraction,
                           double child_zoom, double parent_field_bias, double child_field_bias,
                           double output_field_bias, int palette_max_iter, int feather, int threads) {
    return guarded("native scalar atlas compositor failed with an unknown exception", [&] {
        if (!parent || !output || !valid_threads(threads)) throw Failure{"invalid native scalar atlas dimensions"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction,
                             palette_max_iter};
        AtlasLaunch a = atlas_field_launch(r, child_zoom, parent_field_bias, child_field_bias, output_field_bias,
                                           feather);
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        atlas_from_host(rt, a, parent, child, output, true);
    });
}

// fractal_atlas_field (renderer.h:797-813): the extended call with no
// biases, child zoom 1 and a 48-pixel seam.
int fractal_atlas_field(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                        const float* child, int child_width, int child_height, int child_max_iter, float* output,
                        int output_width, int output_height, double parent_zoom, double child_fraction,
                        int palette_max_iter, int threads) {
    return fractal_atlas_field_ex(parent, parent_width, parent_height, parent_max_iter, child, child_width,
                                  child_height, child_max_iter, output, output_width, output_height, parent_zoom,
                                  child_fraction, 1.0, 0.0, 0.0, 0.0, palette_max_iter, 48, threads);
}

}  // extern "C"

namespace {

int atlas_colourise_common(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                           const float* child, int child_width, int child_height, int child_max_iter,
                           uint8_t* output, int output_width, int output_height, double parent_zoom,
                           double child_fraction, int palette_max_iter, double phase, double vocal,
                           double instrumental, double pitch, int threads, const int* interior_color,
                           const std::uint8_t* accents) {
    return guarded("native atlas colouriser failed with an unknown exception", [&] {
        if (!parent || !output || !valid_threads(threads)) throw Failure{"invalid native atlas dimensions or controls"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction,
                             palette_max_iter};
        AtlasLaunch a = atlas_colour_launch(r, phase, vocal, instrumental, pitch, interior_color);
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        attach_aurora(rt, a, phase, vocal, pitch, accents);
        atlas_from_host(rt, a, parent, child, output, false);
    });
}

}  // namespace

extern "C" {

// fractal_atlas_colourise (renderer.h:997-1017, renderer.cpp:19138-19455).
int fractal_atlas_colourise(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                            const float* child, int child_width, int child_height, int child_max_iter,
                            uint8_t* output, int output_width, int output_height, double parent_zoom,
                            double child_fraction, int palette_max_iter, double phase, double vocal,
                            double instrumental, double pitch, int threads) {
    return atlas_colourise_common(parent, parent_width, parent_height, parent_max_iter, child, child_width,
                                  child_height, child_max_iter, output, output_width, output_height, parent_zoom,
                                  child_fraction, palette_max_iter, phase, vocal, instrumental, pitch, threads,
                                  nullptr, nullptr);
}

// fractal_atlas_colourise_interior (renderer.h:1018-1042): the same with an
// explicit interior colour.
int fractal_atlas_colourise_interior(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                                     const float* child, int child_width, int child_height, int child_max_iter,
                                     uint8_t* output, int output_width, int output_height, double parent_zoom,
                                     double child_fraction, int palette_max_iter, double phase, double vocal,
                                     double instrumental, double pitch, int interior_red, int interior_green,
                                     int interior_blue, int threads) {
    const int interior[3] = {interior_red, interior_green, interior_blue};
    return atlas_colourise_common(parent, parent_width, parent_height, parent_max_iter, child, child_width,
                                  child_height, child_max_iter, output, output_width, output_height, parent_zoom,
                                  child_fraction, palette_max_iter, phase, vocal, instrumental, pitch, threads,
                                  interior, nullptr);
}

// fractal_atlas_colourise_accents (renderer.h:1043-1067): the aurora waves
// projected through three RGB accents, with an interior colour.
int fractal_atlas_colourise_accents(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                                    const float* child, int child_width, int child_height, int child_max_iter,
                                    uint8_t* output, int output_width, int output_height, double parent_zoom,
                                    double child_fraction, int palette_max_iter, double phase, double vocal,
                                    double instrumental, double pitch, const uint8_t* accents, int interior_red,
                                    int interior_green, int interior_blue, int threads) {
    if (accents == nullptr) {
        set_error("ordinary palette accents are required");
        return 1;
    }
    const int interior[3] = {interior_red, interior_green, interior_blue};
    return atlas_colourise_common(parent, parent_width, parent_height, parent_max_iter, child, child_width,
                                  child_height, child_max_iter, output, output_width, output_height, parent_zoom,
                                  child_fraction, palette_max_iter, phase, vocal, instrumental, pitch, threads,
                                  interior, accents);
}

// fractal_atlas_colourise_kfp_raw (renderer.h:663-687, renderer.cpp:
// 17969-18304): the parent and child composed into one scalar surface
// (device, L2-resident at 4K), then one KFP colour pass over it.
int fractal_atlas_colourise_kfp_raw(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                                    const float* child, int child_width, int child_height, int child_max_iter,
                                    uint8_t* output, int output_width, int output_height, double parent_zoom,
                                    double child_fraction, double child_zoom, int max_iter, double phase,
                                    double vocal, double instrumental, double pitch,
                                    const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                    int threads) {
    return guarded("native raw KFP atlas colourizer failed with an unknown exception", [&] {
        if (!parent || !output || !valid_threads(threads)) {
            throw Failure{"invalid native raw KFP atlas dimensions or controls"};
        }
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction, 0};
        AtlasLaunch a = kfp_raw_launch(r, child_zoom, max_iter, phase, vocal, instrumental, pitch, options, lut,
                                       lut_size);
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        void* tables = stage_atlas_sources(rt, a, parent, child);
        const std::size_t pixels = static_cast<std::size_t>(output_width) * output_height;
        a.field_out = static_cast<float*>(scratch(rt, kScratchSurface, pixels * sizeof(float)));
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, *options, lut, lut_size, false);
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        check_cuda(run_atlas(rt, a, tables, rt.stream), "atlas surface launch");
        kfp_colour(a.field_out, d_rgb, output_width, output_height, max_iter, *options, in, lut_size, rt, rt.stream);
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream),
                   "copy atlas RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "raw KFP atlas");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

// fractal_atlas_colourise_kfp (renderer.h:554-576, renderer.cpp:
// 16750-17321): parent and child coloured as separate KFP tiles at output
// scale, each with its own stencil edges and ColorMethod 4 bounds, the child
// over its rectangle with a smoothstep band of `feather` pixels.
int fractal_atlas_colourise_kfp(const float* parent, int parent_width, int parent_height, const float* child,
                                int child_width, int child_height, uint8_t* output, int output_width,
                                int output_height, int max_iter, int child_left, int child_top, int feather,
                                double phase, double vocal, double instrumental, double pitch,
                                const FractalKfpOptions* options, const uint8_t* lut, int lut_size, int threads) {
    return guarded("native KFP atlas colouriser failed with an unknown exception", [&] {
        if (!parent || !output || !valid_dims(parent_width, parent_height) || !valid_dims(output_width, output_height)
            || parent_width != output_width || parent_height != output_height || !valid_iterations(max_iter)
            || !valid_threads(threads) || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut
            || !valid_kfp(options, lut_size)) {
            throw Failure{"invalid native KFP atlas dimensions or controls"};
        }
        const bool use_child = child != nullptr;
        if (use_child) {
            if (!valid_dims(child_width, child_height) || child_left < 0 || child_top < 0
                || child_width > output_width - child_left || child_height > output_height - child_top || feather < 0
                || feather > std::min(child_width, child_height)) {
                throw Failure{"invalid native KFP atlas child rectangle"};
            }
        } else if (child_width != 0 || child_height != 0 || child_left != 0 || child_top != 0 || feather != 0) {
            throw Failure{"invalid native KFP atlas child absence"};
        }
        const FractalKfpOptions& o = *options;
        if (o.field_bias > static_cast<double>(max_iter)) throw Failure{"native KFP field bias exceeds iteration cap"};
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        auto up = [](std::size_t v) { return (v + 255) / 256 * 256; };
        const std::size_t pixels = static_cast<std::size_t>(output_width) * output_height;
        const std::size_t child_pixels = use_child ? static_cast<std::size_t>(child_width) * child_height : 0;
        char* base = static_cast<char*>(scratch(rt, kScratchAtlas, up(pixels * 4) + up(child_pixels * 4)));
        check_cuda(cudaMemcpyAsync(base, parent, pixels * 4, cudaMemcpyHostToDevice, rt.stream), "atlas parent");
        float* d_child = reinterpret_cast<float*>(base + up(pixels * 4));
        if (use_child) {
            check_cuda(cudaMemcpyAsync(d_child, child, child_pixels * 4, cudaMemcpyHostToDevice, rt.stream),
                       "atlas child");
        }
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, o, lut, lut_size, false);
        KfpLaunch k = kfp_constants(o, output_width, output_height, max_iter, lut_size);
        KfpAtlasLaunch at{};
        at.parent = reinterpret_cast<const float*>(base);
        at.child = use_child ? d_child : nullptr;
        at.child_width = child_width;
        at.child_height = child_height;
        at.child_left = child_left;
        at.child_top = child_top;
        at.feather = feather;
        at.child_transfer_min = 0.0;
        at.child_transfer_max = 1.0;
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        if (o.color_method == 4) {
            kfp_transfer_bounds(rt, at.parent, static_cast<long long>(pixels), max_iter, o, k.smooth_offset, rt.stream,
                                k.transfer_min, k.transfer_max);
            if (use_child) {
                kfp_transfer_bounds(rt, d_child, static_cast<long long>(child_pixels), max_iter, o, k.smooth_offset,
                                    rt.stream, at.child_transfer_min, at.child_transfer_max);
            }
        }
        check_cuda(launch_kfp_atlas(at, d_rgb, k, in.lut, in.period, in.type, rt.stream), "KFP atlas launch");
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream),
                   "copy atlas RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "KFP atlas");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

// fractal_atlas_colourise_kfp_precise (renderer.h:577-603): the same pass
// under its compatibility name.
int fractal_atlas_colourise_kfp_precise(const float* parent, int parent_width, int parent_height, const float* child,
                                        int child_width, int child_height, uint8_t* output, int output_width,
                                        int output_height, int max_iter, int child_left, int child_top, int feather,
                                        double phase, double vocal, double instrumental, double pitch,
                                        const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                        int threads) {
    return fractal_atlas_colourise_kfp(parent, parent_width, parent_height, child, child_width, child_height, output,
                                       output_width, output_height, max_iter, child_left, child_top, feather, phase,
                                       vocal, instrumental, pitch, options, lut, lut_size, threads);
}

// fractal_atlas_colourise_kfp_planes (renderer.h:604-631, renderer.cpp:
// 17323-17783): the scalar surface and every present render plane of the
// primary tile (the child when it fills the frame) reprojected to the
// output, the child blended in over its rectangle, then the plane-aware KFP
// pass over the composed frame.
int fractal_atlas_colourise_kfp_planes(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                                       const FractalKfpPlanes* parent_planes, const float* child, int child_width,
                                       int child_height, int child_max_iter, const FractalKfpPlanes* child_planes,
                                       uint8_t* output, int output_width, int output_height, double parent_zoom,
                                       double child_fraction, double child_zoom, int max_iter, int centered_input,
                                       double phase, double vocal, double instrumental, double pitch,
                                       const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                       int threads) {
    return guarded("native plane-aware KFP atlas colourizer failed with an unknown exception", [&] {
        if (!parent || !output || !parent_planes || !valid_dims(parent_width, parent_height)
            || !valid_dims(output_width, output_height) || !valid_iterations(parent_max_iter)
            || !valid_iterations(max_iter) || !valid_threads(threads) || centered_input < 0 || centered_input > 1
            || !std::isfinite(parent_zoom) || parent_zoom <= 0.0 || !std::isfinite(child_fraction)
            || child_fraction < 0.0 || child_fraction > 1.0 || !std::isfinite(child_zoom) || child_zoom <= 0.0
            || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut || !valid_kfp(options, lut_size)
            || !valid_kfp_planes(parent_planes, parent_width, parent_height)) {
            throw Failure{"invalid native plane-aware KFP atlas dimensions or controls"};
        }
        const bool use_child = child != nullptr && child_fraction > 0.0;
        if (use_child) {
            if (!valid_dims(child_width, child_height) || !valid_iterations(child_max_iter) || !child_planes
                || !valid_kfp_planes(child_planes, child_width, child_height)) {
                throw Failure{"invalid native plane-aware KFP atlas child tile"};
            }
        } else if (child != nullptr || child_planes != nullptr || child_width != 0 || child_height != 0
                   || child_max_iter != 0) {
            throw Failure{"invalid native plane-aware KFP atlas child absence"};
        }
        const FractalKfpOptions& o = *options;
        if (o.field_bias > static_cast<double>(max_iter)) throw Failure{"native KFP field bias exceeds iteration cap"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction, 0};
        AtlasLaunch a = atlas_geometry(r);
        a.mode = kAtlasKfpPlanes;
        a.parent_zoom = std::max(parent_zoom, 1.0);
        a.child_zoom = std::max(child_zoom, 1.0);
        a.parent_bias = centered_input ? static_cast<double>(parent_max_iter) : 0.0;
        a.child_bias = centered_input ? static_cast<double>(child_max_iter) : 0.0;
        a.output_bias = o.field_bias;
        const int target_max_iter = a.full_child ? child_max_iter : max_iter;
        a.effective_iter = target_max_iter;
        const bool secondary = a.use_child && !a.full_child;
        a.feather = secondary ? kfp_seam_feather(a.child_visible_width, a.child_visible_height) : 0;
        const FractalKfpPlanes* primary_planes = a.full_child ? child_planes : parent_planes;
        const FractalKfpPlanes* secondary_planes = secondary ? child_planes : nullptr;
        // Texture coordinates are screen space: one source's image is kept.
        const FractalKfpPlanes* texture_planes = primary_planes;
        if (texture_planes->texture_rgb == nullptr && secondary_planes != nullptr
            && secondary_planes->texture_rgb != nullptr) {
            texture_planes = secondary_planes;
        }
        const bool texture = texture_planes->texture_rgb != nullptr && o.texture_enabled != 0;

        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        void* tables = stage_atlas_sources(rt, a, parent, child);
        auto up = [](std::size_t v) { return (v + 255) / 256 * 256; };
        const std::size_t pixels = static_cast<std::size_t>(output_width) * output_height;
        auto members = [](const FractalKfpPlanes* p, const void* out[9]) {
            const void* v[9] = {p ? p->orbit_iteration : nullptr, p ? p->iteration : nullptr, p ? p->bailout : nullptr,
                                p ? p->transition : nullptr, p ? p->phase : nullptr, p ? p->de_x : nullptr,
                                p ? p->de_y : nullptr, p ? p->test1 : nullptr, p ? p->test2 : nullptr};
            for (int i = 0; i < 9; ++i) out[i] = v[i];
        };
        const void* primary_host[9];
        const void* secondary_host[9];
        members(primary_planes, primary_host);
        members(secondary_planes, secondary_host);
        const std::size_t primary_pixels = a.full_child ? static_cast<std::size_t>(child_width) * child_height
                                                        : static_cast<std::size_t>(parent_width) * parent_height;
        const std::size_t secondary_pixels = secondary ? static_cast<std::size_t>(child_width) * child_height : 0;
        const std::size_t texture_size = texture ? texture_bytes(*texture_planes) : 0;
        std::size_t in_total = up(texture_size);
        std::size_t out_total = up(pixels * 8) + up(pixels) + up(pixels);
        for (int i = 0; i < 9; ++i) {
            in_total += (primary_host[i] ? up(primary_pixels * 8) : 0) + (secondary_host[i] ? up(secondary_pixels * 8) : 0);
            out_total += primary_host[i] || secondary_host[i] ? up(pixels * 8) : 0;
        }
        char* in_base = static_cast<char*>(scratch(rt, kScratchPlanesIn, in_total));
        char* out_base = static_cast<char*>(scratch(rt, kScratchPlanesOut, out_total));
        std::size_t in_at = 0, out_at = 0;
        auto put = [&](const void* data, std::size_t bytes) -> void* {
            void* dst = in_base + in_at;
            check_cuda(cudaMemcpyAsync(dst, data, bytes, cudaMemcpyHostToDevice, rt.stream), "upload planes");
            in_at += up(bytes);
            return dst;
        };
        auto take = [&](std::size_t bytes) -> void* {
            void* dst = out_base + out_at;
            out_at += up(bytes);
            return dst;
        };
        KfpPlaneSet primary{}, second{};
        KfpPlaneOutputs composed{};
        for (int i = 0; i < 9; ++i) {
            const void* pd = primary_host[i] ? put(primary_host[i], primary_pixels * 8) : nullptr;
            const void* sd = secondary_host[i] ? put(secondary_host[i], secondary_pixels * 8) : nullptr;
            void* od = primary_host[i] || secondary_host[i] ? take(pixels * 8) : nullptr;
            if (i < 2) {
                primary.ints[i] = static_cast<const long long*>(pd);
                second.ints[i] = static_cast<const long long*>(sd);
                composed.ints[i] = static_cast<long long*>(od);
            } else {
                primary.doubles[i - 2] = static_cast<const double*>(pd);
                second.doubles[i - 2] = static_cast<const double*>(sd);
                composed.doubles[i - 2] = static_cast<double*>(od);
            }
        }
        const void* d_texture = texture ? put(texture_planes->texture_rgb, texture_size) : nullptr;
        void* samples = take(pixels * 8);
        std::uint8_t* flags = static_cast<std::uint8_t*>(take(pixels));
        a.inside_out = static_cast<std::uint8_t*>(take(pixels));
        a.field_out = static_cast<float*>(scratch(rt, kScratchSurface, pixels * sizeof(float)));
        KfpPlanesLaunch pl{};
        pl.orbit_iteration = composed.ints[0];
        pl.iteration = composed.ints[1];
        pl.bailout = composed.doubles[0];
        pl.transition = composed.doubles[1];
        pl.phase = composed.doubles[2];
        pl.de_x = composed.doubles[3];
        pl.de_y = composed.doubles[4];
        pl.test1 = composed.doubles[5];
        pl.test2 = composed.doubles[6];
        plane_context(pl, o);
        if (texture) attach_texture(pl, *texture_planes, o, d_texture);
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, o, lut, lut_size, false);
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        check_cuda(run_atlas(rt, a, tables, rt.stream), "atlas surface launch");
        check_cuda(launch_atlas_planes(a, primary, second, composed, target_max_iter, rt.stream),
                   "atlas planes launch");
        if (pl.has_iteration) {
            check_cuda(launch_kfp_plane_samples(pl, target_max_iter, static_cast<long long>(pixels), samples, flags,
                                                rt.stream), "KFP plane samples launch");
        }
        kfp_colour(a.field_out, d_rgb, output_width, output_height, target_max_iter, o, in, lut_size, rt, rt.stream,
                   &pl, samples, flags);
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream),
                   "copy atlas RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "plane-aware KFP atlas");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

// fractal_atlas_colourise_kfp_planes_precise (renderer.h:632-662): the same
// pass under its compatibility name.
int fractal_atlas_colourise_kfp_planes_precise(const float* parent, int parent_width, int parent_height,
                                               int parent_max_iter, const FractalKfpPlanes* parent_planes,
                                               const float* child, int child_width, int child_height,
                                               int child_max_iter, const FractalKfpPlanes* child_planes,
                                               uint8_t* output, int output_width, int output_height,
                                               double parent_zoom, double child_fraction, double child_zoom,
                                               int max_iter, int centered_input, double phase, double vocal,
                                               double instrumental, double pitch, const FractalKfpOptions* options,
                                               const uint8_t* lut, int lut_size, int threads) {
    return fractal_atlas_colourise_kfp_planes(parent, parent_width, parent_height, parent_max_iter, parent_planes,
                                              child, child_width, child_height, child_max_iter, child_planes, output,
                                              output_width, output_height, parent_zoom, child_fraction, child_zoom,
                                              max_iter, centered_input, phase, vocal, instrumental, pitch, options,
                                              lut, lut_size, threads);
}

// fractal_atlas_colourise_kfp_raw_precise (renderer.h:688-711): the same
// transfer under its compatibility name.
int fractal_atlas_colourise_kfp_raw_precise(const float* parent, int parent_width, int parent_height,
                                            int parent_max_iter, const float* child, int child_width,
                                            int child_height, int child_max_iter, uint8_t* output, int output_width,
                                            int output_height, double parent_zoom, double child_fraction,
                                            double child_zoom, int max_iter, double phase, double vocal,
                                            double instrumental, double pitch, const FractalKfpOptions* options,
                                            const uint8_t* lut, int lut_size, int threads) {
    return fractal_atlas_colourise_kfp_raw(parent, parent_width, parent_height, parent_max_iter, child, child_width,
                                           child_height, child_max_iter, output, output_width, output_height,
                                           parent_zoom, child_fraction, child_zoom, max_iter, phase, vocal,
                                           instrumental, pitch, options, lut, lut_size, threads);
}

// Device-pointer raw KFP atlas frame (no reference counterpart): device
// parent, child, LUT and RGB8 output; the surface lives in the thread's
// scratch.
int fractal_gb300_atlas_colourise_kfp_raw_device(const float* parent, int parent_width, int parent_height,
                                                 int parent_max_iter, const float* child, int child_width,
                                                 int child_height, int child_max_iter, uint8_t* output,
                                                 int output_width, int output_height, double parent_zoom,
                                                 double child_fraction, double child_zoom, int max_iter,
                                                 const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                                 void* stream_handle) {
    return guarded("device raw KFP atlas failed with an unknown exception", [&] {
        if (!parent || !output) throw Failure{"invalid native raw KFP atlas dimensions or controls"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction, 0};
        AtlasLaunch a = kfp_raw_launch(r, child_zoom, max_iter, 0.0, 0.0, 0.0, 0.0, options, lut, lut_size);
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        wait_scratch(rt, rt.stream);
        bool uploaded = false;
        const KfpDeviceInputs in = kfp_inputs(rt, *options, lut, lut_size, true, &uploaded);
        if (uploaded) check_cuda(cudaStreamSynchronize(rt.stream), "KFP inputs");
        wait_scratch(rt, stream);
        a.parent = parent;
        a.child = child;
        const std::size_t pixels = static_cast<std::size_t>(output_width) * output_height;
        a.field_out = static_cast<float*>(scratch(rt, kScratchSurface, pixels * sizeof(float)));
        void* tables = scratch(rt, kScratchAtlas, atlas_table_bytes(a));
        check_cuda(run_atlas(rt, a, tables, stream), "atlas surface launch");
        kfp_colour(a.field_out, output, output_width, output_height, max_iter, *options, in, lut_size, rt, stream);
        release_scratch(rt, stream);
    });
}

// The raw KFP atlas surface alone (no reference counterpart): the scalar
// frame fractal_atlas_colourise_kfp_raw colours, into device `surface`, for
// callers that colour it later or differently.  `field_bias` is the KFP
// field bias (a positive bias means centred sources).
int fractal_gb300_atlas_kfp_surface_device(const float* parent, int parent_width, int parent_height,
                                           int parent_max_iter, const float* child, int child_width,
                                           int child_height, int child_max_iter, float* surface, int output_width,
                                           int output_height, double parent_zoom, double child_fraction,
                                           double child_zoom, int max_iter, double field_bias, void* stream_handle) {
    return guarded("device raw KFP atlas failed with an unknown exception", [&] {
        if (!parent || !surface || !std::isfinite(field_bias) || field_bias < 0.0) {
            throw Failure{"invalid native raw KFP atlas dimensions or controls"};
        }
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction, 0};
        try {
            check_atlas_common(r);
        } catch (const Failure&) {
            throw Failure{"invalid native raw KFP atlas dimensions or controls"};
        }
        if (!valid_iterations(max_iter) || !std::isfinite(child_zoom) || child_zoom <= 0.0) {
            throw Failure{"invalid native raw KFP atlas dimensions or controls"};
        }
        AtlasLaunch a = kfp_surface_launch(r, child_zoom, max_iter, field_bias);
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        wait_scratch(rt, stream);
        a.parent = parent;
        a.child = child;
        a.field_out = surface;
        void* tables = scratch(rt, kScratchAtlas, atlas_table_bytes(a));
        check_cuda(run_atlas(rt, a, tables, stream), "atlas surface launch");
        release_scratch(rt, stream);
    });
}

// fractal_crop_field (renderer.h:786-795, renderer.cpp:18631-18696): plain
// bilinear crop of one field by `zoom_factor` (at least 1) about its centre.
int fractal_crop_field(const float* source, int source_width, int source_height, float* output, int output_width,
                       int output_height, double zoom_factor, int threads) {
    return guarded("native raw-field crop failed with an unknown exception", [&] {
        if (!source || !output || !valid_dims(source_width, source_height) || !valid_dims(output_width, output_height)
            || !valid_threads(threads) || !std::isfinite(zoom_factor) || zoom_factor <= 0.0) {
            throw Failure{"invalid native raw-field crop dimensions"};
        }
        AtlasLaunch a{};
        a.mode = kAtlasCropField;
        a.parent_width = source_width;
        a.parent_height = source_height;
        a.parent_zoom = std::max(zoom_factor, 1.0);
        a.out_width = output_width;
        a.out_height = output_height;
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        atlas_from_host(rt, a, source, nullptr, output, true);
    });
}

// fractal_crop_rgb (renderer.h:716-725, renderer.cpp:18399-18465): bilinear
// crop of an RGB8 image.
int fractal_crop_rgb(const uint8_t* source, int source_width, int source_height, uint8_t* output, int output_width,
                     int output_height, double zoom_factor, int threads) {
    return guarded("native RGB crop failed with an unknown exception", [&] {
        if (!source || !output || !valid_dims(source_width, source_height) || !valid_dims(output_width, output_height)
            || !valid_threads(threads) || !std::isfinite(zoom_factor) || zoom_factor <= 0.0) {
            throw Failure{"invalid native RGB crop dimensions"};
        }
        zoom_factor = std::max(zoom_factor, 1.0);
        if (source_width == output_width && source_height == output_height && zoom_factor == 1.0) {
            // The identity crop (renderer.cpp:18418-18427).
            std::memcpy(output, source, static_cast<std::size_t>(output_width) * output_height * 3);
            return;
        }
        AtlasLaunch a{};
        a.mode = kAtlasRgb;
        a.parent_width = source_width;
        a.parent_height = source_height;
        a.parent_zoom = zoom_factor;
        a.out_width = output_width;
        a.out_height = output_height;
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        atlas_from_host(rt, a, source, nullptr, output, false);
    });
}

// fractal_atlas_composite_rgb (renderer.h:726-741, renderer.cpp:18467-18629):
// already-coloured parent and child tiles composed with a double smoothstep
// seam of `feather` pixels.
int fractal_atlas_composite_rgb(const uint8_t* parent, int parent_width, int parent_height, const uint8_t* child,
                                int child_width, int child_height, uint8_t* output, int output_width,
                                int output_height, double parent_zoom, double child_fraction, double child_zoom,
                                int feather, int threads) {
    return guarded("native RGB atlas compositor failed with an unknown exception", [&] {
        if (!parent || !output || !valid_dims(parent_width, parent_height) || !valid_dims(output_width, output_height)
            || !valid_threads(threads) || !std::isfinite(parent_zoom) || parent_zoom <= 0.0
            || !std::isfinite(child_fraction) || child_fraction < 0.0 || child_fraction > 1.0
            || !std::isfinite(child_zoom) || child_zoom <= 0.0 || feather < 0) {
            throw Failure{"invalid native RGB atlas dimensions or controls"};
        }
        const bool use_child = child != nullptr && child_fraction > 0.0;
        if (!use_child && child_fraction > 0.0) throw Failure{"RGB atlas child data is missing for a positive fraction"};
        if (!use_child && child != nullptr) throw Failure{"RGB atlas child needs a positive visible fraction"};
        if (!use_child && (child_width != 0 || child_height != 0)) throw Failure{"invalid native RGB atlas child absence"};
        if (use_child && (!valid_dims(child_width, child_height) || feather > std::min(output_width, output_height))) {
            throw Failure{"invalid native RGB atlas child tile"};
        }
        const AtlasRequest r{parent_width, parent_height, 1, child_width, child_height, 1, use_child, output_width,
                             output_height, parent_zoom, child_fraction, 0};
        AtlasLaunch a = atlas_geometry(r);
        a.mode = kAtlasRgb;
        a.full_child = 0;
        a.parent_zoom = std::max(parent_zoom, 1.0);
        a.child_zoom = std::max(child_zoom, 1.0);
        a.feather = use_child ? std::min(feather, std::min(a.child_visible_width, a.child_visible_height)) : 0;
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        atlas_from_host(rt, a, parent, use_child ? child : nullptr, output, false);
    });
}

}  // extern "C"

namespace {

// crop_colourise_impl (renderer.cpp:18977-19020).
int crop_colourise_common(const float* source, int source_width, int source_height, uint8_t* output,
                          int output_width, int output_height, double zoom_factor, int max_iter, double phase,
                          double vocal, double instrumental, double pitch, int threads, const int* interior_color,
                          const std::uint8_t* accents) {
    return guarded("native crop colouriser failed with an unknown exception", [&] {
        if (!source || !output || !valid_dims(source_width, source_height) || !valid_dims(output_width, output_height)
            || !valid_iterations(max_iter) || !valid_threads(threads) || !std::isfinite(zoom_factor)
            || zoom_factor <= 0.0 || !valid_colour_controls(phase, vocal, instrumental, pitch)
            || (interior_color != nullptr
                && (interior_color[0] < 0 || interior_color[0] > 255 || interior_color[1] < 0
                    || interior_color[1] > 255 || interior_color[2] < 0 || interior_color[2] > 255))) {
            throw Failure{"invalid native crop/colour dimensions or palette"};
        }
        AtlasLaunch a{};
        a.mode = kAtlasCropAurora;
        a.parent_width = source_width;
        a.parent_height = source_height;
        a.parent_max_iter = max_iter;
        a.parent_zoom = std::max(zoom_factor, 1.0);
        a.out_width = output_width;
        a.out_height = output_height;
        a.palette_iter = max_iter;
        for (int c = 0; c < 3; ++c) a.interior[c] = interior_color ? interior_color[c] : 0;
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        attach_aurora(rt, a, phase, vocal, pitch, accents);
        atlas_from_host(rt, a, source, nullptr, output, false);
    });
}

// fractal_crop_colourise_kfp's crop, then the KFP pass (renderer.cpp:
// 17803-17967): the interior-preserving crop biased and encoded by the KFP
// field bias.
int crop_colourise_kfp_common(const float* source, int source_width, int source_height, uint8_t* output,
                              int output_width, int output_height, double zoom_factor, int max_iter, double phase,
                              double vocal, double instrumental, double pitch, const FractalKfpOptions* options,
                              const uint8_t* lut, int lut_size, int threads) {
    return guarded("native KFP crop colourizer failed with an unknown exception", [&] {
        if (!source || !output || !valid_dims(source_width, source_height) || !valid_dims(output_width, output_height)
            || !valid_iterations(max_iter) || !valid_threads(threads) || !std::isfinite(zoom_factor)
            || zoom_factor <= 0.0 || !valid_colour_controls(phase, vocal, instrumental, pitch) || !lut
            || !valid_kfp(options, lut_size)) {
            throw Failure{"invalid native KFP crop dimensions or controls"};
        }
        if (options->field_bias > static_cast<double>(max_iter)) {
            throw Failure{"native KFP field bias exceeds iteration cap"};
        }
        AtlasLaunch a{};
        a.mode = kAtlasKfpSurface;
        a.parent_width = source_width;
        a.parent_height = source_height;
        a.parent_max_iter = max_iter;
        a.parent_bias = options->field_bias;
        a.parent_zoom = std::max(zoom_factor, 1.0);
        a.out_width = output_width;
        a.out_height = output_height;
        a.output_bias = options->field_bias;
        a.effective_iter = max_iter;
        ThreadRuntime& rt = thread_runtime();
        wait_scratch(rt, rt.stream);
        void* tables = stage_atlas_sources(rt, a, source, nullptr);
        const std::size_t pixels = static_cast<std::size_t>(output_width) * output_height;
        a.field_out = static_cast<float*>(scratch(rt, kScratchSurface, pixels * sizeof(float)));
        std::uint8_t* d_rgb = static_cast<std::uint8_t*>(scratch(rt, kScratchRgb, pixels * 3));
        const KfpDeviceInputs in = kfp_inputs(rt, *options, lut, lut_size, false);
        check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
        check_cuda(run_atlas(rt, a, tables, rt.stream), "crop surface launch");
        kfp_colour(a.field_out, d_rgb, output_width, output_height, max_iter, *options, in, lut_size, rt, rt.stream);
        check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
        check_cuda(cudaMemcpyAsync(output, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, rt.stream),
                   "copy crop RGB to host");
        check_cuda(cudaStreamSynchronize(rt.stream), "KFP crop");
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt.start, rt.stop) == cudaSuccess) rt.last_kernel_ms = ms;
    });
}

}  // namespace

extern "C" {

// fractal_crop_colourise (renderer.h:943-956).
int fractal_crop_colourise(const float* source, int source_width, int source_height, uint8_t* output,
                           int output_width, int output_height, double zoom_factor, int max_iter, double phase,
                           double vocal, double instrumental, double pitch, int threads) {
    return crop_colourise_common(source, source_width, source_height, output, output_width, output_height,
                                 zoom_factor, max_iter, phase, vocal, instrumental, pitch, threads, nullptr, nullptr);
}

// fractal_crop_colourise_interior (renderer.h:957-975).
int fractal_crop_colourise_interior(const float* source, int source_width, int source_height, uint8_t* output,
                                    int output_width, int output_height, double zoom_factor, int max_iter,
                                    double phase, double vocal, double instrumental, double pitch, int interior_red,
                                    int interior_green, int interior_blue, int threads) {
    const int interior[3] = {interior_red, interior_green, interior_blue};
    return crop_colourise_common(source, source_width, source_height, output, output_width, output_height,
                                 zoom_factor, max_iter, phase, vocal, instrumental, pitch, threads, interior, nullptr);
}

// fractal_crop_colourise_accents (renderer.h:976-996); NULL accents give the
// plain aurora palette, as in the reference.
int fractal_crop_colourise_accents(const float* source, int source_width, int source_height, uint8_t* output,
                                   int output_width, int output_height, double zoom_factor, int max_iter,
                                   double phase, double vocal, double instrumental, double pitch,
                                   const uint8_t* accents, int interior_red, int interior_green, int interior_blue,
                                   int threads) {
    const int interior[3] = {interior_red, interior_green, interior_blue};
    return crop_colourise_common(source, source_width, source_height, output, output_width, output_height,
                                 zoom_factor, max_iter, phase, vocal, instrumental, pitch, threads, interior, accents);
}

// fractal_crop_colourise_kfp (renderer.h:518-535) and its compatibility name
// (renderer.h:536-553).
int fractal_crop_colourise_kfp(const float* source, int source_width, int source_height, uint8_t* output,
                               int output_width, int output_height, double zoom_factor, int max_iter, double phase,
                               double vocal, double instrumental, double pitch, const FractalKfpOptions* options,
                               const uint8_t* lut, int lut_size, int threads) {
    return crop_colourise_kfp_common(source, source_width, source_height, output, output_width, output_height,
                                     zoom_factor, max_iter, phase, vocal, instrumental, pitch, options, lut, lut_size,
                                     threads);
}

int fractal_crop_colourise_kfp_precise(const float* source, int source_width, int source_height, uint8_t* output,
                                       int output_width, int output_height, double zoom_factor, int max_iter,
                                       double phase, double vocal, double instrumental, double pitch,
                                       const FractalKfpOptions* options, const uint8_t* lut, int lut_size,
                                       int threads) {
    return crop_colourise_kfp_common(source, source_width, source_height, output, output_width, output_height,
                                     zoom_factor, max_iter, phase, vocal, instrumental, pitch, options, lut, lut_size,
                                     threads);
}

// Pixels of the last atlas frame on this thread that the fast pass left to
// the exact FP64 pass (synchronises with the device); -1 before any frame.
long long fractal_gb300_atlas_last_exact_pixels(void) {
    try {
        ThreadRuntime& rt = thread_runtime();
        if (rt.atlas_exact_count == nullptr) return -1;
        unsigned count = 0;
        check_cuda(cudaDeviceSynchronize(), "atlas exact count");
        check_cuda(cudaMemcpy(&count, rt.atlas_exact_count, sizeof count, cudaMemcpyDeviceToHost), "atlas exact count");
        return static_cast<long long>(count);
    } catch (...) {
        return -1;
    }
}

// Video-frame handoff (no reference counterpart): device RGB8 packed into
// the encoder pipe's layout (rgb24, rgb0, rgba, yuv420p, nv12 = 0..4).
long long fractal_gb300_packed_frame_bytes(int width, int height, int format) {
    if (!valid_dims(width, height)) return -1;
    const std::size_t bytes = packed_frame_bytes(width, height, format);
    return bytes == 0 ? -1 : static_cast<long long>(bytes);
}

int fractal_gb300_pack_frame_device(const uint8_t* rgb, int width, int height, int format, uint8_t* output,
                                    void* stream_handle) {
    return guarded("device frame pack failed with an unknown exception", [&] {
        if (!rgb || !output || !valid_dims(width, height) || packed_frame_bytes(width, height, format) == 0) {
            throw Failure{"invalid frame pack dimensions or format"};
        }
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        check_cuda(launch_pack_frame(rgb, width, height, format, output, stream), "frame pack launch");
    });
}

// Device-pointer atlas frames (no reference counterpart): sources and output
// in device memory, enqueued on `stream` without synchronising.
int fractal_gb300_atlas_field_device(const float* parent, int parent_width, int parent_height, int parent_max_iter,
                                     const float* child, int child_width, int child_height, int child_max_iter,
                                     float* output, int output_width, int output_height, double parent_zoom,
                                     double child_fraction, double child_zoom, double parent_field_bias,
                                     double child_field_bias, double output_field_bias, int palette_max_iter,
                                     int feather, void* stream_handle) {
    return guarded("device atlas compositor failed with an unknown exception", [&] {
        if (!parent || !output) throw Failure{"invalid native scalar atlas dimensions"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction,
                             palette_max_iter};
        AtlasLaunch a = atlas_field_launch(r, child_zoom, parent_field_bias, child_field_bias, output_field_bias,
                                           feather);
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        wait_scratch(rt, stream);
        a.parent = parent;
        a.child = child;
        a.field_out = output;
        void* tables = scratch(rt, kScratchAtlas, atlas_table_bytes(a));
        check_cuda(run_atlas(rt, a, tables, stream), "atlas kernel launch");
        release_scratch(rt, stream);
    });
}

int fractal_gb300_atlas_colourise_device(const float* parent, int parent_width, int parent_height,
                                         int parent_max_iter, const float* child, int child_width, int child_height,
                                         int child_max_iter, uint8_t* output, int output_width, int output_height,
                                         double parent_zoom, double child_fraction, int palette_max_iter,
                                         double phase, double vocal, double instrumental, double pitch,
                                         const int* interior_rgb, const uint8_t* accents, void* stream_handle) {
    return guarded("device atlas colouriser failed with an unknown exception", [&] {
        if (!parent || !output) throw Failure{"invalid native atlas dimensions or controls"};
        const AtlasRequest r{parent_width, parent_height, parent_max_iter, child_width, child_height, child_max_iter,
                             child != nullptr, output_width, output_height, parent_zoom, child_fraction,
                             palette_max_iter};
        AtlasLaunch a = atlas_colour_launch(r, phase, vocal, instrumental, pitch, interior_rgb);
        ThreadRuntime& rt = thread_runtime();
        cudaStream_t stream = stream_handle ? static_cast<cudaStream_t>(stream_handle) : rt.stream;
        wait_scratch(rt, rt.stream);
        attach_aurora(rt, a, phase, vocal, pitch, accents);
        wait_scratch(rt, stream);
        a.parent = parent;
        a.child = child;
        a.rgb = output;
        void* tables = scratch(rt, kScratchAtlas, atlas_table_bytes(a));
        check_cuda(run_atlas(rt, a, tables, stream), "atlas kernel launch");
        release_scratch(rt, stream);
    });
}

}  // extern "C"
