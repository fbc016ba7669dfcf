// Device-side table layout and kernel launch interfaces.
//
// HBM layout of one reference (uploaded once per handle generation):
//   OrbitRec[orbit_size]            128 B per reference index (orbit value,
//                                   plain-double copy, FloatExp parts,
//                                   escape-margin constant, glitch bound)
//   CubicStep[sum of level sizes]   cubic BLA hierarchy, levels back to back
//   LinearStep[...] x 2             linear and deep-linear hierarchies
//   AltStep[...]                    2x2 hierarchy (non-Mandelbrot formulas)
//   Sc[order + 1]                   image-series coefficients
//   FP32-mantissa mirrors of all of the above for the floatexp kernels
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <string>

#include "fractal_gb300.h"
#include "floatexp32.h"
#include "reference.h"

namespace fgb {

struct LevelIndex {
    int levels = 0;
    int offset[kMaxLevels] = {};
    int count[kMaxLevels] = {};
};

// FP32-mantissa / int32-exponent mirrors used by the floatexp form.  The
// records are 16-byte aligned so that kernels read them in 16-byte loads.
struct alignas(16) FxOrbitRec {
    float zr, zi;  // Z_i as plain float (0 below the float range)
    f32x::F2e z;   // Z_i as floatexp
    // Mandelbrot references: |Z_i|^2.  Other formulas: the signed escape
    // margin |Z_i|^2 - R^2 from the MPFR orbit (read as an f32x::R1e).
    f32x::N1e z2;
    int pad;
};

// FP32 mirror of AltStep: the real 2x2 maps d' = M d + P c, coefficients
// c[0..3] = M (row-major), c[4..7] = P, and the squared validity radius.
struct FxAltStep {
    f32x::R1e c[8];
    f32x::N1e r2;
    int len;
    int pad;
};

// BLA blocks start with a 16-byte head (squared radius, length), so the
// lookup reads a level's candidate with one load.
struct alignas(16) FxLinear {
    f32x::N1e r2;
    int len;
    int pad;
    f32x::F2e a;
    f32x::F2e b;
};

struct alignas(16) FxCubic {
    f32x::N1e r2;
    int len;
    int pad;
    f32x::F2e c[9];
};

static_assert(sizeof(FxOrbitRec) == 32, "FxOrbitRec is two 16-byte halves");
static_assert(sizeof(FxLinear) % 16 == 0 && sizeof(FxCubic) % 16 == 0, "16-byte block records");

struct DeviceTables {
    int device = -1;
    OrbitRec* orbit = nullptr;
    int orbit_size = 0;
    CubicStep* cubic = nullptr;
    LevelIndex cubic_index;
    LinearStep* linear = nullptr;
    LevelIndex linear_index;
    LinearStep* deep_linear = nullptr;
    LevelIndex deep_linear_index;
    AltStep* alt = nullptr;
    LevelIndex alt_index;
    fx::Sc* series = nullptr;
    int series_terms = 0;
    // floatexp mirrors (built on the first floatexp render)
    bool fx_ready = false;
    FxOrbitRec* fx_orbit = nullptr;
    FxCubic* fx_cubic = nullptr;
    FxLinear* fx_linear = nullptr;
    FxLinear* fx_deep_linear = nullptr;
    FxAltStep* fx_alt = nullptr;
    f32x::F2e* fx_series = nullptr;
    // Device copies of the level indexes for the floatexp kernels, which
    // take them by pointer (the batched queue's parameters hold 64 fields):
    // [0] cubic, [1] linear, [2] deep linear, [3] alternate.
    LevelIndex* fx_index = nullptr;
    ~DeviceTables();
};

// Parameters of one plain-form deep Mandelbrot field render.
struct PlainParams {
    const OrbitRec* orbit;
    int orbit_size;
    const CubicStep* cubic;
    LevelIndex cubic_index;
    const LinearStep* linear;  // normal or deep hierarchy chosen by the host
    LevelIndex linear_index;
    const fx::Sc* series;
    int series_terms;
    int series_iteration;
    int series_on;
    fx::Nrm series_r2;
    fx::Fe view_width;   // dc = (view_width * x_fraction, view_height * y_fraction)
    fx::Fe view_height;
    int coordinate_mode;
    int width;
    int height;
    int max_iter;
    int map_end;
    int disable_bla;
    int strict;
    int allow_recovery;
    int strict_cycle;
    int cycle;  // Brent cycle detection (non-strict or strict_cycle renders)
    int escape_mode;
    int max_bla_len;
    int max_lin_len;
    int approx_order;
    double output_bias;
    fx::Fe pixel_spacing;
    float* out;
    std::uint32_t* counts;
    std::int64_t* p_iter;
    double* p_phase;
    double* p_dex;
    double* p_dey;
    double* p_t1;
    double* p_t2;
    const unsigned long long* deadline_base;  // globaltimer at launch, or null
    unsigned long long budget_ns;
    unsigned long long* stats;
    // Point renders (fractal_render_points): pixel i takes dc = points[i]
    // instead of the grid offset; glitch pixels are flagged in exact_flags
    // (when non-null) and left for the host's exact MPFR repair.
    const fx::Sc* points;
    std::uint8_t* exact_flags;
};

// Parameters of one plain-form deep alternate-formula field render.
struct AltParams {
    const OrbitRec* orbit;
    int orbit_size;
    const AltStep* alt;
    LevelIndex alt_index;
    int alt_start;
    fx::Fe alt_input_radius2;
    const fx::Sc* series;
    int series_terms;
    int series_iteration;
    int series_on;
    fx::Nrm series_r2;
    fx::Fe view_width;
    fx::Fe view_height;
    int coordinate_mode;
    int width;
    int height;
    int max_iter;
    int map_end;
    int formula;
    int disable_bla;
    int strict;
    int allow_recovery;
    int cycle;
    int escape_mode;
    int max_lin_len;
    double output_bias;
    fx::Fe pixel_spacing;
    fx::Sc parameter;
    fx::Fe current_input_radius2;
    float* out;
    std::uint32_t* counts;
    std::int64_t* p_iter;
    double* p_phase;
    double* p_dex;
    double* p_dey;
    double* p_t1;
    double* p_t2;
    const unsigned long long* deadline_base;
    unsigned long long budget_ns;
    unsigned long long* stats;
    const fx::Sc* points;  // point renders: dc = points[i] (see PlainParams)
};

// Direct (shallow, plain double) render of any formula.
struct DirectParams {
    double center_re;
    double center_im;
    double width_span;
    double height_span;
    int coordinate_mode;
    int width;
    int height;
    int max_iter;
    int formula;
    double julia_re;
    double julia_im;
    double output_bias;
    int escape_mode;
    float* out;
    std::uint32_t* counts;
    std::int64_t* p_iter;
    double* p_phase;
    double* p_dex;
    double* p_dey;
    double* p_t1;
    double* p_t2;
    int need_phase;
    int need_de;
    double pixel_spacing;
};

// Outputs of one field render (device pointers; planes optional).
struct Outputs {
    float* field = nullptr;
    std::uint32_t* counts = nullptr;
    std::int64_t* p_iter = nullptr;
    double* p_phase = nullptr;
    double* p_dex = nullptr;
    double* p_dey = nullptr;
    double* p_t1 = nullptr;
    double* p_t2 = nullptr;
};

// Host-resolved parameters of one KFP colour pass (scalar-field ABI).
struct KfpLaunch {
    int width, height, max_iter;
    double field_bias, smooth_offset;
    int color_method, differences, smooth, flat, inverse_transition;
    int needs_difference, needs_slopes;
    double iter_div, color_offset, transfer_min, transfer_max;
    int multi_color, blend_multi_color, multi_count;
    double slope_cos, slope_sin, slope_power, slope_ratio;
    int interior[3];
    int lut_size;
};

// The plane inputs of fractal_colourise_kfp_planes (device copies of the
// FractalKfpPlanes arrays, null when absent) and the smoothing constants of
// kfp_pixel_context (renderer.cpp:5723-5763), resolved on the host.
struct KfpPlanesLaunch {
    const long long* orbit_iteration;
    const double* bailout;
    const long long* iteration;
    const double* transition;
    const double* phase;
    const double* de_x;
    const double* de_y;
    const double* test1;
    const double* test2;
    int has_iteration;   // orbit_iteration or iteration present
    int show_glitches;
    int analytic;        // Differences 7 with both DE planes
    int smooth_method;
    int has_constant_bailout;
    double smooth_bailout_radius, power;
    int has_smooth_power_log, has_smooth_bailout_log, has_smooth_norm_exponent;
    double smooth_power_log, smooth_bailout_log, smooth_norm_exponent;
    double phase_scale;  // phase_color_strength / 100 * 1024
    // FP32 copies for the SmoothMethod 0 term: log(power) when power is
    // finite and > 1 (else smooth_power_ok = 0), log of the constant bailout
    // radius when it is finite and > 1 (else smooth_radius_ok = 0).
    int smooth_power_ok, smooth_radius_ok;
    float smooth_power_log_f, smooth_radius_log_f;
    // Texture merging (planes->texture_rgb with texture_enabled): top-down
    // RGB8 rows of `texture_stride` bytes on the device.
    const std::uint8_t* texture;
    int texture_active, texture_width, texture_height, texture_stride;
    int image_offset;    // int(clamp(texture_power / 64)), 0 for a non-finite power
    double texture_power, texture_ratio, texture_merge;
};
// Plane samples (double-float) and flags of every pixel into samples/flags.
cudaError_t launch_kfp_plane_samples(const KfpPlanesLaunch& planes, int max_iter, long long pixels, void* samples,
                                     std::uint8_t* flags, cudaStream_t stream);
cudaError_t launch_kfp_plane_bounds(const void* samples, const std::uint8_t* flags, long long pixels, int max_iter,
                                    unsigned long long* bounds, cudaStream_t stream);
// With `planes` non-null the plane path runs (samples/flags from
// launch_kfp_plane_samples when the planes carry iterations).
// fractal_atlas_colourise_kfp (renderer.cpp:16750-17321): parent and child
// coloured as separate tiles at output scale (each with its own stencil
// edges and ColorMethod 4 bounds), the child over the rectangle at
// (child_left, child_top), blended across a smoothstep band of `feather`.
struct KfpAtlasLaunch {
    const float* parent;
    const float* child;  // null: parent only
    int child_width, child_height, child_left, child_top, feather;
    double child_transfer_min, child_transfer_max;
};
cudaError_t launch_kfp_atlas(const KfpAtlasLaunch& atlas, std::uint8_t* rgb, const KfpLaunch& parent_launch,
                             const std::uint8_t* lut, const double* mc_period, const int* mc_type,
                             cudaStream_t stream);
// Counts the float inputs for which the colour pass's constant division
// (div_const) differs from IEEE division by `divisor` (all 2^32 patterns).
cudaError_t launch_division_check(float divisor, unsigned long long* mismatches, cudaStream_t stream);
cudaError_t launch_kfp(const float* field, std::uint8_t* rgb, const KfpLaunch& launch, const std::uint8_t* lut,
                       const double* mc_period, const int* mc_type, cudaStream_t stream,
                       const KfpPlanesLaunch* planes = nullptr, const void* samples = nullptr,
                       const std::uint8_t* flags = nullptr);
cudaError_t launch_kfp_bounds(const float* field, long long pixels, int max_iter, double field_bias,
                              double smooth_offset, unsigned long long* bounds, cudaStream_t stream);

// Stats slots (the reference's extended stats order, renderer.cpp:4676-4706).
constexpr int kStatsSlots = 39;

// Parameters of one floatexp-form deep Mandelbrot field render.
// The image series rescaled for one field: delta = 2^shift * sum_k b[k] u^k
// (k >= 1) with u = dc * 2^-scale, |u| <= 1 over the view, so every pixel
// evaluates it in plain float (kernel-side prologue, render_fe.cu).
constexpr int kMaxSeriesTerms = 33;
struct alignas(8) FxSeriesScaled {
    float b[kMaxSeriesTerms][2];
    int terms;
    int shift;
    int scale;
    int pad;
};

struct FxParams {
    const FxOrbitRec* orbit;
    int orbit_size;
    const FxCubic* cubic;
    const LevelIndex* cubic_index;   // device copies (DeviceTables::fx_index)
    const FxLinear* linear;
    const LevelIndex* linear_index;
    const f32x::F2e* series;
    int series_terms;
    int series_iteration;
    int series_on;
    f32x::N1e series_r2;
    f32x::F2e view_width;   // real parts carry the spans
    f32x::F2e view_height;
    int coordinate_mode;
    int width;
    int height;
    int max_iter;
    int map_end;
    int disable_bla;
    int strict;
    int allow_recovery;
    int escape_mode;
    int max_bla_len;
    int max_lin_len;
    int approx_order;
    float output_bias;
    float* out;
    std::uint32_t* counts;
    FxSeriesScaled* series_scaled;  // per-field slot filled by the series prologue (nullptr: F2e Horner)
    // Shallow mode (a field the reference pipeline renders on the direct
    // path, below 1e12): plain FP32 perturbation against the orbit from
    // iteration 0 with unlimited rebasing, no series, no BLA; pixels that the
    // cardioid / period-2 bulb test puts clearly inside are written as
    // interior without iterating (interior_test: the view reaches either).
    int shallow;
    int interior_test;
    float centre_re;  // the view centre rounded to float (interior test only)
    float centre_im;
    // Other formulas (kFormulaJulia / BurningShip / Tricorn): the FP32 2x2
    // hierarchy `alt` (its levels indexed by linear_index), the reference
    // index its level 0 starts at, the bound on |c|^2 for using it, and the
    // parameter (Julia's c; the reference's c for the parameter planes).
    int formula;
    const FxAltStep* alt;
    int alt_start;
    f32x::N1e alt_input_radius2;
    f32x::F2e parameter;
    // Derivative planes (optional, both or neither): the analytic distance
    // estimate (render_plane_de, renderer.cpp:7844-7990) per pixel, and the
    // pixel spacing it is measured in.
    double* de_x;
    double* de_y;
    f32x::N1e pixel_spacing;
};

cudaError_t launch_floatexp_mandelbrot(const FxParams& params, cudaStream_t stream);

// Launch shape of a persistent queue kernel: pixels per warp claim and
// resident blocks per SM (0 = as many as fit).
struct QueueShape {
    int chunk = 0;
    int blocks_per_sm = 0;
    int steps = 0;  // direct queue: steps between refills in its first phase (0 = 2)
};

constexpr int kMaxFxFields = 64;
constexpr int kTileSide = 64;      // scheduling tile (pixels per side)
constexpr int kProbeStride = 4;    // coarse probe: every 4th pixel each way
struct FxBatch {
    FxParams field[kMaxFxFields];
    long long first[kMaxFxFields + 1];
    int tiles_first[kMaxFxFields + 1];  // 64x64-tile prefix over the batch
    int tiles_x[kMaxFxFields];
    float log_zoom[kMaxFxFields];       // log10 zoom of each field (tile features)
    int count;
    int chunk;
    unsigned long long* counter;
    // Tile mode (tile_rows > 0): a work unit is a band of tile_rows rows of
    // one tile; tiles are claimed in `order` (tile ids; nullptr = ascending),
    // per-tile warp time is accumulated in tile_cost (SM cycles; optional)
    // and timing[] gets {first claim, last claim, last finish} (%globaltimer
    // ns; optional).
    int tile_rows;
    const unsigned* order;
    unsigned long long* tile_cost;
    unsigned long long* timing;
};
// Many floatexp fields in one persistent launch (counter: 8 bytes of device
// memory, zeroed on the stream before the kernel).
cudaError_t launch_floatexp_batch(const FxParams* fields, int count, unsigned long long* counter,
                                  const QueueShape& shape, cudaStream_t stream);

// Tile scheduling of a floatexp batch (64x64 tiles of every field).
struct TileSchedule {
    int tile_rows = 8;                   // rows per work unit (divides 64)
    const unsigned* order = nullptr;     // claim order (nullptr = ascending tile id)
    unsigned long long* tile_cost = nullptr;
    unsigned long long* timing = nullptr;
};
int batch_tiles(const FxParams* fields, int count);
// Fill each field's series_scaled slot (before any launch that renders it).
cudaError_t launch_series_prologue(const FxParams* fields, int count, cudaStream_t stream);
// Resident 128-thread blocks per SM of the persistent queue kernels, and
// their register / shared-memory use (for sharing an SM between the two).
int floatexp_queue_occupancy(bool tiles);
int direct_queue_occupancy();
cudaError_t floatexp_queue_attributes(bool tiles, cudaFuncAttributes* attributes);
cudaError_t direct_queue_attributes(cudaFuncAttributes* attributes);
cudaError_t launch_floatexp_tiles(const FxParams* fields, const float* log_zoom, int count,
                                  unsigned long long* counter, const QueueShape& shape, const TileSchedule& schedule,
                                  cudaStream_t stream);
// Coarse probe (16x16 samples per tile, iteration counts) and the network's
// BF16 features (rows padded to a multiple of 128 with zero rows).
cudaError_t launch_tile_probe(const FxParams* fields, const float* log_zoom, int count, std::uint32_t* probe,
                              __nv_bfloat16* features, int feature_rows, cudaStream_t stream);
// Heaviest-first claim order from predicted (normalised log) tile costs.
cudaError_t launch_tile_order(const float* predicted, int tiles, unsigned* order, cudaStream_t stream);

struct ThreadRuntime;
// Floatexp (FP32 mantissa / int32 exponent) form of a reference render.
void render_floatexp_from_reference(ReferenceContext& ctx, const Outputs& out, int width, int height,
                                    const char* zoom_text, int max_iter, int series_order, int series_block,
                                    const FractalRenderOptions& options, ThreadRuntime& rt,
                                    cudaStream_t stream);

cudaError_t launch_plain_mandelbrot(const PlainParams& params, bool planes, bool stats, cudaStream_t stream);
// With `queue_counter` (8 bytes of device memory no other launch uses at
// the same time) a Julia field renders through the persistent lane-refill
// queue; other formulas, point lists and calls without a counter run one
// thread per pixel.
cudaError_t launch_plain_alternate(const AltParams& params, bool planes, bool stats,
                                   unsigned long long* queue_counter, cudaStream_t stream);
// A batch of direct fields (one kernel over all of them); the batch struct
// travels as a __grid_constant__ kernel parameter.
constexpr int kMaxDirectFields = 64;
// A pixel that ran past its iteration budget, parked with its whole state
// so that another warp resumes it bit for bit; `ready` carries the batch's
// generation once the entry is written.
struct alignas(128) DirectSpill {
    double zr, zi, dr, di, test1, test2;
    unsigned long long saved_r, saved_i, mark_r, mark_i;
    int it, check_at, field, local;
    unsigned long long ready;
};
// Device counters of a direct batch (at the start of its scratch).
enum DirectCounter {
    kClaimFresh = 0,   // pixels claimed
    kSpillReserved,    // spill slots taken by producers
    kSpillClaimed,     // spill slots taken by consumers
    kStepsExecuted,    // iterations computed
    kQueueError,       // a wait on a spill entry gave up
    kGeneration,       // batch generation (not reset; bumped per launch)
};
struct DirectBatch {
    DirectParams field[kMaxDirectFields];
    long long first[kMaxDirectFields + 1];  // pixel prefix over the batch
    int coord_offset[kMaxDirectFields];     // cx then cy table of each field
    int interior_test[kMaxDirectFields];    // cardioid/bulb culling needed
    int count;
    int chunk;                              // pixels per warp claim
    double* coords;
    unsigned long long* counter;            // DirectCounter slots
    // A fresh pixel still running after `budget` steps is spilled (when the
    // list has room) and resumed, to its end, by whichever warp refills
    // first: long orbits end up 32 to a warp and start early.
    int budget;
    int steps;                              // steps between refills (fresh pixels in the warp)
    int long_steps;                         // steps between refills (only resumed pixels)
    int fast_smooth;                        // smooth value in FP32 (floatexp form's direct levels)
    DirectSpill* spill;
    long long spill_capacity;
    // Bound on a consumer's wait for a spilled entry's generation mark (then
    // kQueueError is set and the entry is dropped), and a fault-injection
    // switch for tests: spilled entries are written but never published.
    int spin_limit;
    int withhold_publish;
};
// Spill-wait bound and publish suppression of the calling thread's next
// direct launches (tests of the queue's error path); 0, 0 restores the
// defaults (1 << 22 spins, publish).
void set_direct_fault_injection(int spin_limit, int withhold_publish);
// Device scratch for one batch: counters, coordinate tables and a spill list
// of `spill_entries` (0: no spilling).
std::size_t direct_scratch_bytes(const DirectParams* fields, int count, long long spill_entries);
cudaError_t launch_direct_batch(const DirectParams* fields, int count, void* scratch, const QueueShape& shape,
                                long long spill_entries, cudaStream_t stream, bool fast_smooth = false);
// One direct field with its scratch taken from a fixed array compiled into
// the library (render_noalloc.cu): no device allocation at all.
bool launch_direct_noalloc(const DirectParams& params, cudaStream_t stream, std::string& why);
std::size_t noalloc_scratch_limit();
// Atlas compositor (compose.cu): one output frame from a parent and a child
// keyframe.  Axes map output columns/rows to source indices and weights; the
// launcher builds them (and the child's edge ramps) on the device.
struct AtlasAxis {
    const int* index0;
    const int* index1;
    const float* weight;
};
// Per-axis constants, formed on the host in the reference's order.
struct AtlasAxisPlan {
    double left, step, crop, span;
    int source;
    int window;  // fill_bilinear_axis_window form (raw KFP child axes)
};
struct AtlasTables {
    AtlasAxisPlan plan[4];  // parent x, parent y, child x, child y
    struct Axis {
        int* i0;
        int* i1;
        float* w;
    };
    Axis parent_x, parent_y, child_x, child_y;
    float* edge_x;
    float* edge_y;
    double* alpha;
    int parent_x_size, parent_y_size, child_x_size, child_y_size, edge_x_size, edge_y_size, alpha_size;
};
enum AtlasMode {
    kAtlasField = 0,        // fractal_atlas_field_ex: interior-preserving scalar frame
    kAtlasAurora = 1,       // atlas_colourise_impl: aurora RGB8 frame
    kAtlasKfpSurface = 2,   // fractal_atlas_colourise_kfp_raw / fractal_crop_colourise_kfp surface
    kAtlasCropField = 3,    // fractal_crop_field: plain bilinear scalar crop
    kAtlasRgb = 4,          // fractal_crop_rgb / fractal_atlas_composite_rgb: RGB8 sources
    kAtlasCropAurora = 5,   // crop_colourise_impl: aurora crop of one field
    kAtlasKfpPlanes = 6,    // fractal_atlas_colourise_kfp_planes surface (+ interior flags)
};
struct AtlasLaunch {
    int mode;  // AtlasMode: field_out (field, KFP surface) or rgb (aurora)
    const float* parent;
    int parent_width, parent_height, parent_max_iter;
    double parent_bias, parent_zoom;
    const float* child;
    int child_width, child_height, child_max_iter;
    double child_bias, child_zoom;
    const std::uint8_t* parent_rgb;  // kAtlasRgb sources (3 bytes per pixel)
    const std::uint8_t* child_rgb;
    int out_width, out_height;
    int use_child, full_child;
    int feather;  // edge-ramp width; < 2 = no ramp
    int child_left, child_top, child_visible_width, child_visible_height;
    // Filled by launch_atlas.
    AtlasAxis parent_x, parent_y, child_x, child_y;
    const float* edge_x;
    const float* edge_y;
    const double* alpha;                    // kAtlasRgb: seam alpha by edge distance, feather entries
    float parent_limit, child_limit;        // smallest float >= cap - bias
    float parent_bias_hi, parent_bias_lo;   // biases as double-float
    float child_bias_hi, child_bias_lo;
    float output_bias_f;
    int output_bias_exact;                  // output_bias is a float
    float interior_value;                   // the output value of an interior sample
    unsigned* exact_count;                  // pixels queued for the exact (FP64) pass
    unsigned* exact_pixels;
    // Scalar output (fractal_atlas_field_ex; the KFP surface, where
    // output_bias is the KFP field bias and effective_iter the cap) ...
    float* field_out;
    double output_bias;
    int effective_iter;
    // ... or aurora RGB8 (atlas_colourise_impl) when field_out is null.
    std::uint8_t* rgb;
    const std::uint8_t* lut;
    int lut_size;
    float index_scale;
    int palette_iter;
    int interior[3];
    // kAtlasKfpPlanes: per output pixel, bit 0 = the primary sample is
    // interior, bit 1 = the child sample is (inside the child rectangle).
    std::uint8_t* inside_out;
};
// The KFP render planes of one atlas source, or of the composed frame
// (device; any may be null): orbit_iteration, iteration; bailout,
// transition, phase, de_x, de_y, test1, test2.
struct KfpPlaneSet {
    const long long* ints[2];
    const double* doubles[7];
};
struct KfpPlaneOutputs {
    long long* ints[2];
    double* doubles[7];
};
// fractal_atlas_colourise_kfp_planes' plane reprojection (renderer.cpp:
// 17553-17765) over the tables and interior flags of a kAtlasKfpPlanes
// launch: nearest-sample integer planes, bilinear double planes (transition
// keeps negative glitch markers), interior resets, the child blend.
cudaError_t launch_atlas_planes(const AtlasLaunch& launch, const KfpPlaneSet& primary, const KfpPlaneSet& secondary,
                                const KfpPlaneOutputs& out, long long target_max_iter, cudaStream_t stream);
// Device bytes of the per-frame tables of `launch` (axes and ramps).
std::size_t atlas_table_bytes(const AtlasLaunch& launch);
// Builds the tables in `tables` (atlas_table_bytes, 256-byte aligned), then
// composes the frame: two kernels on `stream`.
cudaError_t launch_atlas(AtlasLaunch& launch, void* tables, cudaStream_t stream);

// Video-frame packing (pack.cu): RGB8 into rgb24 / rgb0 / rgba / yuv420p /
// nv12 (format 0..4); bytes of a packed frame, 0 for an unknown format.
std::size_t packed_frame_bytes(int width, int height, int format);
cudaError_t launch_pack_frame(const std::uint8_t* rgb, int width, int height, int format, std::uint8_t* out,
                              cudaStream_t stream);

// Records %globaltimer into *slot (the time-budget origin of the next kernel).
cudaError_t launch_stamp_time(unsigned long long* slot, cudaStream_t stream);
cudaError_t launch_aurora(const float* field, std::uint8_t* rgb, long long pixels,
                          const std::uint8_t* lut, int lut_size, float index_scale, int max_iter,
                          cudaStream_t stream, std::uint32_t interior = 0);  // interior RGB as 0xBBGGRR

}  // namespace fgb
