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
//   FloatExp-free FP32 mirrors for the floatexp kernels (see render_fe.cu)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fractal_gb300.h"
#include "reference.h"

namespace fgb {

struct LevelIndex {
    int levels = 0;
    int offset[kMaxLevels] = {};
    int count[kMaxLevels] = {};
};

// FP32-mantissa / int32-exponent mirrors used by the floatexp form.
struct FeOrbitRec {
    float zr, zi;   // Z_i mantissas sharing exponent ze
    int ze;
    float zd_re;    // Z_i as plain float when representable, else 0
    float zd_im;
    float margin_m; // |Z_i|^2 - R^2 as float mantissa/exponent
    int margin_e;
    float glitch_m; // 1e-7 |Z_i|^2
    int glitch_e;
    float pad[7];
};

struct FeLinearStep {
    float ar, ai;
    int ae;
    float br, bi;
    int be;
    float r2m;
    int r2e;
    int len;
    int pad[7];
};

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
    // floatexp mirrors
    FeOrbitRec* fe_orbit = nullptr;
    FeLinearStep* fe_linear = nullptr;
    FeLinearStep* fe_deep_linear = nullptr;
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

// Stats slots (the reference's extended stats order, renderer.cpp:4676-4706).
constexpr int kStatsSlots = 39;

struct ThreadRuntime;
// Floatexp (FP32 mantissa / int32 exponent) form of a reference render.
void render_floatexp_from_reference(ReferenceContext& ctx, const Outputs& out, int width, int height,
                                    const char* zoom_text, int max_iter, int series_order, int series_block,
                                    const FractalRenderOptions& options, ThreadRuntime& rt,
                                    cudaStream_t stream);

cudaError_t launch_plain_mandelbrot(const PlainParams& params, bool planes, bool stats, cudaStream_t stream);
cudaError_t launch_plain_alternate(const AltParams& params, bool planes, bool stats,
                                   cudaStream_t stream);
cudaError_t launch_direct(const DirectParams& params, cudaStream_t stream);
// Records %globaltimer into *slot (the time-budget origin of the next kernel).
cudaError_t launch_stamp_time(unsigned long long* slot, cudaStream_t stream);
cudaError_t launch_aurora(const float* field, std::uint8_t* rgb, long long pixels,
                          const std::uint8_t* lut, int lut_size, float index_scale, int max_iter,
                          cudaStream_t stream);

}  // namespace fgb
