// Host-side reference context: the serial MPFR orbit and the tables every
// device kernel reads (image series, BLA hierarchies, per-orbit records).
//
// Mirrors the reference's ReferenceContext (renderer.cpp:8881-8924) and the
// builders make_reference_orbit (:10640), build_image_series (:11206),
// build_bla (:11612), build_alternate_linear_bla (:11414), the retargeting
// clone (:11776-11868, :13705) and the alternate cycle stabiliser (:9691).
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "scaled.h"

namespace fgb {

constexpr int kFormulaMandelbrot = 0;
constexpr int kFormulaJulia = 1;
constexpr int kFormulaBurningShip = 2;
constexpr int kFormulaTricorn = 3;

constexpr int kMaxSafeBlaLength = 64;          // cubic hierarchy limit
constexpr int kMaxSafeLinearBlaLength = 4096;  // ultra-deep linear limit
constexpr int kMaxSafeDeepLinearBlaLength = 1024;
constexpr int kMaxLevels = 16;

// Render-form cubic BLA step: the nine bivariate coefficients
// A d + B c + C d^2 + D d c + E c^2 + F d^3 + G d^2 c + H d c^2 + I c^3.
struct CubicStep {
    fx::Sc c[9];
    fx::Fe r2;
    int len;
    int pad;
};

struct LinearStep {
    fx::Sc a;
    fx::Sc b;
    fx::Fe r2;
    int len;
    int pad;
};

// Real 2x2 M,P map for the non-holomorphic formulas: d' = M d + P dc.
struct AltStep {
    fx::Fe c[8];
    fx::Fe r2;
    int len;
    int pad;
};

// Everything one perturbation step needs about reference index i, packed so
// a lane touches a single 128-byte record.
struct alignas(128) OrbitRec {
    fx::Sc z;          // compact orbit value Z_i
    double zd_re;      // Z_i as plain double (double-tail path)
    double zd_im;
    fx::Fec parts;     // Z_i components as FloatExp (escape margin input)
    fx::Fe margin;     // |Z_i|^2 - R^2 (escape margin constant term)
    fx::Fe glitch;     // 1e-7 |Z_i|^2, zero when the glitch test is off
};

struct OrbitData {
    std::vector<fx::Sc> scaled;
    std::vector<double> re_d;
    std::vector<double> im_d;
    std::vector<fx::Fe> escape_margin;
};

struct ImageSeries {
    bool enabled = false;
    int order = 0;
    int iteration = 1;
    fx::Fe r2 = {0.0, 0};
    std::vector<fx::Sc> coeff;
};

struct DeviceTables;  // device copies, owned by the context (device.cu)

struct ReferenceContext {
    std::uint64_t generation = 0;
    std::vector<fx::Fec> fast_orbit;  // builder orbit (kept for reusable roots)
    std::shared_ptr<const OrbitData> orbit;
    // Mandelbrot BLA hierarchies (render form).
    std::vector<std::vector<CubicStep>> cubic;
    std::vector<std::vector<LinearStep>> linear;
    std::vector<std::vector<LinearStep>> deep_linear;
    fx::Fe input_radius = {0.0, 0};
    fx::Fe deep_input_radius = {0.0, 0};
    int map_end = 0;
    // Alternate-formula hierarchy.
    std::vector<std::vector<AltStep>> alt;
    fx::Fe alt_input_radius = {0.0, 0};
    fx::Fe alt_input_radius2 = {0.0, 0};
    int alt_start = 0;
    ImageSeries series;
    int requested_max_iter = 0;
    int requested_series_order = 8;
    std::uint64_t reference_build_ns = 0;
    std::uint64_t series_build_ns = 0;
    std::uint64_t bla_build_ns = 0;
    long double x_center = 0.0L;
    long double y_center = 0.0L;
    std::string x_text;
    std::string y_text;
    int formula = kFormulaMandelbrot;
    double julia_re = 0.0;
    double julia_im = 0.0;
    fx::Sc parameter = {0.0, 0.0, 0};
    int escape_mode = 0;
    int coordinate_mode = 0;
    long precision_bits = 0;
    bool bla_on_device = false;  // hierarchy levels >= 1 merged by the GPU

    std::mutex device_mutex;
    std::shared_ptr<DeviceTables> device;
};

// Thrown for invalid arguments; the ABI layer turns it into last_error.
struct Failure {
    std::string message;
};

// Locale-independent decimal parsing (renderer.cpp:214-246).
long double parse_coordinate(const char* text, const char* label);
long double parse_zoom_direct(const char* text);
fx::Fe parse_zoom_fe(const char* text, long precision_bits);
bool mpfr_available(std::string* why);

double viewport_height_factor(int coordinate_mode);
double pixel_axis_offset(int index, int dimension, int coordinate_mode);

std::unique_ptr<ReferenceContext> create_reference_context(
    const char* x_center, const char* y_center, const char* viewport_zoom,
    int max_iter, int precision_bits, int series_order, bool retain_builder_orbit,
    int formula, const char* julia_re, const char* julia_im, int escape_mode,
    int coordinate_mode);

std::unique_ptr<ReferenceContext> clone_reference_context(
    const ReferenceContext& source, const char* viewport_zoom);

// Registry of opaque handles (tokens from 0x1000, renderer.cpp:9800-9836).
void* register_reference(std::unique_ptr<ReferenceContext> context);
std::shared_ptr<ReferenceContext> acquire_reference(void* handle);
std::shared_ptr<ReferenceContext> remove_reference(void* handle);

// Build the per-index records the kernels read (escape-mode specific).
std::vector<OrbitRec> make_orbit_records(const ReferenceContext& context);

// Where the BLA hierarchies are built: true (default) = on the GPU
// (bla_build.cu), false = on the host.  Both give identical tables.
bool device_table_builder();
void set_device_table_builder(bool on_device);
void build_bla_on_device(ReferenceContext& ctx, int base_count);
void build_alt_bla_on_device(ReferenceContext& ctx, int first_index, int base_count);
void retarget_bla_on_device(ReferenceContext& ctx, const ReferenceContext& source);

// One point's render planes (FractalRenderPlanes entries).
struct ExactPlanes {
    long long iteration;
    double phase, de_x, de_y, test1, test2;
};

// render_exact_mandelbrot_pixel (renderer.cpp:10931-11150): the pixel at
// centre + dc iterated from scratch in MPFR (host), with its derivative for
// the planes.  False when the context cannot support it (no centre text, <128
// bits, no MPFR) or the escape log is not finite.
bool exact_mandelbrot_pixel(const ReferenceContext& ctx, const fx::Sc& dc, int max_iter, double output_bias,
                            int escape_mode, const fx::Fe& pixel_spacing, float& out, ExactPlanes* planes);

}  // namespace fgb
