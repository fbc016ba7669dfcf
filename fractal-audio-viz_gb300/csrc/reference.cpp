// Host reference stage: MPFR orbit, image series and BLA hierarchies.
//
// The orbit is the one serial, arbitrary-precision part of the path and stays
// on the host, as in the reference (renderer.cpp:10640-10922).  MPFR is the
// system library libmpfr.so.6, loaded with dlopen so that the library still
// loads (and reports a clear error on use) where MPFR is missing.  The table
// builders restate the reference algorithms over the shared scaled.h
// arithmetic, so the tables are bit-identical to the reference's.
#include "reference.h"

#include <dlfcn.h>
#include <locale.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <unordered_map>

#include "bla_math.h"

namespace fgb {

namespace {

constexpr long double kLogTwo = 0.693147180559945309417232121458176568L;
constexpr long double kLogTen = 2.302585092994045684017991454684364208L;
constexpr std::size_t kMaxTextLength = 50000;

// ---------------------------------------------------------------- MPFR API
// Public MPFR 4 types as documented in the MPFR manual.
struct MpfrStruct {
    long prec;
    int sign;
    long exp;
    void* limbs;
};
using mpfr_ptr = MpfrStruct*;
using mpfr_srcptr = const MpfrStruct*;
constexpr int RNDN = 0;

struct MpfrApi {
    bool ok = false;
    std::string error;
    void (*init2)(mpfr_ptr, long) = nullptr;
    void (*clear)(mpfr_ptr) = nullptr;
    int (*set_str)(mpfr_ptr, const char*, int, int) = nullptr;
    int (*set)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    int (*set_d)(mpfr_ptr, double, int) = nullptr;
    int (*set_ui)(mpfr_ptr, unsigned long, int) = nullptr;
    void (*set_zero)(mpfr_ptr, int) = nullptr;
    int (*mul)(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, int) = nullptr;
    int (*add)(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, int) = nullptr;
    int (*sub)(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, int) = nullptr;
    int (*div)(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, int) = nullptr;
    int (*sqrt)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    int (*neg)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    int (*abs)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    int (*mul_ui)(mpfr_ptr, mpfr_srcptr, unsigned long, int) = nullptr;
    int (*add_ui)(mpfr_ptr, mpfr_srcptr, unsigned long, int) = nullptr;
    int (*ui_sub)(mpfr_ptr, unsigned long, mpfr_srcptr, int) = nullptr;
    int (*div_2ui)(mpfr_ptr, mpfr_srcptr, unsigned long, int) = nullptr;
    int (*pow_si)(mpfr_ptr, mpfr_srcptr, long, int) = nullptr;
    int (*log10)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    int (*sgn)(mpfr_srcptr) = nullptr;
    int (*number_p)(mpfr_srcptr) = nullptr;
    int (*cmp)(mpfr_srcptr, mpfr_srcptr) = nullptr;
    int (*cmp_ui)(mpfr_srcptr, unsigned long) = nullptr;
    double (*get_d)(mpfr_srcptr, int) = nullptr;
    double (*get_d_2exp)(long*, mpfr_srcptr, int) = nullptr;
    // Used by the exact point repair only.
    int (*log)(mpfr_ptr, mpfr_srcptr, int) = nullptr;
    long double (*get_ld)(mpfr_srcptr, int) = nullptr;
    int (*cmp_d)(mpfr_srcptr, double) = nullptr;
    int (*mul_2si)(mpfr_ptr, mpfr_srcptr, long, int) = nullptr;
    bool exact_ok = false;
};

template <typename T>
bool bind_symbol(void* library, const char* name, T& target, std::string& error) {
    void* symbol = dlsym(library, name);
    if (!symbol) {
        error = std::string("libmpfr.so.6 lacks ") + name;
        return false;
    }
    target = reinterpret_cast<T>(symbol);
    return true;
}

const MpfrApi& mpfr() {
    static const MpfrApi api = [] {
        MpfrApi result;
        void* library = dlopen("libmpfr.so.6", RTLD_NOW | RTLD_LOCAL);
        if (!library) {
            result.error = "the MPFR runtime (libmpfr.so.6) is not available: deep references need it";
            return result;
        }
        std::string& e = result.error;
        const bool ok = bind_symbol(library, "mpfr_init2", result.init2, e)
            && bind_symbol(library, "mpfr_clear", result.clear, e)
            && bind_symbol(library, "mpfr_set_str", result.set_str, e)
            && bind_symbol(library, "mpfr_set", result.set, e)
            && bind_symbol(library, "mpfr_set_d", result.set_d, e)
            && bind_symbol(library, "mpfr_set_ui", result.set_ui, e)
            && bind_symbol(library, "mpfr_set_zero", result.set_zero, e)
            && bind_symbol(library, "mpfr_mul", result.mul, e)
            && bind_symbol(library, "mpfr_add", result.add, e)
            && bind_symbol(library, "mpfr_sub", result.sub, e)
            && bind_symbol(library, "mpfr_div", result.div, e)
            && bind_symbol(library, "mpfr_sqrt", result.sqrt, e)
            && bind_symbol(library, "mpfr_neg", result.neg, e)
            && bind_symbol(library, "mpfr_abs", result.abs, e)
            && bind_symbol(library, "mpfr_mul_ui", result.mul_ui, e)
            && bind_symbol(library, "mpfr_add_ui", result.add_ui, e)
            && bind_symbol(library, "mpfr_ui_sub", result.ui_sub, e)
            && bind_symbol(library, "mpfr_div_2ui", result.div_2ui, e)
            && bind_symbol(library, "mpfr_pow_si", result.pow_si, e)
            && bind_symbol(library, "mpfr_log10", result.log10, e)
            && bind_symbol(library, "mpfr_sgn", result.sgn, e)
            && bind_symbol(library, "mpfr_number_p", result.number_p, e)
            && bind_symbol(library, "mpfr_cmp", result.cmp, e)
            && bind_symbol(library, "mpfr_cmp_ui", result.cmp_ui, e)
            && bind_symbol(library, "mpfr_get_d", result.get_d, e)
            && bind_symbol(library, "mpfr_get_d_2exp", result.get_d_2exp, e);
        result.ok = ok;
        std::string unused;
        result.exact_ok = ok && bind_symbol(library, "mpfr_log", result.log, unused)
            && bind_symbol(library, "mpfr_get_ld", result.get_ld, unused)
            && bind_symbol(library, "mpfr_cmp_d", result.cmp_d, unused)
            && bind_symbol(library, "mpfr_mul_2si", result.mul_2si, unused);
        return result;
    }();
    return api;
}

const MpfrApi& need_mpfr() {
    const MpfrApi& api = mpfr();
    if (!api.ok) throw Failure{api.error};
    return api;
}

// RAII multi-precision value.
class Mp {
public:
    explicit Mp(long precision) { need_mpfr().init2(&value_, precision); }
    ~Mp() { mpfr().clear(&value_); }
    Mp(const Mp&) = delete;
    Mp& operator=(const Mp&) = delete;
    mpfr_ptr get() { return &value_; }
    operator mpfr_ptr() { return &value_; }

private:
    MpfrStruct value_{};
};

// FloatExp::from_mpfr (renderer.cpp:7569-7579).
fx::Fe fe_from_mpfr(mpfr_srcptr value) {
    long exponent = 0;
    const double mantissa = mpfr().get_d_2exp(&exponent, value, RNDN);
    if (!std::isfinite(mantissa)) return fx::fe_make(mantissa, 0);
    if (exponent > std::numeric_limits<int>::max()) {
        return fx::fe_make(std::copysign(std::numeric_limits<double>::infinity(), mantissa), 0);
    }
    if (exponent < std::numeric_limits<int>::min()) return fx::fe_make(0.0, 0);
    return fx::fe_from(mantissa, static_cast<int>(exponent));
}

long double fe_log(const fx::Fe& value) {
    if (value.m == 0.0) return -std::numeric_limits<long double>::infinity();
    return std::log(std::fabs(static_cast<long double>(value.m)))
        + static_cast<long double>(value.e) * kLogTwo;
}

bool valid_text(const char* text) {
    if (!text) return false;
    for (std::size_t length = 0; length <= kMaxTextLength; ++length) {
        if (text[length] == '\0') return true;
    }
    return false;
}

bool parse_classic(const char* text, long double& value) {
    if (!valid_text(text)) return false;
    // Only plain decimal notation is accepted, as by a classic-locale
    // std::istream (no hex floats, no inf/nan words).
    for (const char* p = text; *p; ++p) {
        const char ch = *p;
        const bool allowed = (ch >= '0' && ch <= '9') || ch == '.' || ch == '+' || ch == '-'
            || ch == 'e' || ch == 'E' || ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r';
        if (!allowed) return false;
    }
    static locale_t classic = newlocale(LC_NUMERIC_MASK, "C", static_cast<locale_t>(0));
    char* end = nullptr;
    value = strtold_l(text, &end, classic);
    if (end == text) return false;
    while (*end == ' ' || *end == '\t' || *end == '\n' || *end == '\r') ++end;
    return *end == '\0';
}


}  // namespace

bool mpfr_available(std::string* why) {
    const MpfrApi& api = mpfr();
    if (!api.ok && why) *why = api.error;
    return api.ok;
}

double viewport_height_factor(int coordinate_mode) { return coordinate_mode == 1 ? 4.0 : 2.8; }

double pixel_axis_offset(int index, int dimension, int coordinate_mode) {
    const double origin = coordinate_mode == 1
        ? static_cast<double>(dimension / 2)
        : static_cast<double>(dimension - 1) / 2.0;
    return static_cast<double>(index) - origin;
}

long double parse_coordinate(const char* text, const char* label) {
    if (!valid_text(text) || !label) throw Failure{"native coordinate text is too long or null"};
    long double value = 0.0L;
    if (!parse_classic(text, value) || !std::isfinite(value)) {
        throw Failure{std::string("invalid ") + label + " coordinate"};
    }
    return value;
}

long double parse_zoom_direct(const char* text) {
    if (!valid_text(text)) throw Failure{"native zoom text is too long or null"};
    long double zoom = 0.0L;
    if (!parse_classic(text, zoom) || !std::isfinite(zoom) || zoom <= 0.0L) {
        throw Failure{"invalid Mandelbrot zoom"};
    }
    const long double log10_zoom = std::log10(zoom);
    if (!std::isfinite(log10_zoom) || log10_zoom < -300.0L || log10_zoom > 9800.0L) {
        throw Failure{"Mandelbrot zoom is outside the supported range"};
    }
    return zoom;
}

// parse_zoom_float_exp (renderer.cpp:11892-11915).
fx::Fe parse_zoom_fe(const char* text, long precision_bits) {
    if (!valid_text(text)) throw Failure{"native zoom text is too long or null"};
    const MpfrApi& api = need_mpfr();
    Mp value(precision_bits);
    const int status = api.set_str(value, text, 10, RNDN);
    if (status != 0 || api.sgn(value) <= 0 || !api.number_p(value)) {
        throw Failure{"invalid deep Mandelbrot zoom"};
    }
    const fx::Fe result = fe_from_mpfr(value);
    if (!fx::fe_finite(result) || fx::fe_is_zero(result)) {
        throw Failure{"deep Mandelbrot zoom is outside the native exponent range"};
    }
    const long double log10_zoom = fe_log(result) / kLogTen;
    if (!std::isfinite(log10_zoom) || log10_zoom < -300.0L || log10_zoom > 9800.0L) {
        throw Failure{"deep Mandelbrot zoom is outside the supported range"};
    }
    return result;
}

namespace {

// ------------------------------------------------------------ orbit stage
void stabilize_alternate_cycle(std::vector<fx::Fec>& fast, OrbitData& orbit, int mode) {
    const std::size_t count = std::min(fast.size(), orbit.scaled.size());
    if (count < 6 || orbit.re_d.size() != count || orbit.im_d.size() != count) return;
    std::size_t last_finite = count;
    while (last_finite > 0) {
        const std::size_t i = last_finite - 1;
        if (std::isfinite(orbit.re_d[i]) && std::isfinite(orbit.im_d[i])) break;
        --last_finite;
    }
    if (last_finite < 6) return;
    const std::size_t scan_limit = std::min<std::size_t>(last_finite - 1, 1024);
    const int max_period = std::min<int>(64, static_cast<int>((scan_limit + 1) / 4));
    const double tolerance = 1.0e-12;
    const double bound = fx::escape_r2_d(mode);
    for (int period = 1; period <= max_period; ++period) {
        for (std::size_t end = static_cast<std::size_t>(4 * period - 1); end <= scan_limit; ++end) {
            const std::size_t start = end - static_cast<std::size_t>(3 * period) + 1U;
            bool matches = true;
            for (int k = 0; k < period && matches; ++k) {
                const std::size_t a = start + static_cast<std::size_t>(k);
                const std::size_t b = a + static_cast<std::size_t>(period);
                const std::size_t c = b + static_cast<std::size_t>(period);
                const double ra = std::hypot(orbit.re_d[a], orbit.im_d[a]);
                const double rb = std::hypot(orbit.re_d[b], orbit.im_d[b]);
                const double rc = std::hypot(orbit.re_d[c], orbit.im_d[c]);
                if (!std::isfinite(ra) || !std::isfinite(rb) || !std::isfinite(rc)
                    || ra * ra >= bound || rb * rb >= bound || rc * rc >= bound) {
                    matches = false;
                    break;
                }
                const double scale = std::max(1.0, std::max(ra, std::max(rb, rc)));
                const double d1 = std::hypot(orbit.re_d[b] - orbit.re_d[a], orbit.im_d[b] - orbit.im_d[a]);
                const double d2 = std::hypot(orbit.re_d[c] - orbit.re_d[b], orbit.im_d[c] - orbit.im_d[b]);
                if (!(d1 <= tolerance * scale && d2 <= tolerance * scale)) matches = false;
            }
            if (!matches) continue;
            for (std::size_t target = start; target < count; ++target) {
                const std::size_t source = start + (target - start) % static_cast<std::size_t>(period);
                fast[target] = fast[source];
                orbit.scaled[target] = orbit.scaled[source];
                orbit.re_d[target] = orbit.re_d[source];
                orbit.im_d[target] = orbit.im_d[source];
                if (target < orbit.escape_margin.size() && source < orbit.escape_margin.size()) {
                    orbit.escape_margin[target] = orbit.escape_margin[source];
                }
            }
            return;
        }
    }
}

void make_orbit(ReferenceContext& ctx, const char* x_text, const char* y_text,
                const char* zoom_text, int max_iter, int precision_bits, int formula,
                const char* julia_re_text, const char* julia_im_text) {
    const MpfrApi& m = need_mpfr();
    ctx.requested_max_iter = max_iter;
    ctx.x_text = x_text;
    ctx.y_text = y_text;
    precision_bits = std::max(128, precision_bits);
    const long p = precision_bits;
    Mp cx(p), cy(p), zoom(p), radius(p), par_re(p), par_im(p), zr(p), zi(p), next_re(p),
        next_im(p), tmp(p), abs_re(p), abs_im(p), norm2(p), margin(p);
    if (m.set_str(cx, x_text, 10, RNDN) != 0 || m.set_str(cy, y_text, 10, RNDN) != 0) {
        throw Failure{"invalid MPFR Mandelbrot centre"};
    }
    const bool zoom_ok = zoom_text && m.set_str(zoom, zoom_text, 10, RNDN) == 0 && m.sgn(zoom) > 0;
    if (zoom_ok) {
        m.set_d(radius, viewport_height_factor(ctx.coordinate_mode), RNDN);
        m.div(radius, radius, zoom, RNDN);
        ctx.input_radius = fe_from_mpfr(radius);
    } else {
        ctx.input_radius = fx::fe_from(1.0, 0);
    }
    if (formula == kFormulaJulia) {
        if (m.set_str(par_re, julia_re_text, 10, RNDN) != 0 || m.set_str(par_im, julia_im_text, 10, RNDN) != 0) {
            throw Failure{"invalid MPFR Julia constant"};
        }
        m.set(zr, cx, RNDN);
        m.set(zi, cy, RNDN);
    } else {
        m.set(par_re, cx, RNDN);
        m.set(par_im, cy, RNDN);
        m.set_zero(zr, 0);
        m.set_zero(zi, 0);
    }
    ctx.formula = formula;
    ctx.julia_re = static_cast<double>(parse_coordinate(julia_re_text, "Julia real"));
    ctx.julia_im = static_cast<double>(parse_coordinate(julia_im_text, "Julia imaginary"));
    ctx.parameter = fx::sc_from_fe(fe_from_mpfr(par_re), fe_from_mpfr(par_im));
    ctx.precision_bits = p;

    bool fixed_point = false;
    if (formula == kFormulaJulia) {
        // Repelling fixed point of z^2 + c recovered at working precision
        // (renderer.cpp:10737-10815): z* = (1 +- sqrt(1 - 4c)) / 2, the root
        // with the larger modulus, used when the centre text matches it.
        Mp disc_re(p), disc_im(p), disc_mag(p), root_re(p), root_im(p), a_re(p), a_im(p),
            b_re(p), b_im(p), a_norm(p), b_norm(p), dist2(p), mult2(p), tol(p), zlog(p);
        m.set_ui(tmp, 4, RNDN);
        m.mul(disc_re, par_re, tmp, RNDN);
        m.ui_sub(disc_re, 1, disc_re, RNDN);
        m.mul(disc_im, par_im, tmp, RNDN);
        m.neg(disc_im, disc_im, RNDN);
        m.mul(norm2, disc_re, disc_re, RNDN);
        m.mul(tmp, disc_im, disc_im, RNDN);
        m.add(norm2, norm2, tmp, RNDN);
        m.sqrt(disc_mag, norm2, RNDN);
        m.add(root_re, disc_mag, disc_re, RNDN);
        m.div_2ui(root_re, root_re, 1, RNDN);
        m.sqrt(root_re, root_re, RNDN);
        m.sub(root_im, disc_mag, disc_re, RNDN);
        m.div_2ui(root_im, root_im, 1, RNDN);
        m.sqrt(root_im, root_im, RNDN);
        if (m.sgn(disc_im) < 0) m.neg(root_im, root_im, RNDN);
        m.add_ui(a_re, root_re, 1, RNDN);
        m.div_2ui(a_re, a_re, 1, RNDN);
        m.div_2ui(a_im, root_im, 1, RNDN);
        m.set_ui(tmp, 1, RNDN);
        m.sub(b_re, tmp, root_re, RNDN);
        m.div_2ui(b_re, b_re, 1, RNDN);
        m.neg(b_im, a_im, RNDN);
        m.mul(a_norm, a_re, a_re, RNDN);
        m.mul(tmp, a_im, a_im, RNDN);
        m.add(a_norm, a_norm, tmp, RNDN);
        m.mul(b_norm, b_re, b_re, RNDN);
        m.mul(tmp, b_im, b_im, RNDN);
        m.add(b_norm, b_norm, tmp, RNDN);
        if (m.cmp(a_norm, b_norm) >= 0) {
            m.set(next_re, a_re, RNDN);
            m.set(next_im, a_im, RNDN);
            m.set(norm2, a_norm, RNDN);
        } else {
            m.set(next_re, b_re, RNDN);
            m.set(next_im, b_im, RNDN);
            m.set(norm2, b_norm, RNDN);
        }
        m.mul_ui(mult2, norm2, 4, RNDN);
        m.log10(zlog, zoom, RNDN);
        const double log_zoom = m.get_d(zlog, RNDN);
        const int digits = std::max(32, static_cast<int>(std::ceil(std::max(0.0, log_zoom))) + 16);
        m.set_ui(tol, 10, RNDN);
        m.pow_si(tol, tol, -static_cast<long>(digits), RNDN);
        m.sub(tmp, cx, next_re, RNDN);
        m.mul(dist2, tmp, tmp, RNDN);
        m.sub(tmp, cy, next_im, RNDN);
        m.mul(norm2, tmp, tmp, RNDN);
        m.add(dist2, dist2, norm2, RNDN);
        m.mul(norm2, tol, tol, RNDN);
        if (m.cmp_ui(mult2, 1) > 0 && m.cmp(dist2, norm2) <= 0) {
            m.set(zr, next_re, RNDN);
            m.set(zi, next_im, RNDN);
            fixed_point = true;
        }
    }

    ctx.fast_orbit.clear();
    ctx.fast_orbit.reserve(static_cast<std::size_t>(max_iter) + 1U);
    std::vector<fx::Fe> margins;
    margins.reserve(static_cast<std::size_t>(max_iter) + 1U);
    fx::Fe orbit_re = fe_from_mpfr(zr);
    fx::Fe orbit_im = fe_from_mpfr(zi);
    std::size_t finite_size = 0;
    for (int i = 0; i <= max_iter; ++i) {
        if (!fx::fe_finite(orbit_re) || !fx::fe_finite(orbit_im)) break;
        ctx.fast_orbit.push_back(fx::fec_make(orbit_re, orbit_im));
        m.mul(norm2, zr, zr, RNDN);
        m.mul(tmp, zi, zi, RNDN);
        m.add(norm2, norm2, tmp, RNDN);
        m.set_d(tmp, fx::escape_r2_d(ctx.escape_mode), RNDN);
        m.sub(margin, norm2, tmp, RNDN);
        margins.push_back(fe_from_mpfr(margin));
        finite_size = ctx.fast_orbit.size();
        if (fixed_point) continue;
        if (formula == kFormulaBurningShip) {
            m.abs(abs_re, zr, RNDN);
            m.abs(abs_im, zi, RNDN);
            m.mul(next_re, abs_re, abs_re, RNDN);
            m.mul(tmp, abs_im, abs_im, RNDN);
            m.sub(next_re, next_re, tmp, RNDN);
            m.add(next_re, next_re, par_re, RNDN);
            m.mul(next_im, abs_re, abs_im, RNDN);
            m.mul_ui(next_im, next_im, 2, RNDN);
            m.add(next_im, next_im, par_im, RNDN);
        } else {
            m.mul(next_re, zr, zr, RNDN);
            m.mul(tmp, zi, zi, RNDN);
            m.sub(next_re, next_re, tmp, RNDN);
            m.mul(next_im, zr, zi, RNDN);
            m.mul_ui(next_im, next_im, 2, RNDN);
            if (formula == kFormulaTricorn) m.neg(next_im, next_im, RNDN);
            m.add(next_re, next_re, par_re, RNDN);
            m.add(next_im, next_im, par_im, RNDN);
        }
        m.set(zr, next_re, RNDN);
        m.set(zi, next_im, RNDN);
        orbit_re = fe_from_mpfr(zr);
        orbit_im = fe_from_mpfr(zi);
    }
    if (finite_size == 0) throw Failure{"reference orbit lost finite state at iteration zero"};
    const fx::Fe escape_r2 = fx::escape_r2_fe(ctx.escape_mode);
    ctx.map_end = static_cast<int>(finite_size) - 1;
    for (std::size_t i = 1; i < finite_size; ++i) {
        if (fx::fe_cmp(fx::fec_norm2(ctx.fast_orbit[i]), escape_r2) > 0) {
            ctx.map_end = static_cast<int>(i);
            break;
        }
    }
    auto orbit = std::make_shared<OrbitData>();
    orbit->scaled.resize(ctx.fast_orbit.size());
    orbit->escape_margin = std::move(margins);
    for (std::size_t i = 0; i < ctx.fast_orbit.size(); ++i) {
        orbit->scaled[i] = fx::sc_from_fe(ctx.fast_orbit[i].re, ctx.fast_orbit[i].im);
    }
    orbit->re_d.resize(orbit->scaled.size());
    orbit->im_d.resize(orbit->scaled.size());
    for (std::size_t i = 0; i < orbit->scaled.size(); ++i) {
        orbit->re_d[i] = fx::scale2(orbit->scaled[i].re, orbit->scaled[i].e);
        orbit->im_d[i] = fx::scale2(orbit->scaled[i].im, orbit->scaled[i].e);
    }
    if (formula != kFormulaMandelbrot) {
        stabilize_alternate_cycle(ctx.fast_orbit, *orbit, ctx.escape_mode);
        ctx.map_end = static_cast<int>(orbit->scaled.size()) - 1;
        for (std::size_t i = 1; i < orbit->scaled.size(); ++i) {
            if (fx::fe_cmp(fx::fec_norm2(ctx.fast_orbit[i]), escape_r2) > 0) {
                ctx.map_end = static_cast<int>(i);
                break;
            }
        }
    }
    ctx.orbit = std::move(orbit);
}

// ------------------------------------------------------------ image series
fx::Fec series_value(const std::vector<fx::Fec>& coeff, const fx::Fec& dc) {
    if (coeff.size() <= 1) return fx::fec_make(fx::fe_zero(), fx::fe_zero());
    fx::Fec r = coeff.back();
    for (std::size_t i = coeff.size() - 1; i > 1; --i) r = fx::fec_add(fx::fec_mul(r, dc), coeff[i - 1]);
    return fx::fec_mul(r, dc);
}

bool probe_ok(const fx::Fec& reference, const fx::Fec& exact, const fx::Fec& approx,
              const fx::Fe& min_scale2, const fx::Fe& tol2, int mode) {
    const fx::Fec err = fx::fec_sub(approx, exact);
    fx::Fe scale = fx::fec_norm2(exact);
    if (fx::fe_cmp(scale, min_scale2) < 0) scale = min_scale2;
    const fx::Fe allowed = fx::fe_mul(scale, tol2);
    if (fx::fe_cmp(fx::fec_norm2(err), allowed) > 0) return false;
    const bool exact_in = fx::fe_cmp(fx::fec_escape_margin(reference, exact, mode), fx::fe_zero()) <= 0;
    const bool approx_in = fx::fe_cmp(fx::fec_escape_margin(reference, approx, mode), fx::fe_zero()) <= 0;
    return exact_in && approx_in;
}

// build_image_series (renderer.cpp:11206-11334): a polynomial in dc with no
// constant term, advanced one reference step at a time and kept while all
// twelve probes agree with the exact recurrence within 2^-38 relative.
void build_image_series(ReferenceContext& ctx, const std::vector<fx::Fec>* override_orbit = nullptr) {
    ctx.series = ImageSeries{};
    const bool julia = ctx.formula == kFormulaJulia;
    if (ctx.formula != kFormulaMandelbrot && !julia) return;
    const std::vector<fx::Fec>& orbit = override_orbit ? *override_orbit : ctx.fast_orbit;
    if (orbit.size() < 16 || ctx.requested_max_iter < 8) return;
    const int order = std::clamp(ctx.requested_series_order, 8, 32);
    const int map_end = std::clamp(ctx.map_end, 2, static_cast<int>(orbit.size()) - 1);
    const int last_candidate = std::max(2, map_end - 1);
    const fx::Fe radius = ctx.input_radius;
    if (fx::fe_is_zero(radius) || !fx::fe_finite(radius)) return;
    const fx::Fe probe_r = fx::fe_mul(radius, 1.5);
    const fx::Fe diag = fx::fe_mul(probe_r, 0.7071067811865476);
    const fx::Fe inner = fx::fe_mul(probe_r, 0.47);
    const fx::Fe z = fx::fe_zero();
    const std::array<fx::Fec, 12> probes{{
        fx::fec_make(probe_r, z),
        fx::fec_make(fx::fe_neg(probe_r), z),
        fx::fec_make(z, probe_r),
        fx::fec_make(z, fx::fe_neg(probe_r)),
        fx::fec_make(diag, diag),
        fx::fec_make(fx::fe_neg(diag), diag),
        fx::fec_make(diag, fx::fe_neg(diag)),
        fx::fec_make(fx::fe_neg(diag), fx::fe_neg(diag)),
        fx::fec_make(inner, fx::fe_mul(inner, 0.63)),
        fx::fec_make(fx::fe_neg(inner), fx::fe_mul(inner, 0.63)),
        fx::fec_make(fx::fe_mul(inner, 0.63), inner),
        fx::fec_make(fx::fe_mul(inner, 0.63), fx::fe_neg(inner)),
    }};
    const fx::Fec zero_c = fx::fec_make(z, z);
    std::vector<fx::Fec> coeff(static_cast<std::size_t>(order + 1), zero_c);
    std::vector<fx::Fec> next(static_cast<std::size_t>(order + 1), zero_c);
    std::array<fx::Fec, 12> exact;
    exact.fill(zero_c);
    if (julia) {
        coeff[1] = fx::fec_make(fx::fe_from(1.0, 0), z);
        for (std::size_t k = 0; k < probes.size(); ++k) exact[k] = probes[k];
    }
    std::vector<fx::Fec> best;
    int best_iteration = 1;
    const fx::Fe tol2 = fx::fe_from(std::ldexp(1.0, -38), 0);
    const fx::Fe min_scale2 = fx::fe_sqr(probe_r);
    const fx::Fe two = fx::fe_from(2.0, 0);
    const fx::Fec one_c = fx::fec_make(fx::fe_from(1.0, 0), z);
    for (int it = 0; it < last_candidate; ++it) {
        const fx::Fec& ref = orbit[static_cast<std::size_t>(it)];
        std::fill(next.begin(), next.end(), zero_c);
        for (int term = 1; term <= order; ++term) {
            fx::Fec value = fx::fec_scale(fx::fec_mul(ref, coeff[static_cast<std::size_t>(term)]), two);
            for (int left = 1; left < term; ++left) {
                value = fx::fec_add(value, fx::fec_mul(coeff[static_cast<std::size_t>(left)],
                                                       coeff[static_cast<std::size_t>(term - left)]));
            }
            if (!julia && term == 1) value = fx::fec_add(value, one_c);
            next[static_cast<std::size_t>(term)] = value;
        }
        coeff.swap(next);
        bool safe = true;
        for (std::size_t k = 0; k < probes.size(); ++k) {
            const fx::Fec& dc = probes[k];
            const fx::Fec exact_next = fx::fec_add(
                fx::fec_scale(fx::fec_mul(ref, exact[k]), two),
                fx::fec_add(fx::fec_mul(exact[k], exact[k]), julia ? zero_c : dc));
            exact[k] = exact_next;
            if (it + 1 >= order) {
                const fx::Fec approx = series_value(coeff, dc);
                if (!probe_ok(orbit[static_cast<std::size_t>(it + 1)], exact_next, approx, min_scale2,
                              tol2, ctx.escape_mode)) {
                    safe = false;
                    break;
                }
            }
        }
        if (!safe) break;
        if (it + 1 >= order) {
            best_iteration = it + 1;
            best = coeff;
        }
    }
    if (best_iteration <= 1 || best.empty()) return;
    ctx.series.enabled = true;
    ctx.series.order = order;
    ctx.series.iteration = best_iteration;
    ctx.series.r2 = fx::fe_sqr(probe_r);
    ctx.series.coeff.reserve(best.size());
    for (const fx::Fec& c : best) ctx.series.coeff.push_back(fx::sc_from_fe(c.re, c.im));
}

// -------------------------------------------------------- Mandelbrot BLA
std::vector<std::vector<LinearStep>> build_linear_levels(const ReferenceContext& ctx, int base_count,
                                                        const fx::Fe& input_radius) {
    std::vector<std::vector<BuilderLinear>> levels;
    levels.emplace_back(static_cast<std::size_t>(base_count));
    for (int start = 1; start <= base_count; ++start) {
        levels[0][static_cast<std::size_t>(start - 1)] = linear_base(ctx.fast_orbit[static_cast<std::size_t>(start)]);
    }
    for (std::size_t level = 1;; ++level) {
        if ((1ULL << level) > static_cast<unsigned long long>(kMaxSafeLinearBlaLength)) break;
        const std::size_t prev = levels[level - 1].size();
        const std::size_t cur = (prev + 1) / 2;
        if (cur == 0) break;
        levels.emplace_back(cur);
        for (std::size_t i = 0; i < cur; ++i) {
            const std::size_t first = i * 2;
            levels[level][i] = first + 1 < prev
                ? merge_linear(levels[level - 1][first + 1], levels[level - 1][first], input_radius)
                : levels[level - 1][first];
        }
    }
    std::vector<std::vector<LinearStep>> out;
    out.reserve(levels.size());
    for (const auto& level : levels) {
        auto& dst = out.emplace_back();
        dst.reserve(level.size());
        for (const BuilderLinear& s : level) dst.push_back(compact_linear(s));
    }
    return out;
}

std::uint64_t elapsed_ns(std::chrono::steady_clock::time_point start) {
    return static_cast<std::uint64_t>(
        std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - start)
            .count());
}

// build_bla (renderer.cpp:11612-11769).
void build_bla(ReferenceContext& ctx, bool retain_builder_orbit) {
    const int max_iter = static_cast<int>(ctx.fast_orbit.size()) - 1;
    const int map_end = std::clamp(ctx.map_end, 0, max_iter);
    const int base_count = std::max(0, std::min(max_iter, map_end) - 1);
    const auto series_started = std::chrono::steady_clock::now();
    build_image_series(ctx);
    ctx.series_build_ns = elapsed_ns(series_started);
    ctx.cubic.clear();
    ctx.linear.clear();
    ctx.deep_linear.clear();
    if (base_count == 0) {
        if (!retain_builder_orbit) {
            ctx.fast_orbit.clear();
            ctx.fast_orbit.shrink_to_fit();
        }
        return;
    }
    if (device_table_builder()) {
        build_bla_on_device(ctx, base_count);
        if (!retain_builder_orbit) {
            ctx.fast_orbit.clear();
            ctx.fast_orbit.shrink_to_fit();
        }
        return;
    }
    std::vector<std::vector<BuilderCubic>> levels;
    levels.emplace_back(static_cast<std::size_t>(base_count));
    for (int start = 1; start <= base_count; ++start) {
        levels[0][static_cast<std::size_t>(start - 1)] = cubic_base(ctx.fast_orbit[static_cast<std::size_t>(start)]);
    }
    for (std::size_t level = 1;; ++level) {
        if ((1ULL << level) > static_cast<unsigned long long>(kMaxSafeBlaLength)) break;
        const std::size_t prev = levels[level - 1].size();
        const std::size_t cur = prev / 2;
        if (cur == 0) break;
        levels.emplace_back(cur);
        for (std::size_t i = 0; i < cur; ++i) {
            levels[level][i] = merge_cubic(levels[level - 1][i * 2 + 1], levels[level - 1][i * 2],
                                           ctx.input_radius);
        }
    }
    ctx.cubic.reserve(levels.size());
    for (const auto& level : levels) {
        auto& dst = ctx.cubic.emplace_back();
        dst.reserve(level.size());
        for (const BuilderCubic& s : level) dst.push_back(compact_cubic(s));
    }
    ctx.deep_input_radius = fx::fe_mul(ctx.input_radius, 1.0e-20);
    ctx.linear = build_linear_levels(ctx, base_count, ctx.input_radius);
    ctx.deep_linear = build_linear_levels(ctx, base_count, ctx.deep_input_radius);
    if (!retain_builder_orbit) {
        ctx.fast_orbit.clear();
        ctx.fast_orbit.shrink_to_fit();
    }
}

void retarget_cubic(std::vector<std::vector<CubicStep>>& levels, const fx::Fe& input_radius) {
    for (std::size_t level = 1; level < levels.size(); ++level) {
        const auto& prev = levels[level - 1];
        auto& cur = levels[level];
        for (std::size_t i = 0; i < cur.size(); ++i) {
            const CubicStep& x = prev[i * 2];
            const CubicStep& y = prev[i * 2 + 1];
            cur[i].r2 = retarget_radius(x.r2, y.r2, x.c[0], x.c[1], input_radius);
        }
    }
}

void retarget_linear(std::vector<std::vector<LinearStep>>& levels, const fx::Fe& input_radius) {
    for (std::size_t level = 1; level < levels.size(); ++level) {
        const auto& prev = levels[level - 1];
        auto& cur = levels[level];
        for (std::size_t i = 0; i < cur.size(); ++i) {
            const std::size_t first = i * 2;
            if (first + 1 >= prev.size()) {
                cur[i].r2 = prev[first].r2;
                continue;
            }
            cur[i].r2 = retarget_radius(prev[first].r2, prev[first + 1].r2, prev[first].a, prev[first].b,
                                        input_radius);
        }
    }
}

// ------------------------------------------------------ alternate formulas
// build_alternate_linear_bla (renderer.cpp:11414-11526).
void build_alt_bla(ReferenceContext& ctx, bool retain_builder_orbit) {
    using namespace fx;
    ctx.alt.clear();
    ctx.alt_input_radius = ctx.input_radius;
    ctx.alt_input_radius2 = fe_sqr(ctx.input_radius);
    ctx.alt_start = ctx.formula == kFormulaJulia ? 0 : 1;
    if (ctx.fast_orbit.size() < 2) return;
    const int first = ctx.alt_start;
    const int last = std::min(ctx.map_end, static_cast<int>(ctx.fast_orbit.size()) - 1);
    const int base_count = last - first;
    if (base_count <= 0) return;
    if (device_table_builder()) {
        build_alt_bla_on_device(ctx, first, base_count);
        if (!retain_builder_orbit) {
            ctx.fast_orbit.clear();
            ctx.fast_orbit.shrink_to_fit();
        }
        return;
    }
    auto& base = ctx.alt.emplace_back(static_cast<std::size_t>(base_count));
    for (int k = 0; k < base_count; ++k) {
        base[static_cast<std::size_t>(k)] = alt_base(ctx.fast_orbit[static_cast<std::size_t>(first + k)], ctx.formula);
    }
    for (std::size_t level = 1;; ++level) {
        if ((1ULL << level) > static_cast<unsigned long long>(kMaxSafeLinearBlaLength)) break;
        const std::size_t prev = ctx.alt[level - 1].size();
        const std::size_t cur = (prev + 1) / 2;
        if (cur == 0) break;
        auto& dst = ctx.alt.emplace_back(cur);
        const auto& src = ctx.alt[level - 1];
        for (std::size_t i = 0; i < cur; ++i) {
            const std::size_t f = i * 2;
            dst[i] = f + 1 < prev ? merge_alt(src[f + 1], src[f], ctx.alt_input_radius) : src[f];
        }
    }
    if (!retain_builder_orbit) {
        ctx.fast_orbit.clear();
        ctx.fast_orbit.shrink_to_fit();
    }
}

// ------------------------------------------------------------ registry
std::mutex registry_mutex;
std::unordered_map<std::uintptr_t, std::shared_ptr<ReferenceContext>> registry;
std::uintptr_t next_token = 0x1000U;

}  // namespace

std::unique_ptr<ReferenceContext> create_reference_context(
    const char* x_center, const char* y_center, const char* viewport_zoom, int max_iter,
    int precision_bits, int series_order, bool retain_builder_orbit, int formula,
    const char* julia_re, const char* julia_im, int escape_mode, int coordinate_mode) {
    if (!valid_text(x_center) || !valid_text(y_center) || !valid_text(viewport_zoom)) {
        throw Failure{"native reference text is too long or null"};
    }
    (void)parse_zoom_fe(viewport_zoom, precision_bits);
    if (formula < 0 || formula > 3 || (escape_mode != 0 && escape_mode != 1)
        || (coordinate_mode != 0 && coordinate_mode != 1) || !valid_text(julia_re)
        || !valid_text(julia_im)) {
        throw Failure{"invalid native reference formula or Julia constant"};
    }
    auto ctx = std::make_unique<ReferenceContext>();
    ctx->x_center = parse_coordinate(x_center, "real");
    ctx->y_center = parse_coordinate(y_center, "imaginary");
    ctx->formula = formula;
    ctx->escape_mode = escape_mode;
    ctx->coordinate_mode = coordinate_mode;
    ctx->julia_re = static_cast<double>(parse_coordinate(julia_re, "Julia real"));
    ctx->julia_im = static_cast<double>(parse_coordinate(julia_im, "Julia imaginary"));
    ctx->requested_series_order = std::clamp(series_order, 8, 32);
    const auto orbit_started = std::chrono::steady_clock::now();
    make_orbit(*ctx, x_center, y_center, viewport_zoom, max_iter, precision_bits, formula, julia_re,
               julia_im);
    ctx->reference_build_ns = elapsed_ns(orbit_started);
    const auto bla_started = std::chrono::steady_clock::now();
    if (formula == kFormulaMandelbrot) {
        build_bla(*ctx, retain_builder_orbit);
    } else {
        if (formula == kFormulaJulia) {
            const auto series_started = std::chrono::steady_clock::now();
            build_image_series(*ctx);
            ctx->series_build_ns = elapsed_ns(series_started);
        } else {
            ctx->series_build_ns = 0;
        }
        build_alt_bla(*ctx, retain_builder_orbit);
    }
    ctx->bla_build_ns = elapsed_ns(bla_started);
    return ctx;
}

// clone_reference_context (renderer.cpp:13705-13768).
std::unique_ptr<ReferenceContext> clone_reference_context(const ReferenceContext& source,
                                                          const char* viewport_zoom) {
    if (!source.orbit || source.fast_orbit.empty()) {
        throw Failure{"reference was not created as a reusable tier root"};
    }
    const auto started = std::chrono::steady_clock::now();
    auto ctx = std::make_unique<ReferenceContext>();
    ctx->orbit = source.orbit;
    ctx->map_end = source.map_end;
    ctx->requested_max_iter = source.requested_max_iter;
    ctx->requested_series_order = source.requested_series_order;
    ctx->x_center = source.x_center;
    ctx->y_center = source.y_center;
    ctx->x_text = source.x_text;
    ctx->y_text = source.y_text;
    ctx->formula = source.formula;
    ctx->julia_re = source.julia_re;
    ctx->julia_im = source.julia_im;
    ctx->parameter = source.parameter;
    ctx->escape_mode = source.escape_mode;
    ctx->coordinate_mode = source.coordinate_mode;
    ctx->precision_bits = source.precision_bits;
    ctx->reference_build_ns = elapsed_ns(started);
    const auto bla_started = std::chrono::steady_clock::now();
    const fx::Fe zoom = parse_zoom_fe(viewport_zoom, ctx->precision_bits);
    ctx->input_radius = fx::fe_div(fx::fe_from(viewport_height_factor(ctx->coordinate_mode), 0), zoom);
    if (source.formula != kFormulaMandelbrot) {
        ctx->fast_orbit = source.fast_orbit;
        if (source.formula == kFormulaJulia) {
            const auto series_started = std::chrono::steady_clock::now();
            build_image_series(*ctx);
            ctx->series_build_ns = elapsed_ns(series_started);
        }
        build_alt_bla(*ctx, false);
        if (source.formula != kFormulaJulia) ctx->series_build_ns = 0;
        ctx->bla_build_ns = elapsed_ns(bla_started);
        return ctx;
    }
    const auto series_started = std::chrono::steady_clock::now();
    build_image_series(*ctx, &source.fast_orbit);
    ctx->series_build_ns = elapsed_ns(series_started);
    if (source.bla_on_device) {
        retarget_bla_on_device(*ctx, source);
        ctx->bla_build_ns = elapsed_ns(bla_started);
        return ctx;
    }
    ctx->cubic = source.cubic;
    retarget_cubic(ctx->cubic, ctx->input_radius);
    ctx->linear = source.linear;
    retarget_linear(ctx->linear, ctx->input_radius);
    ctx->deep_input_radius = fx::fe_mul(ctx->input_radius, 1.0e-20);
    ctx->deep_linear = source.linear;
    retarget_linear(ctx->deep_linear, ctx->deep_input_radius);
    ctx->bla_build_ns = elapsed_ns(bla_started);
    return ctx;
}

namespace {
std::atomic<bool> table_builder_on_device{true};
}

bool device_table_builder() { return table_builder_on_device.load(std::memory_order_relaxed); }
void set_device_table_builder(bool on_device) { table_builder_on_device.store(on_device, std::memory_order_relaxed); }

void* register_reference(std::unique_ptr<ReferenceContext> context) {
    if (!context) throw Failure{"cannot register an empty reference"};
    std::shared_ptr<ReferenceContext> shared(std::move(context));
    std::lock_guard<std::mutex> lock(registry_mutex);
    for (;;) {
        const std::uintptr_t token = next_token++;
        if (token == 0 || registry.count(token) != 0) continue;
        shared->generation = static_cast<std::uint64_t>(token);
        registry.emplace(token, std::move(shared));
        return reinterpret_cast<void*>(token);
    }
}

std::shared_ptr<ReferenceContext> acquire_reference(void* handle) {
    if (!handle) return {};
    std::lock_guard<std::mutex> lock(registry_mutex);
    const auto found = registry.find(reinterpret_cast<std::uintptr_t>(handle));
    return found == registry.end() ? nullptr : found->second;
}

std::shared_ptr<ReferenceContext> remove_reference(void* handle) {
    if (!handle) return {};
    std::lock_guard<std::mutex> lock(registry_mutex);
    const auto found = registry.find(reinterpret_cast<std::uintptr_t>(handle));
    if (found == registry.end()) return {};
    auto context = std::move(found->second);
    registry.erase(found);
    return context;
}

std::vector<OrbitRec> make_orbit_records(const ReferenceContext& ctx) {
    const OrbitData& orbit = *ctx.orbit;
    std::vector<OrbitRec> records(orbit.scaled.size());
    const fx::Fe escape_r2 = fx::escape_r2_fe(ctx.escape_mode);
    for (std::size_t i = 0; i < orbit.scaled.size(); ++i) {
        OrbitRec& r = records[i];
        std::memset(&r, 0, sizeof r);
        r.z = orbit.scaled[i];
        r.zd_re = orbit.re_d[i];
        r.zd_im = orbit.im_d[i];
        r.parts = fx::sc_to_fec(orbit.scaled[i]);
        // Mandelbrot rebuilds the escape margin from the compact orbit
        // (renderer.cpp:8374-8390); the other formulas use the MPFR margin
        // of each step (renderer.cpp:12037-12052).
        r.margin = ctx.formula == kFormulaMandelbrot || i >= orbit.escape_margin.size()
            ? fx::fe_sub(fx::fec_norm2(r.parts), escape_r2)
            : orbit.escape_margin[i];
        const fx::Nrm n = fx::sc_norm2(orbit.scaled[i]);
        const fx::Fe norm = fx::fe_make(n.m, n.e);
        r.glitch = (norm.m != 0.0 && fx::fe_finite(norm)) ? fx::fe_mul(norm, 1.0e-7) : fx::fe_zero();
    }
    return records;
}


// ------------------------------------------------------------ exact points
namespace {

// render_plane_phase (renderer.cpp:8075-8082).
double exact_plane_phase(const fx::Sc& v) {
    const double re = fx::sc_re_d(v);
    const double im = fx::sc_im_d(v);
    if (!std::isfinite(re) || !std::isfinite(im)) return 0.0;
    constexpr double two_pi = 6.283185307179586476925286766559005768;
    double phase = std::atan2(im, re) / two_pi;
    phase -= std::floor(phase);
    return std::isfinite(phase) ? phase : 0.0;
}

// render_plane_de (renderer.cpp:7845-7897), with its long double log2 term.
bool exact_plane_de(const fx::Sc& total, const fx::Sc& derivative, const fx::Fe& spacing, double& out_re,
                    double& out_im) {
    constexpr long double log_two = 0.693147180559945309417232121458176568L;
    const double mag = std::hypot(total.re, total.im);
    if (!(mag > 0.0) || !std::isfinite(mag)) return false;
    const double log_mag = static_cast<double>(std::log(mag) + static_cast<double>(total.e) * log_two);
    if (!(log_mag > 0.0) || !std::isfinite(log_mag)) return false;
    const fx::Sc unit = fx::sc_from_fe(fx::fe_from(total.re / mag, 0), fx::fe_from(total.im / mag, 0));
    const fx::Sc spacing_c = fx::sc_from_fe(spacing, fx::fe_zero());
    const fx::Sc den = fx::sc_mul(unit, fx::sc_mul(fx::sc_conj(derivative), spacing_c));
    const double den2 = den.re * den.re + den.im * den.im;
    if (!(den2 > 0.0) || !std::isfinite(den2)) return false;
    fx::Sc r = fx::sc_make(mag * log_mag * den.re / den2, -mag * log_mag * den.im / den2,
                           fx::sat_exp(static_cast<long long>(total.e) - den.e));
    fx::sc_normalize(r);
    out_re = fx::sc_re_d(r);
    out_im = fx::sc_im_d(r);
    return std::isfinite(out_re) && std::isfinite(out_im);
}

}  // namespace

bool exact_mandelbrot_pixel(const ReferenceContext& ctx, const fx::Sc& dc, int max_iter, double output_bias,
                            int escape_mode, const fx::Fe& pixel_spacing, float& out, ExactPlanes* planes) {
    const MpfrApi& m = mpfr();
    if (!m.exact_ok || ctx.x_text.empty() || ctx.y_text.empty() || ctx.precision_bits < 128
        || !fx::sc_finite(dc)) {
        return false;
    }
    // Precision floor from the pixel spacing (renderer.cpp:10953-10961).
    long precision = ctx.precision_bits;
    if (pixel_spacing.e < 0) {
        const long spacing_precision = -static_cast<long>(pixel_spacing.e) + 128;
        precision = std::min(precision, std::max(256L, spacing_precision));
    }
    Mp cr(precision), ci(precision), zr(precision), zi(precision), dr(precision), di(precision);
    Mp nr(precision), ni(precision), ndr(precision), ndi(precision), t(precision), n2(precision);
    if (m.set_str(cr, ctx.x_text.c_str(), 10, RNDN) != 0 || m.set_str(ci, ctx.y_text.c_str(), 10, RNDN) != 0) {
        return false;
    }
    // c = centre + dc, the binary offset added at full precision.
    m.set_d(t, dc.re, RNDN);
    m.mul_2si(t, t, static_cast<long>(dc.e), RNDN);
    m.add(cr, cr, t, RNDN);
    m.set_d(t, dc.im, RNDN);
    m.mul_2si(t, t, static_cast<long>(dc.e), RNDN);
    m.add(ci, ci, t, RNDN);
    m.set_zero(zr, 0);
    m.set_zero(zi, 0);
    m.set_zero(dr, 0);
    m.set_zero(di, 0);
    fx::Nrm previous = fx::nrm_make(0.0, 0);
    const double escape2 = fx::escape_r2_d(escape_mode);
    for (int iteration = 1; iteration <= max_iter; ++iteration) {
        m.mul(nr, zr, zr, RNDN);
        m.mul(t, zi, zi, RNDN);
        m.sub(nr, nr, t, RNDN);
        m.mul(ni, zr, zi, RNDN);
        m.mul_ui(ni, ni, 2, RNDN);
        m.add(nr, nr, cr, RNDN);
        m.add(ni, ni, ci, RNDN);
        m.mul(ndr, zr, dr, RNDN);
        m.mul(t, zi, di, RNDN);
        m.sub(ndr, ndr, t, RNDN);
        m.mul_ui(ndr, ndr, 2, RNDN);
        m.add_ui(ndr, ndr, 1, RNDN);
        m.mul(ndi, zr, di, RNDN);
        m.mul(t, zi, dr, RNDN);
        m.add(ndi, ndi, t, RNDN);
        m.mul_ui(ndi, ndi, 2, RNDN);
        m.set(zr, nr, RNDN);
        m.set(zi, ni, RNDN);
        m.set(dr, ndr, RNDN);
        m.set(di, ndi, RNDN);
        m.mul(n2, zr, zr, RNDN);
        m.mul(t, zi, zi, RNDN);
        m.add(n2, n2, t, RNDN);
        const fx::Sc total = fx::sc_from_fe(fe_from_mpfr(zr), fe_from_mpfr(zi));
        const fx::Nrm current = fx::sc_norm2(total);
        if (m.cmp_d(n2, escape2) > 0) {
            m.log(t, n2, RNDN);
            const long double log_magnitude = 0.5L * m.get_ld(t, RNDN);
            if (!(log_magnitude > 0.0L) || !std::isfinite(log_magnitude)) return false;
            constexpr long double log_two = 0.693147180559945309417232121458176568L;
            const long double smooth = static_cast<long double>(iteration) - std::log(log_magnitude) / log_two;
            out = static_cast<float>(smooth - static_cast<long double>(output_bias));
            if (planes) {
                const fx::Sc derivative = fx::sc_from_fe(fe_from_mpfr(dr), fe_from_mpfr(di));
                planes->iteration = iteration - 1 > 0 ? iteration - 1 : 0;
                planes->phase = exact_plane_phase(total);
                planes->de_x = 0.0;
                planes->de_y = 0.0;
                double de_x = 0.0, de_y = 0.0;
                if (exact_plane_de(total, derivative, pixel_spacing, de_x, de_y)) {
                    planes->de_x = de_x;
                    planes->de_y = de_y;
                }
                planes->test1 = fx::nrm_to_d(current);
                planes->test2 = fx::nrm_to_d(previous);
            }
            return true;
        }
        previous = current;
    }
    out = static_cast<float>(static_cast<long double>(max_iter) - static_cast<long double>(output_bias));
    if (planes) *planes = ExactPlanes{max_iter, 0.0, 0.0, 0.0, 0.0, 0.0};
    return true;
}

}  // namespace fgb
