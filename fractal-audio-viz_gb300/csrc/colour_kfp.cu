// Kalles .kfp colour transfer on the scalar field, one thread per pixel.
//
// Restates fractal_colourise_kfp_impl / write_kfp_pixel for the scalar-field
// ABI (renderer.cpp:16314-16545, 6696-7289): reflected stencil samples
// (:5427-5496), the Differences 0-7 gradient (:5498-5578), the ColorMethod
// 0-11 transfer with IterDiv and ColorOffset, the cyclic LUT with linear
// interpolation, MultiColor HSV waves (:5580-5630), slopes (3D relief) and
// Kalles' ordered dither (:5246-5258, 5314-5332).
//
// Algorithmically HBM-bound (4 B of field in, 3 B of RGB out per pixel; the
// stencil re-reads and the palette hit L1); in practice issue-bound.  Precision: stencil differences are
// formed in FP32, which is exact for neighbouring values within a factor of
// two (Sterbenz); the transcendentals (log, sqrt, pow, atan, sin) run in
// FP32; the palette position (division by IterDiv, offset, modulo, floor) is
// formed in FP64 so the LUT index follows the reference.  Output agrees with
// the reference to +-1 LSB per channel.
#include <cuda_runtime.h>

#include <cmath>
#include <limits>

#include <cstdint>

#include "device.h"

namespace fgb {

namespace {

constexpr float kPiF = 3.14159265358979323846f;

struct KfpDevice {
    int width, height, max_iter;
    float field_bias;
    double field_bias_d;
    float smooth_offset;
    double smooth_offset_d;
    int color_method, differences, smooth, flat, inverse_transition;
    int needs_difference, needs_slopes;
    double iter_div, color_offset;
    double transfer_min, transfer_max;
    int multi_color, blend_multi_color, multi_count;
    float slope_cos, slope_sin, slope_power, slope_ratio;
    int interior[3];
    int lut_size;
    // Double-float (hi + lo FP32 pair) copies of the double constants of the
    // palette position (set on the host).
    float shift_hi, shift_lo;          // field_bias + smooth_offset
    float inv_div_hi, inv_div_lo;      // 1 / iter_div
    float offset_hi, offset_lo;        // color_offset
    float tmin_hi, tmin_lo;            // transfer_min (ColorMethod 4)
    float tscale_hi, tscale_lo;        // 1024 / max(transfer_max - transfer_min, 1e-12)
    int has_div;                       // iter_div != 1
    // FP32 shortcuts of exact double tests (set on the host):
    float sample_hi;     // smallest float >= max_iter - field_bias
    int sample_fast;     // field_bias >= 0 and smooth_offset >= 0
    double inv_iter_div; // 1 / iter_div
    int lut_shift;       // log2(lut_size) when a power of two, else -1
    int spatial_width;   // the output width the gradient and slopes scale by
};

// A stencil sample is kept as its raw field value sv with the sample equal to
// sv + field_bias + smooth_offset (kfp_colour_sample, renderer.cpp:5427-5458).
// The bias and offset are common to every sample, so stencil differences are
// differences of raw float field values, which FP32 forms exactly for
// neighbouring values; only the special cases (interior, glitch, clamps) are
// shifted into the same frame.
__device__ __forceinline__ float sample(const float* __restrict__ field, const KfpDevice& k, int x, int y) {
    const float v = __ldg(field + static_cast<long long>(y) * k.width + x);
    // Common case without FP64: a finite value in [0, max_iter - bias) with a
    // non-negative bias and offset passes through unchanged (v >= 0 makes both
    // shifted values non-negative; v < sample_hi is the double comparison
    // against max_iter - bias, exactly, for a float v).
    if (k.sample_fast && v >= 0.0f && v < k.sample_hi) return v;
    const double shift = k.field_bias_d + k.smooth_offset_d;
    if (!isfinite(v)) return static_cast<float>(fmax(0.0, k.smooth_offset_d) - shift);
    const double biased = static_cast<double>(v) + k.field_bias_d;
    if (static_cast<double>(v) >= static_cast<double>(k.max_iter) - k.field_bias_d) {
        return static_cast<float>(static_cast<double>(k.max_iter) + 1.0 - shift);
    }
    if (biased < 0.0 || biased + k.smooth_offset_d < 0.0) {
        const double s = fmax(0.0, fmin(fmax(biased, 0.0), static_cast<double>(k.max_iter)) + k.smooth_offset_d);
        return static_cast<float>(s - shift);
    }
    return v;
}

// x / d for a constant divisor d with r = RN(1 / d), by Markstein's
// correction of the rounded product (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): q0 = RN(x r), e = x - q0 d (exact by FMA), q = RN(q0 +
// e r).  Three FP32 operations instead of a division; for the divisors the
// colour pass uses, q equals the IEEE quotient x / d for every x with |x| in
// [2^-100, 2^100], which fractal_gb300_check_division verifies for all 2^32
// inputs; zero, tiny, huge and non-finite x take the division.
__device__ __forceinline__ float div_const(float x, float d, float r) {
    const float ax = fabsf(x);
    if (!(ax >= 0x1p-100f && ax <= 0x1p100f)) return x / d;
    const float q0 = __fmul_rn(x, r);
    const float e = __fmaf_rn(-q0, d, x);
    return __fmaf_rn(e, r, q0);
}

constexpr float kHalfPiF = kPiF / 2.0f;
#define FGB_DIV(x, d) div_const((x), (d), 1.0f / (d))

// kfp_reflected_sample: out-of-frame neighbours mirror through the centre.
__device__ __forceinline__ float reflected(const float* __restrict__ field, const KfpDevice& k, int x, int y,
                                           int dx, int dy, float centre) {
    const int sx = x + dx, sy = y + dy;
    if (sx >= 0 && sx < k.width && sy >= 0 && sy < k.height) return sample(field, k, sx, sy);
    const int ox = x - dx, oy = y - dy;
    if (ox >= 0 && ox < k.width && oy >= 0 && oy < k.height) return 2.0f * centre - sample(field, k, ox, oy);
    return centre;
}

// kfp_difference_magnitude (renderer.cpp:5498-5578) written on differences
// from the centre so every term is an exact FP32 difference.
__device__ float difference_magnitude(int differences, float c, float l, float r, float u, float d, float tl,
                                      float tr, float bl, float br) {
    const float s = 2.8284271247461903f;
    const float dl = l - c, dr = r - c, du = u - c, dd = d - c;
    const float dtl = tl - c, dtr = tr - c, dbl = bl - c, dbr = br - c;
    switch (differences) {
        case 0:
            return fabsf(dl) * 1.414f + fabsf(du) * 1.414f + fabsf(dtl) + fabsf(dbl);
        case 1: {
            const float q = dl * dl + dr * dr + du * du + dd * dd + (dtl * dtl + dbr * dbr) * 0.5f
                + (dbl * dbl + dtr * dtr) * 0.5f;
            return sqrtf(fmaxf(0.0f, q * 0.25f)) * s;
        }
        case 2: {
            const float a = r - l, b = d - u, e = br - tl, f = tr - bl;
            const float q = a * a * 0.25f + b * b * 0.25f + e * e * 0.125f + f * f * 0.125f;
            return sqrtf(fmaxf(0.0f, q * 0.5f)) * s;
        }
        case 3: {
            const float a = l - u;
            const float q = dtl * dtl * 0.5f + a * a * 0.5f;
            return sqrtf(fmaxf(0.0f, q)) * s;
        }
        case 4: {
            const float dx = ((u - tl) + (c - l)) * 0.5f;
            const float dy = ((l - tl) + (c - u)) * 0.5f;
            return sqrtf(dx * dx + dy * dy) * s;
        }
        case 5: {
            const float dx = FGB_DIV((r - l) + (tr - tl) + (br - bl), 6.0f);
            const float dy = FGB_DIV((d - u) + (bl - tl) + (br - tr), 6.0f);
            return sqrtf(dx * dx + dy * dy) * s;
        }
        case 6: {
            const float lap = dtl + 4.0f * du + dtr + 4.0f * dl + 4.0f * dr + dbl + 4.0f * dd + dbr;
            return sqrtf(fabsf(FGB_DIV(lap, 6.0f) * 1.4426950408889634f)) * s;
        }
        default:
            return 0.0f;  // analytic DE needs planes
    }
}

__device__ void hsv_to_rgb(float hue, float sat, float val, float& r, float& g, float& b) {
    const float scaled = hue * 6.0f;
    const int sector = static_cast<int>(floorf(scaled));
    float f = scaled - static_cast<float>(sector);
    if ((sector & 1) == 0) f = 1.0f - f;
    const float m = val * (1.0f - sat);
    const float n = val * (1.0f - sat * f);
    r = g = b = 0.0f;
    switch (sector) {
        case 0: case 6: r = m; g = n; b = val; break;
        case 1: r = m; g = val; b = n; break;
        case 2: r = n; g = val; b = m; break;
        case 3: r = val; g = n; b = m; break;
        case 4: r = val; g = m; b = n; break;
        case 5: r = n; g = m; b = val; break;
        default: break;
    }
}

__device__ __forceinline__ unsigned char dither_byte(float value, int x, int y, int channel) {
    if (!isfinite(value)) value = 0.0f;
    const unsigned int coordinate = (static_cast<unsigned int>(x) + static_cast<unsigned int>(channel) * 67u
                                     + static_cast<unsigned int>(y) * 236u) * 119u;
    const float mask = static_cast<float>(coordinate & 255u) / 256.0f;
    const int q = static_cast<int>(floorf(255.0f * value + mask));
    return static_cast<unsigned char>(q < 0 ? 0 : (q > 255 ? 255 : q));
}

// Double-float arithmetic (unevaluated sum hi + lo of two floats, about 48
// significant bits): Knuth's two-sum and the FMA two-product, after Dekker's
// double-length arithmetic.  The palette position runs in it on the FP32
// pipe instead of in FP64 (1/64 of the FP32 rate on this GPU); it is within
// ~2^-44 relative of the double value, far inside the +-1 LSB colour budget.
struct Df {
    float hi, lo;
};

__device__ __forceinline__ Df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return Df{s, err};
}

__device__ __forceinline__ Df df_norm(float hi, float lo) {
    const float s = __fadd_rn(hi, lo);
    return Df{s, __fsub_rn(lo, __fsub_rn(s, hi))};
}

__device__ __forceinline__ Df df_add(Df x, Df y) {
    const Df s = two_sum(x.hi, y.hi);
    return df_norm(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ Df df_neg(Df x) { return Df{-x.hi, -x.lo}; }

__device__ __forceinline__ Df df_mul(Df x, Df y) {
    const float p = __fmul_rn(x.hi, y.hi);
    const float e = fmaf(x.hi, y.hi, -p);
    return df_norm(p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e)));
}

__device__ __forceinline__ Df df_scale(Df x, float power_of_two) { return Df{x.hi * power_of_two, x.lo * power_of_two}; }

// floor(hi + lo): a non-integral hi is at least an ulp from the next
// integer, farther than |lo|; an integral hi adds floor(lo).
__device__ __forceinline__ Df df_floor(Df x) {
    const float f = floorf(x.hi);
    if (f != x.hi) return Df{f, 0.0f};
    return two_sum(f, floorf(x.lo));
}

__device__ __forceinline__ float df_value(Df x) { return __fadd_rn(x.hi, x.lo); }

__device__ __forceinline__ bool df_negative(Df x) { return x.hi < 0.0f || (x.hi == 0.0f && x.lo < 0.0f); }

// ---- plane path (fractal_colourise_kfp_planes, renderer.cpp:16314-16728)

// kfp_plane_smooth_part (renderer.cpp:5775-5842): the fractional part of a
// Kalles orbit sample from |z|^2 at escape (test1), the previous |z|^2
// (test2) and the bailout, by SmoothMethod 0 (log-log) or 1 (norm roots).
__device__ double plane_smooth_part(const KfpPlanesLaunch& pl, long long i) {
    if (pl.test1 == nullptr) return 0.0;
    const double test1 = pl.test1[i];
    if (!isfinite(test1) || test1 <= 0.0) return 0.0;
    double radius = pl.smooth_bailout_radius;
    if (!pl.has_constant_bailout) {
        const double b = pl.bailout[i];
        radius = isfinite(b) && b > 1.0 ? b : pl.smooth_bailout_radius;
    }
    double smooth = 0.0;
    if (pl.smooth_method == 0) {
        if (radius > 1.0 && isfinite(pl.power) && pl.power > 1.0) {
            const double numerator = log(sqrt(test1));
            const double denominator = pl.has_smooth_bailout_log ? pl.smooth_bailout_log : log(radius);
            const double power_log = pl.has_smooth_power_log ? pl.smooth_power_log : log(pl.power);
            if (isfinite(numerator) && numerator > 0.0 && isfinite(denominator) && denominator != 0.0
                && isfinite(power_log) && power_log != 0.0) {
                smooth = 1.0 - log(numerator / denominator) / power_log;
            }
        }
    } else if (pl.smooth_method == 1 && pl.test2 != nullptr) {
        const double test2 = pl.test2[i];
        if (isfinite(test2) && test2 >= 0.0 && pl.has_smooth_norm_exponent) {
            const double root1 = pow(test1, pl.smooth_norm_exponent);
            const double root2 = pow(test2, pl.smooth_norm_exponent);
            const double denominator = root1 - root2;
            if (isfinite(root1) && isfinite(root2) && isfinite(radius) && denominator != 0.0) {
                smooth = 1.0 - (root1 - radius) / denominator;
            }
        }
    }
    return isfinite(smooth) ? smooth : 0.0;
}

// ln x of a positive finite double in FP32 from its exponent field and the
// top 23 bits of its mantissa (relative error ~2^-23 in the mantissa), so
// that every double magnitude is in range and no FP64 instruction issues.
__device__ __forceinline__ float ln_positive(long long bits) {
    const int exponent = static_cast<int>((bits >> 52) & 0x7ff);
    if (exponent == 0) return static_cast<float>(log(__longlong_as_double(bits)));  // subnormal
    const float mantissa = __int_as_float(0x3f800000 | static_cast<int>((bits >> 29) & 0x7fffff));
    return (static_cast<float>(exponent - 1023) + log2f(mantissa)) * 0.693147180559945309f;
}

// v < 0 for a double, on its bit pattern (false for -0 and NaN).
__device__ __forceinline__ bool negative_bits(double v) {
    const long long b = __double_as_longlong(v);
    return b < 0 && b != static_cast<long long>(0x8000000000000000ull)
        && (b & 0x7fffffffffffffffll) <= 0x7ff0000000000000ll;
}

// SmoothMethod 0 of kfp_plane_smooth_part in FP32: 1 - ln(ln|z| / ln R) /
// ln p with ln|z| = ln(test1) / 2.  The reference's validity tests reduce to
// test1 > 1 (finite), R > 1 (finite) and p > 1 (finite), decided on bit
// patterns.  The term is below 1, so its FP32 error (~1e-7) moves the
// palette position far less than the +-1 LSB colour budget allows.
__device__ __forceinline__ float plane_smooth_fast(const KfpPlanesLaunch& pl, long long i) {
    const long long t = __double_as_longlong(pl.test1[i]);
    const long long one = 0x3ff0000000000000ll;
    if (t <= one || ((t >> 52) & 0x7ff) == 0x7ff || !pl.smooth_power_ok) return 0.0f;  // test1 <= 1, NaN / inf
    float radius_log = pl.smooth_radius_log_f;
    bool radius_ok = pl.smooth_radius_ok;
    if (!pl.has_constant_bailout) {
        const long long b = __double_as_longlong(pl.bailout[i]);
        if (b > one && ((b >> 52) & 0x7ff) != 0x7ff) {
            radius_log = ln_positive(b);
            radius_ok = true;
        }
    }
    if (!radius_ok) return 0.0f;
    const float numerator = 0.5f * ln_positive(t);
    const float smooth = 1.0f - logf(numerator / radius_log) / pl.smooth_power_log_f;
    return isfinite(smooth) ? smooth : 0.0f;
}

// The colour sample of every pixel from its planes, as a double-float, with
// flags (bit 0 interior, bit 1 hidden glitch): kfp_plane_orbit_sample
// (renderer.cpp:5844-5866) from orbit_iteration + the smoothing part, else
// stored iteration + 1 - transition (kfp_plane_colour_sample, 5868-5911).
__global__ void __launch_bounds__(256, 6) kfp_plane_samples_kernel(const KfpPlanesLaunch pl, int max_iter, long long pixels, float2* samples,
                                         unsigned char* flags) {
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        double value;
        bool inside;
        if (pl.orbit_iteration != nullptr) {
            const long long raw = pl.orbit_iteration[i] > 0 ? pl.orbit_iteration[i] : 0;
            if (raw >= max_iter) {
                value = static_cast<double>(max_iter) + 1.0;
                inside = true;
            } else if (pl.smooth_method == 0) {
                // raw < max_iter <= 10^7 < 2^24 is an exact float, so raw +
                // smooth is an exact double-float, compared with the cap
                // exactly.
                const float smooth = pl.test1 != nullptr ? plane_smooth_fast(pl, i) : 0.0f;
                const Df combined = two_sum(static_cast<float>(static_cast<int>(raw)), smooth);
                const float cap = static_cast<float>(max_iter);
                inside = combined.hi > cap || (combined.hi == cap && combined.lo >= 0.0f);
                samples[i] = inside ? make_float2(cap + 1.0f, 0.0f) : make_float2(combined.hi, combined.lo);
                const bool hidden = pl.transition != nullptr && !pl.show_glitches && negative_bits(pl.transition[i]);
                flags[i] = static_cast<unsigned char>((inside ? 1 : 0) | (hidden ? 2 : 0));
                continue;
            } else {
                const double combined = static_cast<double>(raw) + plane_smooth_part(pl, i);
                inside = combined >= static_cast<double>(max_iter);
                value = inside ? static_cast<double>(max_iter) + 1.0 : combined;
            }
        } else {
            const long long stored = pl.iteration[i];
            inside = stored >= max_iter;
            if (inside) {
                value = static_cast<double>(max_iter) + 1.0;
            } else {
                const double transition = pl.transition != nullptr ? pl.transition[i] : 1.0;
                value = static_cast<double>(stored > 0 ? stored : 0) + 1.0 - (isfinite(transition) ? transition : 1.0);
            }
        }
        const float hi = static_cast<float>(value);
        samples[i] = make_float2(hi, static_cast<float>(value - static_cast<double>(hi)));
        const bool hidden = pl.transition != nullptr && !pl.show_glitches && negative_bits(pl.transition[i]);
        flags[i] = static_cast<unsigned char>((inside ? 1 : 0) | (hidden ? 2 : 0));
    }
}

// ColorMethod 4 bounds over plane samples (kfp_transfer_bounds_planes,
// renderer.cpp:7335-7393): floor(sample) of escaped pixels below max_iter - 1.
__global__ void kfp_plane_bounds_kernel(const float2* __restrict__ samples, const unsigned char* __restrict__ flags,
                                        long long pixels, int max_iter, unsigned long long* bounds);

// write_kfp_pixel (renderer.cpp:6696-7289) for source pixel (x, y) of a
// k.width x k.height field, dithered at output position (dither_x,
// dither_y); `lut` is the palette in global memory (3 KB at the usual 1024
// entries: it stays in L1, which served it faster than a per-block copy into
// shared memory).
template <bool Planes, bool Kalles = false>
__device__ __forceinline__ void kfp_pixel(const float* __restrict__ field, const KfpDevice& k,
                                          const unsigned char* lut, const double* __restrict__ mc_period,
                                          const int* __restrict__ mc_type, const KfpPlanesLaunch& pl,
                                          const float2* __restrict__ psamples, const unsigned char* __restrict__ pflags,
                                          int x, int y, int dither_x, int dither_y, unsigned char* out) {
    const long long index = static_cast<long long>(y) * k.width + x;
    // The Kalles default family (ColorMethod 7, Differences 3, smooth
    // palette, slopes, a power-of-two palette, no flat, inverse or
    // multi-colour transfer) is a compile-time variant: its option switches
    // and dead branches fold away.
    const int color_method = Kalles ? 7 : k.color_method;
    const int differences = Kalles ? 3 : k.differences;
    const int smooth = Kalles ? 1 : k.smooth;
    const int flat = Kalles ? 0 : k.flat;
    const int inverse_transition = Kalles ? 0 : k.inverse_transition;
    const int multi_color = Kalles ? 0 : k.multi_color;
    const int needs_difference = Kalles ? 1 : k.needs_difference;
    const int needs_slopes = Kalles ? 1 : k.needs_slopes;
    const bool lut_pow2 = Kalles || k.lut_shift >= 0;
    // Plane samples (when the planes carry iterations) are double-float
    // values; the stencil then works on their differences from the centre,
    // so `centre` is 0 and each neighbour is its difference.
    const bool plane_samples = Planes && pl.has_iteration;
    // With a texture, interior pixels run the whole pass: the interior colour
    // replaces the palette just before the texture merge (renderer.cpp:
    // 6790-6796, 7181-7189).
    const bool texture = Planes && pl.texture_active;
    bool inside;
    if (plane_samples) {
        const unsigned char f = pflags[index];
        if (f & 2) {  // a hidden glitch pixel: black (renderer.cpp:6733-6743)
            out[0] = 0;
            out[1] = 0;
            out[2] = 0;
            return;
        }
        inside = (f & 1) != 0;
    } else {
        if constexpr (Planes) {
            if (pl.transition != nullptr && pl.transition[index] < 0.0 && !pl.show_glitches) {
                out[0] = 0;
                out[1] = 0;
                out[2] = 0;
                return;
            }
        }
        const float raw = __ldg(field + index);
        inside = isfinite(raw) && raw >= k.sample_hi;  // the double test raw >= max_iter - bias, exactly
    }
    if (inside && !texture) {
        out[0] = static_cast<unsigned char>(k.interior[0]);
        out[1] = static_cast<unsigned char>(k.interior[1]);
        out[2] = static_cast<unsigned char>(k.interior[2]);
        return;
    }
    Df centre_value;
    float centre;
    if (plane_samples) {
        const float2 c = psamples[index];
        centre_value = Df{c.x, c.y};
        centre = 0.0f;
    } else {
        centre = sample(field, k, x, y);
        centre_value = df_add(Df{centre, 0.0f}, Df{k.shift_hi, k.shift_lo});
    }
    const Df colour_iter_df = flat ? df_floor(centre_value) : centre_value;
    const float colour_iter = df_value(colour_iter_df);
    auto plane_difference_df = [&](int dx, int dy) -> Df {
        const int sx = x + dx, sy = y + dy;
        if (sx >= 0 && sx < k.width && sy >= 0 && sy < k.height) {
            const float2 v = psamples[static_cast<long long>(sy) * k.width + sx];
            return df_add(Df{v.x, v.y}, df_neg(centre_value));
        }
        const int ox = x - dx, oy = y - dy;
        if (ox >= 0 && ox < k.width && oy >= 0 && oy < k.height) {
            const float2 v = psamples[static_cast<long long>(oy) * k.width + ox];
            return df_add(centre_value, df_neg(Df{v.x, v.y}));
        }
        return Df{0.0f, 0.0f};
    };
    auto plane_difference = [&](int dx, int dy) -> float { return df_value(plane_difference_df(dx, dy)); };
    auto neighbour = [&](int dx, int dy) -> float {
        if constexpr (Planes) {
            if (plane_samples) return plane_difference(dx, dy);
        }
        return reflected(field, k, x, y, dx, dy, centre);
    };
    float l = centre, r = centre, u = centre, d = centre, tl = centre, tr = centre, bl = centre, br = centre;
    if (needs_difference || needs_slopes || texture) {
        l = neighbour(-1, 0);
        u = neighbour(0, -1);
        if (needs_difference) {
            switch (differences) {
                case 0:
                    tl = neighbour(-1, -1);
                    bl = neighbour(-1, 1);
                    break;
                case 1: case 2: case 5: case 6:
                    r = neighbour(1, 0);
                    d = neighbour(0, 1);
                    tl = neighbour(-1, -1);
                    tr = neighbour(1, -1);
                    bl = neighbour(-1, 1);
                    br = neighbour(1, 1);
                    break;
                case 3: case 4:
                    tl = neighbour(-1, -1);
                    break;
                default:
                    r = neighbour(1, 0);
                    d = neighbour(0, 1);
                    break;
            }
        }
        if (needs_slopes || texture) {
            if (x == 0) r = neighbour(1, 0);
            if (y == 0) d = neighbour(0, 1);
        }
    }
    float gradient = 0.0f;
    float analytic_x = 0.0f, analytic_y = 0.0f;
    bool analytic = false;
    if constexpr (Planes) {
        // Differences 7 with DE planes: Kalles' float reciprocal norm of the
        // analytic derivative (renderer.cpp:6942-6962).
        if ((needs_difference || needs_slopes) && pl.analytic) {
            analytic = true;
            const double ex = pl.de_x[index], ey = pl.de_y[index];
            const float de_x = static_cast<float>(isfinite(ex) ? ex : 0.0);
            const float de_y = static_cast<float>(isfinite(ey) ? ey : 0.0);
            const float denominator = de_x * de_x + de_y * de_y;
            if (denominator > 0.0f && isfinite(denominator)) {
                gradient = 1.0f / sqrtf(denominator);
                analytic_x = de_x / denominator;
                analytic_y = -de_y / denominator;
            }
        }
    }
    if (!analytic && needs_difference) gradient = difference_magnitude(differences, centre, l, r, u, d, tl, tr, bl, br);
    float distance = isnan(gradient) ? 0.0f : FGB_DIV(gradient * static_cast<float>(k.spatial_width), 640.0f);
    if (distance < 0.0f) distance = 0.0f;
    Df transfer_df = colour_iter_df;  // kept in double-float for methods 0, 4 and 6's iteration branch
    bool exact_transfer = color_method == 0 || color_method == 4;
    float transfer = colour_iter;
    switch (color_method) {
        case 1: transfer = sqrtf(fmaxf(0.0f, colour_iter)); break;
        case 2: transfer = powf(fmaxf(0.0f, colour_iter), 1.0f / 3.0f); break;
        case 3: transfer = logf(fmaxf(1.0f, colour_iter)); break;
        case 4:
            transfer_df = df_mul(df_add(colour_iter_df, df_neg(Df{k.tmin_hi, k.tmin_lo})),
                                 Df{k.tscale_hi, k.tscale_lo});
            transfer = df_value(transfer_df);
            break;
        case 5: transfer = fminf(distance, 1024.0f); break;
        case 6: {
            const float dt = fminf(sqrtf(fmaxf(0.0f, distance)), 1024.0f);
            if (static_cast<double>(dt) > k.iter_div) {
                transfer_df = centre_value;
                transfer = df_value(centre_value);
                exact_transfer = true;
            } else {
                transfer = dt;
            }
            break;
        }
        case 7: transfer = logf(fmaxf(1.0f, distance + 1.0f)); break;
        case 8: transfer = sqrtf(fmaxf(0.0f, distance)); break;
        case 9: transfer = logf(1.0f + logf(1.0f + fmaxf(0.0f, colour_iter))); break;
        case 10: transfer = atanf(colour_iter); break;
        case 11: transfer = sqrtf(sqrtf(fmaxf(0.0f, colour_iter))); break;
        default: break;
    }
    Df palette_value = exact_transfer ? transfer_df : Df{transfer, 0.0f};
    if (isnan(palette_value.hi) || isnan(palette_value.lo) || df_negative(palette_value)) palette_value = Df{0.0f, 0.0f};
    if ((color_method == 5 || color_method == 7 || color_method == 8) && palette_value.hi > 1024.0f) {
        palette_value = Df{1024.0f, 0.0f};
    }
    if (k.has_div) palette_value = df_mul(palette_value, Df{k.inv_div_hi, k.inv_div_lo});
    const Df base = df_add(palette_value, Df{k.offset_hi, k.offset_lo});
    // The phase colour shift of the ordinary palette (renderer.cpp:7045-7048).
    Df palette_base = base;
    if constexpr (Planes) {
        if (pl.phase != nullptr) {
            const double ph = pl.phase[index];
            const double shift = pl.phase_scale * (isfinite(ph) ? ph : 0.0);
            const float hi = static_cast<float>(shift);
            palette_base = df_add(base, Df{hi, static_cast<float>(shift - static_cast<double>(hi))});
        }
    }
    float red, green, blue;
    auto palette_rgb = [&](Df input, float& o_r, float& o_g, float& o_b) {
        Df position;
        if (lut_pow2) {
            // input - size * floor(input / size): power-of-two scalings are
            // exact, so this is the cyclic position in [0, size).
            const float size = static_cast<float>(k.lut_size);
            const Df turns = df_floor(df_scale(input, 1.0f / size));
            position = df_add(input, df_neg(df_scale(turns, size)));
        } else {
            const double size = static_cast<double>(k.lut_size);
            double p = fmod(static_cast<double>(input.hi) + static_cast<double>(input.lo), size);
            if (p < 0.0) p += size;
            const float hi = static_cast<float>(p);
            position = Df{hi, static_cast<float>(p - static_cast<double>(hi))};
        }
        const Df lower_position = df_floor(position);
        int lower = static_cast<int>(lower_position.hi) + static_cast<int>(lower_position.lo);
        lower = lower < 0 ? 0 : (lower > k.lut_size - 1 ? k.lut_size - 1 : lower);
        if (smooth) {
            float f = df_value(df_add(position, df_neg(lower_position)));
            if (inverse_transition) f = 1.0f - f;
            const int upper = lower + 1 < k.lut_size ? lower + 1 : 0;  // (lower + 1) mod size, lower in [0, size)
            const float g = 1.0f - f;
            o_r = FGB_DIV(static_cast<float>(lut[lower * 3]) * g + static_cast<float>(lut[upper * 3]) * f, 255.0f);
            o_g = FGB_DIV(static_cast<float>(lut[lower * 3 + 1]) * g + static_cast<float>(lut[upper * 3 + 1]) * f,
                          255.0f);
            o_b = FGB_DIV(static_cast<float>(lut[lower * 3 + 2]) * g + static_cast<float>(lut[upper * 3 + 2]) * f,
                          255.0f);
        } else {
            o_r = FGB_DIV(static_cast<float>(lut[lower * 3]), 255.0f);
            o_g = FGB_DIV(static_cast<float>(lut[lower * 3 + 1]), 255.0f);
            o_b = FGB_DIV(static_cast<float>(lut[lower * 3 + 2]), 255.0f);
        }
    };
    if (multi_color) {
        const double wave_input = static_cast<double>(df_value(smooth ? base : df_floor(base)));
        float hs = 0.0f, ss = 0.0f, vs = 0.0f;
        int hc = 0, sc = 0, vc = 0;
        for (int i = 0; i < k.multi_count; ++i) {
            const double period = __ldg(mc_period + i);
            const float wave = period < 0.0 ? static_cast<float>(-period / 100.0)
                                            : 0.5f + 0.5f * sinf(static_cast<float>(3.14159265358979323846 * wave_input / period));
            const int type = __ldg(mc_type + i);
            if (type == 0) { hs += wave; ++hc; }
            else if (type == 1) { ss += wave; ++sc; }
            else { vs += wave; ++vc; }
        }
        float mr, mg, mb;
        hsv_to_rgb(hc ? hs / hc : 0.0f, sc ? ss / sc : 0.0f, vc ? vs / vc : 0.0f, mr, mg, mb);
        if (k.blend_multi_color) {
            palette_rgb(palette_base, red, green, blue);
            red = (red + mr) * 0.5f;
            green = (green + mg) * 0.5f;
            blue = (blue + mb) * 0.5f;
        } else {
            red = mr;
            green = mg;
            blue = mb;
        }
    } else {
        palette_rgb(palette_base, red, green, blue);
    }
    if constexpr (Planes) {
        if (texture) {
            if (inside) {
                red = static_cast<float>(k.interior[0]) / 255.0f;
                green = static_cast<float>(k.interior[1]) / 255.0f;
                blue = static_cast<float>(k.interior[2]) / 255.0f;
            }
            // SetTexture (renderer.cpp:7191-7248): the texel is displaced by
            // a warp of the one-sided stencil differences, in FP64 because
            // the texel index is a floor of it.
            auto difference = [&](int dx, int dy) -> double {  // in-frame neighbour minus centre
                if (plane_samples) {
                    const Df v = plane_difference_df(dx, dy);
                    return static_cast<double>(v.hi) + static_cast<double>(v.lo);
                }
                return static_cast<double>(sample(field, k, x + dx, y + dy)) - static_cast<double>(centre);
            };
            const double tdx = x > 0 ? difference(-1, 0) : (x + 1 < k.width ? -difference(1, 0) : 0.0);
            const double tdy = y > 0 ? difference(0, -1) : (y + 1 < k.height ? -difference(0, 1) : 0.0);
            auto warp = [&](double delta) -> double {
                const double powered = pow(1.0 + delta, pl.texture_power);
                const bool forward = powered > 1.0;
                const double selected = forward ? powered : 1.0 / powered;
                const double quarter = 3.14159265358979323846 / 4.0;
                const double mapped = !isnan(selected)
                    ? (atan(selected) - quarter) / quarter * (pl.texture_ratio / 100.0) : 0.0;
                return isfinite(mapped) ? (forward ? pl.texture_power * mapped : -pl.texture_power * mapped) : 0.0;
            };
            auto texel = [](double v, int limit) -> int {  // kfp_texture_index (renderer.cpp:5971-5976)
                if (limit <= 0 || !isfinite(v) || v <= 0.0) return 0;
                if (v >= static_cast<double>(limit - 1)) return limit - 1;
                return static_cast<int>(v);
            };
            const int sx = texel(static_cast<double>(static_cast<long long>(x) + pl.image_offset) + warp(tdx),
                                 pl.texture_width);
            const int sy = texel(static_cast<double>(static_cast<long long>(y) + pl.image_offset) + warp(tdy),
                                 pl.texture_height);
            const unsigned char* t = pl.texture + static_cast<long long>(pl.texture_height - 1 - sy) * pl.texture_stride
                + static_cast<long long>(sx) * 3;
            const double merge = pl.texture_merge;
            red = static_cast<float>(static_cast<double>(red) * (1.0 - merge) + merge * static_cast<double>(t[0]) / 255.0);
            green = static_cast<float>(static_cast<double>(green) * (1.0 - merge)
                                       + merge * static_cast<double>(t[1]) / 255.0);
            blue = static_cast<float>(static_cast<double>(blue) * (1.0 - merge)
                                      + merge * static_cast<double>(t[2]) / 255.0);
        }
    }
    if (needs_slopes) {
        const float horizontal = analytic ? analytic_x : (x > 0 ? l - centre : centre - r);
        const float vertical = analytic ? analytic_y : (y == 0 ? centre - d : u - centre);
        const float projected = FGB_DIV((horizontal * k.slope_cos + vertical * k.slope_sin) * k.slope_power
                                            * static_cast<float>(k.spatial_width), 640.0f);
        const float strength = FGB_DIV(FGB_DIV(atanf(fabsf(projected)), kHalfPiF) * k.slope_ratio, 100.0f);
        if (projected >= 0.0f) {
            red *= 1.0f - strength;
            green *= 1.0f - strength;
            blue *= 1.0f - strength;
        } else {
            red = red * (1.0f - strength) + strength;
            green = green * (1.0f - strength) + strength;
            blue = blue * (1.0f - strength) + strength;
        }
    }
    out[0] = dither_byte(red, dither_x, dither_y, 0);
    out[1] = dither_byte(green, dither_x, dither_y, 1);
    out[2] = dither_byte(blue, dither_x, dither_y, 2);
}

template <bool Planes, bool Kalles>
__global__ void __launch_bounds__(256, 6) kfp_kernel(const float* __restrict__ field, unsigned char* __restrict__ rgb,
                                                  const KfpDevice k, const unsigned char* __restrict__ lut_global,
                                                  const double* __restrict__ mc_period, const int* __restrict__ mc_type,
                                                  const KfpPlanesLaunch pl, const float2* __restrict__ psamples,
                                                  const unsigned char* __restrict__ pflags) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= k.width || y >= k.height) return;
    kfp_pixel<Planes, Kalles>(field, k, lut_global, mc_period, mc_type, pl, psamples, pflags, x, y, x, y,
                      rgb + 3 * (static_cast<long long>(y) * k.width + x));
}

// The child tile's smoothstep ramp at distance `i` into a `size`-wide axis
// (renderer.cpp:16895-16910); no contraction, as in the reference.
__device__ __forceinline__ float tile_ramp(int i, int size, int feather) {
    const int edge = i < size - 1 - i ? i : size - 1 - i;
    float linear = __fdiv_rn(static_cast<float>(edge), static_cast<float>(feather));
    linear = linear < 1.0f ? linear : 1.0f;
    return __fmul_rn(__fmul_rn(linear, linear), __fsub_rn(3.0f, __fmul_rn(2.0f, linear)));
}

// fractal_atlas_colourise_kfp's generic per-pixel body (renderer.cpp:
// 17097-17265): outside the child rectangle the parent tile; inside, an
// interior child pixel of the owned region, the child or parent by
// interior test without a feather band, else both tiles blended in FP64
// and rounded half-even (rounded_colour_byte).
__device__ __forceinline__ void kfp_atlas_pixel(const KfpAtlasLaunch& at, unsigned char* __restrict__ rgb,
                                                const KfpDevice& kp, const KfpDevice& kc, const unsigned char* lut,
                                                const double* __restrict__ mc_period,
                                                const int* __restrict__ mc_type, int x, int y) {
    unsigned char* dst = rgb + 3 * (static_cast<long long>(y) * kp.width + x);
    const KfpPlanesLaunch none{};
    const int cx = x - at.child_left, cy = y - at.child_top;
    const bool in_child = at.child != nullptr && cx >= 0 && cx < at.child_width && cy >= 0 && cy < at.child_height;
    if (!in_child) {
        kfp_pixel<false>(at.parent, kp, lut, mc_period, mc_type, none, nullptr, nullptr, x, y, x, y, dst);
        return;
    }
    const float child_raw = __ldg(at.child + static_cast<long long>(cy) * at.child_width + cx);
    const bool child_inside = isfinite(child_raw) && child_raw >= kc.sample_hi;
    float alpha = 1.0f;
    if (at.feather >= 2) {
        const float ax = tile_ramp(cx, at.child_width, at.feather), ay = tile_ramp(cy, at.child_height, at.feather);
        alpha = ay < ax ? ay : ax;
    }
    // Alpha exactly 1 outside the band: the reference's blend p * 0 + c * 1
    // of two finite bytes is c, so only the child tile is coloured.
    if ((child_inside && alpha >= 0.999999f) || (at.feather >= 2 && alpha == 1.0f)) {
        kfp_pixel<false>(at.child, kc, lut, mc_period, mc_type, none, nullptr, nullptr, cx, cy, x, y, dst);
        return;
    }
    if (at.feather < 2) {
        const float parent_raw = __ldg(at.parent + static_cast<long long>(y) * kp.width + x);
        if (!(isfinite(parent_raw) && parent_raw >= kp.sample_hi)) {
            kfp_pixel<false>(at.parent, kp, lut, mc_period, mc_type, none, nullptr, nullptr, x, y, x, y, dst);
        } else {
            kfp_pixel<false>(at.child, kc, lut, mc_period, mc_type, none, nullptr, nullptr, cx, cy, x, y, dst);
        }
        return;
    }
    unsigned char p[3], c[3];
    kfp_pixel<false>(at.parent, kp, lut, mc_period, mc_type, none, nullptr, nullptr, x, y, x, y, p);
    kfp_pixel<false>(at.child, kc, lut, mc_period, mc_type, none, nullptr, nullptr, cx, cy, x, y, c);
    const double a = static_cast<double>(alpha);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        double v = __dadd_rn(__dmul_rn(static_cast<double>(p[ch]), __dsub_rn(1.0, a)),
                             __dmul_rn(static_cast<double>(c[ch]), a));
        v = v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v);
        dst[ch] = static_cast<unsigned char>(__double2int_rn(v));
    }
}

// fractal_atlas_colourise_kfp, one 32 x 8 tile per block.
__global__ void __launch_bounds__(256) kfp_atlas_kernel(const KfpAtlasLaunch at, unsigned char* __restrict__ rgb,
                                                        const KfpDevice kp, const KfpDevice kc,
                                                        const unsigned char* __restrict__ lut_global,
                                                        const double* __restrict__ mc_period,
                                                        const int* __restrict__ mc_type) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < kp.width && y < kp.height) kfp_atlas_pixel(at, rgb, kp, kc, lut_global, mc_period, mc_type, x, y);
}

// ColorMethod 4 bounds: min/max of floor(sample) over escaped pixels below
// max_iter - 1 (kfp_transfer_bounds, renderer.cpp:7296-7331).  Doubles are
// mapped to order-preserving integers so one atomicMin/atomicMax pair works.
__device__ __forceinline__ unsigned long long ordered(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void kfp_plane_bounds_kernel(const float2* __restrict__ samples, const unsigned char* __restrict__ flags,
                                        long long pixels, int max_iter, unsigned long long* bounds) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (flags[i] & 1) continue;
        const float2 s = samples[i];
        double value = static_cast<double>(s.x) + static_cast<double>(s.y);
        value = value > static_cast<double>(max_iter) ? static_cast<double>(max_iter) : value;
        value = floor(value > 0.0 ? value : 0.0);
        if (value >= static_cast<double>(max_iter - 1)) continue;
        const unsigned long long o = ordered(value);
        lo = o < lo ? o : lo;
        hi = o > hi ? o : hi;
    }
    if (lo != ~0ull) atomicMin(bounds, lo);
    if (hi != 0ull) atomicMax(bounds + 1, hi);
}

__global__ void kfp_bounds_kernel(const float* __restrict__ field, long long pixels, int max_iter, double field_bias,
                                  double smooth_offset, unsigned long long* bounds) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float raw = field[i];
        if (isfinite(raw) && static_cast<double>(raw) >= static_cast<double>(max_iter) - field_bias) continue;
        const double safe = isfinite(raw) ? fmin(fmax(static_cast<double>(raw) + field_bias, 0.0),
                                                 static_cast<double>(max_iter))
                                          : 0.0;
        const double value = floor(safe + smooth_offset);
        if (value >= static_cast<double>(max_iter - 1)) continue;
        const unsigned long long o = ordered(value);
        lo = o < lo ? o : lo;
        hi = o > hi ? o : hi;
    }
    for (int offset = 16; offset > 0; offset >>= 1) {
        const unsigned long long a = __shfl_down_sync(0xffffffffu, lo, offset);
        const unsigned long long b = __shfl_down_sync(0xffffffffu, hi, offset);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(bounds, lo);
        atomicMax(bounds + 1, hi);
    }
}

}  // namespace

cudaError_t launch_kfp_bounds(const float* field, long long pixels, int max_iter, double field_bias,
                              double smooth_offset, unsigned long long* bounds, cudaStream_t stream) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    long long blocks = (pixels + 255) / 256;
    if (blocks > sms * 4LL) blocks = sms * 4LL;
    if (blocks < 1) blocks = 1;
    const unsigned long long init[2] = {~0ull, 0ull};
    cudaError_t status = cudaMemcpyAsync(bounds, init, sizeof init, cudaMemcpyHostToDevice, stream);
    if (status != cudaSuccess) return status;
    kfp_bounds_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(field, pixels, max_iter, field_bias,
                                                                          smooth_offset, bounds);
    return cudaGetLastError();
}

cudaError_t launch_kfp_plane_samples(const KfpPlanesLaunch& planes, int max_iter, long long pixels, void* samples,
                                     std::uint8_t* flags, cudaStream_t stream) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    long long blocks = (pixels + 255) / 256;
    if (blocks > static_cast<long long>(sms) * 16) blocks = static_cast<long long>(sms) * 16;
    kfp_plane_samples_kernel<<<static_cast<unsigned>(blocks < 1 ? 1 : blocks), 256, 0, stream>>>(
        planes, max_iter, pixels, static_cast<float2*>(samples), flags);
    return cudaGetLastError();
}

cudaError_t launch_kfp_plane_bounds(const void* samples, const std::uint8_t* flags, long long pixels, int max_iter,
                                    unsigned long long* bounds, cudaStream_t stream) {
    const unsigned long long init[2] = {~0ull, 0ull};
    cudaError_t status = cudaMemcpyAsync(bounds, init, sizeof init, cudaMemcpyHostToDevice, stream);
    if (status != cudaSuccess) return status;
    kfp_plane_bounds_kernel<<<152 * 4, 256, 0, stream>>>(static_cast<const float2*>(samples), flags, pixels, max_iter,
                                                         bounds);
    return cudaGetLastError();
}

namespace {

// The kernel constants of one KFP pass (doubles split into double-float
// pairs, exact FP32 thresholds) for a `launch.width`-wide source.
KfpDevice kfp_device(const KfpLaunch& launch, int spatial_width) {
    KfpDevice k{};
    k.width = launch.width;
    k.height = launch.height;
    k.max_iter = launch.max_iter;
    k.field_bias = static_cast<float>(launch.field_bias);
    k.field_bias_d = launch.field_bias;
    k.smooth_offset = static_cast<float>(launch.smooth_offset);
    k.smooth_offset_d = launch.smooth_offset;
    k.color_method = launch.color_method;
    k.differences = launch.differences;
    k.smooth = launch.smooth;
    k.flat = launch.flat;
    k.inverse_transition = launch.inverse_transition;
    k.needs_difference = launch.needs_difference;
    k.needs_slopes = launch.needs_slopes;
    k.iter_div = launch.iter_div;
    k.color_offset = launch.color_offset;
    k.transfer_min = launch.transfer_min;
    k.transfer_max = launch.transfer_max;
    k.multi_color = launch.multi_color;
    k.blend_multi_color = launch.blend_multi_color;
    k.multi_count = launch.multi_count;
    k.slope_cos = static_cast<float>(launch.slope_cos);
    k.slope_sin = static_cast<float>(launch.slope_sin);
    k.slope_power = static_cast<float>(launch.slope_power);
    k.slope_ratio = static_cast<float>(launch.slope_ratio);
    for (int c = 0; c < 3; ++c) k.interior[c] = launch.interior[c];
    k.lut_size = launch.lut_size;
    {
        const double threshold = static_cast<double>(launch.max_iter) - launch.field_bias;
        float hi = static_cast<float>(threshold);
        if (static_cast<double>(hi) < threshold) hi = std::nextafter(hi, std::numeric_limits<float>::infinity());
        k.sample_hi = hi;
    }
    k.sample_fast = launch.field_bias >= 0.0 && launch.smooth_offset >= 0.0 ? 1 : 0;
    auto split = [](double v, float& hi, float& lo) {
        hi = static_cast<float>(v);
        lo = static_cast<float>(v - static_cast<double>(hi));
    };
    split(launch.field_bias + launch.smooth_offset, k.shift_hi, k.shift_lo);
    split(1.0 / launch.iter_div, k.inv_div_hi, k.inv_div_lo);
    k.has_div = launch.iter_div != 1.0 ? 1 : 0;
    split(launch.color_offset, k.offset_hi, k.offset_lo);
    split(launch.transfer_min, k.tmin_hi, k.tmin_lo);
    split(1024.0 / std::fmax(launch.transfer_max - launch.transfer_min, 1.0e-12), k.tscale_hi, k.tscale_lo);
    k.inv_iter_div = 1.0 / launch.iter_div;
    k.lut_shift = -1;
    for (int shift = 0; shift < 31; ++shift) {
        if ((1 << shift) == launch.lut_size) k.lut_shift = shift;
    }
    k.spatial_width = spatial_width;
    return k;
}

}  // namespace

cudaError_t launch_kfp(const float* field, std::uint8_t* rgb, const KfpLaunch& launch, const std::uint8_t* lut,
                       const double* mc_period, const int* mc_type, cudaStream_t stream,
                       const KfpPlanesLaunch* planes, const void* samples, const std::uint8_t* flags) {
    const KfpDevice k = kfp_device(launch, launch.width);
    const dim3 block(32, 8);
    const dim3 grid((launch.width + 31) / 32, (launch.height + 7) / 8);
    if (planes != nullptr) {
        kfp_kernel<true, false><<<grid, block, 0, stream>>>(field, rgb, k, lut, mc_period, mc_type, *planes,
                                                          static_cast<const float2*>(samples), flags);
    } else {
        const bool kalles = k.color_method == 7 && k.differences == 3 && k.smooth && !k.flat && !k.inverse_transition
            && !k.multi_color && k.needs_slopes && k.lut_shift >= 0;
        if (kalles) {
            kfp_kernel<false, true><<<grid, block, 0, stream>>>(field, rgb, k, lut, mc_period, mc_type,
                                                                KfpPlanesLaunch{}, nullptr, nullptr);
            return cudaGetLastError();
        }
        kfp_kernel<false, false><<<grid, block, 0, stream>>>(field, rgb, k, lut, mc_period, mc_type, KfpPlanesLaunch{},
                                                           nullptr, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_kfp_atlas(const KfpAtlasLaunch& atlas, std::uint8_t* rgb, const KfpLaunch& parent_launch,
                             const std::uint8_t* lut, const double* mc_period, const int* mc_type,
                             cudaStream_t stream) {
    const KfpDevice kp = kfp_device(parent_launch, parent_launch.width);
    KfpLaunch child_launch = parent_launch;
    child_launch.width = atlas.child ? atlas.child_width : 1;
    child_launch.height = atlas.child ? atlas.child_height : 1;
    child_launch.transfer_min = atlas.child_transfer_min;
    child_launch.transfer_max = atlas.child_transfer_max;
    const KfpDevice kc = kfp_device(child_launch, parent_launch.width);
    const dim3 block(32, 8);
    const dim3 grid((parent_launch.width + 31) / 32, (parent_launch.height + 7) / 8);
    kfp_atlas_kernel<<<grid, block, 0, stream>>>(atlas, rgb, kp, kc, lut, mc_period, mc_type);
    return cudaGetLastError();
}

namespace {

// Every 32-bit pattern x: div_const(x, d, RN(1/d)) against the IEEE quotient
// x / d, bit for bit (any two NaNs agree); mismatches are counted.
__global__ void division_check_kernel(float d, unsigned long long* mismatches) {
    const float r = 1.0f / d;
    unsigned long long local = 0;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
         i < (1ull << 32); i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float x = __uint_as_float(static_cast<unsigned>(i));
        const float want = x / d, got = div_const(x, d, r);
        const bool same = __float_as_uint(want) == __float_as_uint(got) || (isnan(want) && isnan(got));
        local += same ? 0 : 1;
    }
    if (local) atomicAdd(mismatches, local);
}

}  // namespace

cudaError_t launch_division_check(float divisor, unsigned long long* mismatches, cudaStream_t stream) {
    cudaError_t status = cudaMemsetAsync(mismatches, 0, sizeof(unsigned long long), stream);
    if (status != cudaSuccess) return status;
    division_check_kernel<<<152 * 16, 256, 0, stream>>>(divisor, mismatches);
    return cudaGetLastError();
}

}  // namespace fgb
