// Atlas compositor: one video frame from a parent keyframe and the next,
// deeper child keyframe (the zoom between two atlas levels), as a scalar
// field or coloured with the aurora palette.
//
// Restates fractal_atlas_field_ex (renderer.cpp:18697-18888) and
// atlas_colourise_impl (renderer.cpp:19138-19430): per output pixel a
// bilinear sample of the parent (centred crop by the parent zoom) and, in the
// centred child rectangle (child_fraction of the frame), of the child, with a
// smoothstep feather at the child's edges.  Samples preserve interior
// (sample_bilinear_mapped_preserving_interior, renderer.cpp:5141-5208): the
// four neighbours' weights split into interior (value >= cap - bias) and
// exterior; interior wins at weight >= 1/2, otherwise the exterior values are
// renormalised.
//
// fractal_atlas_colourise_kfp_raw (renderer.cpp:17969-18304) composes the
// same two sources into one scalar surface instead (child axes over the
// visible rectangle with the window formula, encoded relative to the KFP
// field bias, a 2-D smoothstep seam), which the KFP colour pass then reads
// from L2.
//
// Three launches per frame:
//   atlas_axes_kernel   the per-frame tables (parent x/y and child x/y
//                       bilinear axes: fill_bilinear_axis, renderer.cpp:
//                       4931-4961; the child's edge ramps), one thread per
//                       entry (~12k entries at 4K);
//   atlas_kernel        four output pixels per thread, no FP64: 16-byte
//                       field stores or 12-byte RGB stores; pixels it cannot
//                       decide exactly are queued;
//   atlas_exact_kernel  the queued pixels in the reference's FP64 form.
// This unit is compiled without FMA contraction, so every double and float
// operation rounds on its own exactly as in the reference: frames are
// bit-identical, not merely close.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>

#include "device.h"

namespace fgb {
namespace {

struct Sample {
    float value;
    bool inside;
};

// Per-source constants of a sample.
struct SourceView {
    const float* data;
    int width;
    int max_iter;
    double bias;       // the reference's double bias
    float limit;       // smallest float >= max_iter - bias: v >= limit <=> (double)v >= max_iter - bias
    float bias_hi, bias_lo;  // bias as a double-float
};

// ---- double-float (hi + lo FP32 pairs; Dekker / Knuth error-free sums and
// FMA products).  This unit runs without contraction, so every + and *
// below rounds on its own, as these algorithms require.
struct Df {
    float hi, lo;
};

__device__ __forceinline__ Df two_sum(float a, float b) {
    const float s = a + b;
    const float v = s - a;
    return Df{s, (a - (s - v)) + (b - v)};
}

__device__ __forceinline__ Df quick_two_sum(float a, float b) {
    const float s = a + b;
    return Df{s, b - (s - a)};
}

__device__ __forceinline__ Df df_mul(Df a, Df b) {
    const float p = a.hi * b.hi;
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = e + (a.hi * b.lo + a.lo * b.hi);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ Df df_add(Df a, Df b) {
    const Df s = two_sum(a.hi, b.hi);
    return quick_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

// sample_bilinear_mapped_preserving_interior exactly as the reference forms
// it, in FP64 (renderer.cpp:5141-5208).
__device__ __forceinline__ Sample sample_exact(const SourceView& src, const float values[4], double xw, double yw) {
    const double weights[4] = {(1.0 - yw) * (1.0 - xw), (1.0 - yw) * xw, yw * (1.0 - xw), yw * xw};
    const double limit = static_cast<double>(src.max_iter) - src.bias;
    double interior = 0.0, exterior = 0.0, sum = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float v = values[i];
        if (isfinite(v) && static_cast<double>(v) >= limit) {
            interior += weights[i];
        } else if (isfinite(v)) {
            exterior += weights[i];
            sum += (static_cast<double>(v) + src.bias) * weights[i];
        }
    }
    if (interior >= 0.5) return Sample{static_cast<float>(src.max_iter), true};
    if (exterior <= 1.0e-12) return Sample{0.0f, false};
    return Sample{static_cast<float>(exterior == 1.0 ? sum : sum / exterior), false};  // x / 1 = x
}

// Df quotient a / b (b > 0): one float quotient refined by the exact
// remainder, about 2^-44 relative.
__device__ __forceinline__ Df df_div(Df a, Df b) {
    const float q1 = a.hi / b.hi;
    const float p = q1 * b.hi;
    const float pe = __fmaf_rn(q1, b.hi, -p);
    const Df r = df_add(a, Df{-p, -(pe + q1 * b.lo)});
    return quick_two_sum(q1, r.hi / b.hi);
}

// The float nearest to the Df value v when every value within `tolerance`
// of v rounds to the same float; false when v is too close to a rounding
// boundary to decide.
__device__ __forceinline__ bool decided_float(Df v, float tolerance, float& out) {
    // Half the gaps to the neighbouring floats of v.hi from its exponent
    // bits: 2^(e-24) on both sides, halved towards zero at a power of two.
    const unsigned bits = __float_as_uint(v.hi) & 0x7fffffffu;
    out = v.hi;
    if (bits < 0x0d800000u || bits >= 0x7f000000u) return false;  // tiny, huge or non-finite: undecided
    const float half = __uint_as_float(bits & 0x7f800000u) * 0x1p-24f;
    const float inner = (bits & 0x007fffffu) == 0u ? half * 0.5f : half;
    const float up = v.hi > 0.0f ? half : inner;
    const float down = v.hi > 0.0f ? inner : half;
    return v.lo + tolerance < up && tolerance - v.lo < down;
}

// Df times a float (error < 2^-47 relative).
__device__ __forceinline__ Df df_mul_f(Df a, float s) {
    const float p = a.hi * s;
    const float e = __fmaf_rn(a.hi, s, -p) + a.lo * s;
    return quick_two_sum(p, e);
}

// The same sample without FP64, with identical results.  The four bilinear
// weights W_k are formed in double-float (exact 1 - w, FMA products); the
// interior weight I, the exterior weight E and N = sum of (v_k + bias) W_k
// over exterior corners follow.  The reference's double forms differ from
// these exact sums by < 2^-49 relatively, the double-float forms by
// < 2^-44, so:
//  * interior: I >= 1/2 is decided when |I - 1/2| > 2^-42;
//  * a value: float(N / E) is decided when N / E +- 2^-42 max |v_k + bias|
//    lies inside one float's rounding cell (E = 1 exactly in real
//    arithmetic when all four corners are exterior, so no division then).
//    Both error bounds are relative to the sample scale, not to E: the
//    reference's D errs by < 14 * 2^-53 max |v_k + bias| (weights, products,
//    sums, quotient), the double-float N / E by < 2^-46 of it;
//  * E <= 1e-12 (no usable corner) is decided away from 1e-12.
// Undecided samples (about one in 2^16, and exact 1/2 ties of I) take the
// reference's FP64 form.
template <bool Exact>
__device__ __forceinline__ Sample sample_preserving_interior(const SourceView& src, const AtlasAxis& ax,
                                                             const AtlasAxis& ay, int x, int y, bool& undecided) {
    const int x0 = __ldg(ax.index0 + x), x1 = __ldg(ax.index1 + x);
    const float xw = __ldg(ax.weight + x);
    const int y0 = __ldg(ay.index0 + y), y1 = __ldg(ay.index1 + y);
    const float yw = __ldg(ay.weight + y);
    const float* top = src.data + static_cast<long long>(y0) * src.width;
    const float* bottom = src.data + static_cast<long long>(y1) * src.width;
    const float values[4] = {__ldg(top + x0), __ldg(top + x1), __ldg(bottom + x0), __ldg(bottom + x1)};
    if constexpr (Exact) {
        return sample_exact(src, values, static_cast<double>(xw), static_cast<double>(yw));
    }
    int interior_mask = 0, exterior_mask = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (isfinite(values[i])) {
            if (values[i] >= src.limit) {
                interior_mask |= 1 << i;
            } else {
                exterior_mask |= 1 << i;
            }
        }
    }
    if (interior_mask == 15) return Sample{static_cast<float>(src.max_iter), true};
    if (exterior_mask == 15) {
        // N = T + y (B - T) with the row values T = u0 + x (u1 - u0),
        // B = u2 + x (u3 - u2): the same exact real as the four weighted
        // corners (weights sum to 1), in fewer double-float steps.
        Df u0{values[0], 0.0f}, u2{values[2], 0.0f};
        if (src.bias_hi != 0.0f) {
            u0 = two_sum(values[0], src.bias_hi);
            u0 = quick_two_sum(u0.hi, u0.lo + src.bias_lo);
            u2 = two_sum(values[2], src.bias_hi);
            u2 = quick_two_sum(u2.hi, u2.lo + src.bias_lo);
        }
        const Df row_top = df_add(u0, df_mul_f(two_sum(values[1], -values[0]), xw));
        const Df row_bottom = df_add(u2, df_mul_f(two_sum(values[3], -values[2]), xw));
        const Df n = df_add(row_top, df_mul_f(df_add(row_bottom, Df{-row_top.hi, -row_top.lo}), yw));
        const float magnitude = fmaxf(fmaxf(fabsf(values[0]), fabsf(values[1])), fmaxf(fabsf(values[2]),
                                                                                      fabsf(values[3])))
            + fabsf(src.bias_hi);
        float result;
        if (decided_float(n, magnitude * 0x1p-42f + 0x1p-120f, result)) return Sample{result, false};
        undecided = true;
        return Sample{0.0f, false};
    }
    const Df x_left = two_sum(1.0f, -xw), y_top = two_sum(1.0f, -yw);
    const Df x_right{xw, 0.0f}, y_bottom{yw, 0.0f};
    const Df w[4] = {df_mul(y_top, x_left), df_mul(y_top, x_right), df_mul(y_bottom, x_left),
                     df_mul(y_bottom, x_right)};
    bool decided = true;
    if (interior_mask != 0) {
        Df interior{0.0f, 0.0f};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (interior_mask & (1 << i)) interior = df_add(interior, w[i]);
        }
        const Df margin = df_add(interior, Df{-0.5f, 0.0f});
        if (margin.hi > 0x1p-42f) return Sample{static_cast<float>(src.max_iter), true};
        decided = margin.hi < -0x1p-42f;
    }
    if (decided) {
        Df n{0.0f, 0.0f}, e{0.0f, 0.0f};
        float magnitude = 0.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (!(exterior_mask & (1 << i))) continue;
            Df u{values[i], 0.0f};
            if (src.bias_hi != 0.0f) {
                u = two_sum(values[i], src.bias_hi);
                u = quick_two_sum(u.hi, u.lo + src.bias_lo);
            }
            magnitude = fmaxf(magnitude, fabsf(u.hi));
            n = df_add(n, df_mul(u, w[i]));
            e = df_add(e, w[i]);
        }
        float result;
        if (e.hi > 2.0e-12f) {
            if (decided_float(df_div(n, e), magnitude * 0x1p-42f + 0x1p-120f, result)) return Sample{result, false};
        } else if (e.hi < 0.5e-12f) {
            return Sample{0.0f, false};
        }
    }
    undecided = true;  // left to the exact pass
    return Sample{0.0f, false};
}

// write_colour_pixel (renderer.cpp:5210-5237).  The palette index is
// floor(double(smooth) * double(index_scale)); that product of two floats is
// exact in double, so it is formed exactly as p + e (FMA two-product) and
// compared and floored without FP64.
__device__ __forceinline__ void palette_entry(const AtlasLaunch& a, float smooth, std::uint8_t* dst) {
    if (!isfinite(smooth)) {  // NaN and -inf take entry 0, +inf the last
        const int k = smooth > 0.0f ? a.lut_size - 1 : 0;
        dst[0] = __ldg(a.lut + 3 * k);
        dst[1] = __ldg(a.lut + 3 * k + 1);
        dst[2] = __ldg(a.lut + 3 * k + 2);
        return;
    }
    const float p = smooth * a.index_scale;
    const float e = __fmaf_rn(smooth, a.index_scale, -p);
    const int last = a.lut_size - 1;
    const float last_f = static_cast<float>(last);
    int k;
    if (p > last_f || (p == last_f && e >= 0.0f)) {
        k = last;
    } else if (p < 0.0f || (p == 0.0f && e <= 0.0f)) {
        k = 0;
    } else {
        const float f = floorf(p);
        k = static_cast<int>(f) - (p == f && e < 0.0f ? 1 : 0);
    }
    dst[0] = __ldg(a.lut + 3 * k);
    dst[1] = __ldg(a.lut + 3 * k + 1);
    dst[2] = __ldg(a.lut + 3 * k + 2);
}

__device__ __forceinline__ void aurora_colour(const AtlasLaunch& a, float smooth, std::uint8_t* dst) {
    if (!isfinite(smooth) || smooth >= static_cast<float>(a.palette_iter)) {
        dst[0] = static_cast<std::uint8_t>(a.interior[0]);
        dst[1] = static_cast<std::uint8_t>(a.interior[1]);
        dst[2] = static_cast<std::uint8_t>(a.interior[2]);
        return;
    }
    palette_entry(a, smooth, dst);
}

// rounded_colour_byte (renderer.cpp:5239-5244).
__device__ __forceinline__ std::uint8_t rounded_byte(double v) {
    const double c = v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v);
    const int r = static_cast<int>(rint(c));
    return static_cast<std::uint8_t>(r < 0 ? 0 : (r > 255 ? 255 : r));
}

// rounded_colour_byte(double(p) * (1 - alpha) + double(c) * alpha) for bytes
// p, c and a float alpha in [0, 1] without FP64.  That double expression is
// exact (each product has <= 33 significant bits and the sum stays within 53
// because alpha >= 2^-12 or alpha = 0 on the seam ramps), so its value is
// V = p + (c - p) alpha exactly; (c - p) alpha = h + l by FMA two-product,
// and V is rounded half to even from h, l and the integer p.
__device__ __forceinline__ std::uint8_t blend_byte(std::uint8_t p, std::uint8_t c, float alpha) {
    const float d = static_cast<float>(static_cast<int>(c) - static_cast<int>(p));
    const float h = d * alpha;
    const float l = __fmaf_rn(d, alpha, -h);
    float floor_t = floorf(h);
    if (h == floor_t && l < 0.0f) floor_t -= 1.0f;
    const float frac_hi = h - floor_t;  // exact; frac = frac_hi + l
    int base = static_cast<int>(p) + static_cast<int>(floor_t);
    if (frac_hi > 0.5f || (frac_hi == 0.5f && l > 0.0f)) {
        base += 1;
    } else if (frac_hi == 0.5f && l == 0.0f) {
        base += base & 1;  // half to even
    }
    return static_cast<std::uint8_t>(base < 0 ? 0 : (base > 255 ? 255 : base));
}

// One entry of a bilinear axis (fill_bilinear_axis, renderer.cpp:4931-4961):
// `source` samples resampled after a centred crop, position
// left + (d + 1/2) step - 1/2 with the axis constants formed on the host in
// the reference's order; the window form (fill_bilinear_axis_window,
// renderer.cpp:4969-5003, at the visible child pixel d, where the halo
// offset cancels) is left + (d + 1/2) crop / span - 1/2.
__device__ void axis_entry(const AtlasAxisPlan& plan, int d, int* index0, int* index1, float* weight) {
    const double logical = static_cast<double>(d) + 0.5;
    double position = plan.window ? plan.left + logical * plan.crop / plan.span - 0.5
                                  : plan.left + logical * plan.step - 0.5;
    const double top = static_cast<double>(plan.source - 1);
    position = position < 0.0 ? 0.0 : (position > top ? top : position);
    const int i = static_cast<int>(floor(position));
    index0[d] = i;
    index1[d] = i + 1 < plan.source - 1 ? i + 1 : plan.source - 1;
    weight[d] = static_cast<float>(position - static_cast<double>(i));
}

// encode_render_value (renderer.cpp:119-121): float(value - bias) formed in
// extended precision.  `value` (a float sample or an integer cap) and `bias`
// are doubles; the exact difference is hi + lo (two-sum), and the float
// nearest to it is float(hi) except when hi sits exactly halfway between two
// floats, where lo decides.
__device__ __forceinline__ float encode_exact(double value, double bias) {
    const double hi = value - bias;
    const double b_virtual = hi - value;
    const double lo = (value - (hi - b_virtual)) + (-bias - b_virtual);
    const float f = static_cast<float>(hi);
    if (lo == 0.0 || !isfinite(hi)) return f;
    const float below = static_cast<double>(f) <= hi ? f : nextafterf(f, -INFINITY);
    const float above = nextafterf(below, INFINITY);
    const double middle = 0.5 * (static_cast<double>(below) + static_cast<double>(above));
    if (hi != middle) return f;
    return lo > 0.0 ? above : below;
}

// Smoothstep ramp towards the child's edges (renderer.cpp:18786-18801).
__device__ float edge_ramp(int size, int feather, int i) {
    const int edge = i < size - 1 - i ? i : size - 1 - i;
    float linear = static_cast<float>(edge) / static_cast<float>(feather);
    linear = linear < 1.0f ? linear : 1.0f;
    return linear * linear * (3.0f - 2.0f * linear);
}

__global__ void atlas_axes_kernel(const AtlasLaunch a, AtlasTables t) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.exact_count = 0;
    const int segments[7] = {t.parent_x_size, t.parent_y_size, t.child_x_size, t.child_y_size, t.edge_x_size,
                             t.edge_y_size, t.alpha_size};
    int total = 0;
#pragma unroll
    for (int s = 0; s < 7; ++s) total += segments[s];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int d = e, s = 0;
        while (d >= segments[s]) d -= segments[s++];
        switch (s) {
            case 0: axis_entry(t.plan[0], d, t.parent_x.i0, t.parent_x.i1, t.parent_x.w); break;
            case 1: axis_entry(t.plan[1], d, t.parent_y.i0, t.parent_y.i1, t.parent_y.w); break;
            case 2: axis_entry(t.plan[2], d, t.child_x.i0, t.child_x.i1, t.child_x.w); break;
            case 3: axis_entry(t.plan[3], d, t.child_y.i0, t.child_y.i1, t.child_y.w); break;
            case 4:
                t.edge_x[d] = edge_ramp(t.edge_x_size, a.feather, d);
                break;
            case 5:
                t.edge_y[d] = edge_ramp(t.edge_y_size, a.feather, d);
                break;
            default: {
                // fractal_atlas_composite_rgb's double smoothstep at edge
                // distance d (renderer.cpp:18598-18609).
                double linear = static_cast<double>(d) / static_cast<double>(a.feather);
                linear = linear < 0.0 ? 0.0 : (linear > 1.0 ? 1.0 : linear);
                t.alpha[d] = linear * linear * (3.0 - 2.0 * linear);
                break;
            }
        }
    }
}

__device__ __forceinline__ SourceView parent_view(const AtlasLaunch& a) {
    return SourceView{a.parent, a.parent_width, a.parent_max_iter, a.parent_bias, a.parent_limit, a.parent_bias_hi,
                      a.parent_bias_lo};
}

__device__ __forceinline__ SourceView child_view(const AtlasLaunch& a) {
    return SourceView{a.child, a.child_width, a.child_max_iter, a.child_bias, a.child_limit, a.child_bias_hi,
                      a.child_bias_lo};
}

__device__ __forceinline__ bool in_child(const AtlasLaunch& a, int cx, int cy) {
    return a.use_child && cx >= 0 && cx < a.child_visible_width && cy >= 0 && cy < a.child_visible_height;
}

__device__ __forceinline__ float seam_alpha(const AtlasLaunch& a, int cx, int cy) {
    if (a.feather < 2) return 1.0f;
    const float ex = __ldg(a.edge_x + cx), ey = __ldg(a.edge_y + cy);
    return ex < ey ? ex : ey;
}

// Scalar output of one pixel (fractal_atlas_field_ex's per-pixel body).
template <bool Exact>
__device__ __forceinline__ float field_pixel(bool& undecided, const AtlasLaunch& a, const SourceView& parent, const SourceView& child,
                                             int x, int y) {
    const float bias = a.output_bias_f;
    if (a.full_child) {
        const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, x, y, undecided);
        return c.inside ? a.interior_value : c.value - bias;
    }
    const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
    float value = p.inside ? a.interior_value : p.value - bias;
    const int cx = x - a.child_left, cy = y - a.child_top;
    if (in_child(a, cx, cy)) {
        const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, cx, cy, undecided);
        const float child_value = c.inside ? a.interior_value : c.value - bias;
        const float alpha = seam_alpha(a, cx, cy);
        value = value * (1.0f - alpha) + child_value * alpha;
    }
    return value;
}

// encode_render_value of a sample: with a bias that is itself a float the
// reference's extended-precision difference rounds to float(v - bias).
__device__ __forceinline__ float encode_sample(const AtlasLaunch& a, float value) {
    return a.output_bias_exact ? value - a.output_bias_f : encode_exact(static_cast<double>(value), a.output_bias);
}

// Scalar surface of one pixel (fractal_atlas_colourise_kfp_raw's parent
// view, then the child's ownership blend).
template <bool Exact>
__device__ __forceinline__ float surface_pixel(bool& undecided, const AtlasLaunch& a, const SourceView& parent,
                                               const SourceView& child, int x, int y) {
    // The child owns its rectangle outside the seam band, where the parent
    // sample is not used: it is taken only where a pixel blends.
    const int cx = x - a.child_left, cy = y - a.child_top;
    const bool child_here = in_child(a, cx, cy);
    float child_value = 0.0f, alpha = 0.0f;
    if (child_here) {
        const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, cx, cy, undecided);
        child_value = c.inside ? a.interior_value : encode_sample(a, c.value);
        alpha = seam_alpha(a, cx, cy);
        if (alpha >= 0.999999f) return child_value;
    }
    const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
    const float parent_value = p.inside ? a.interior_value : encode_sample(a, p.value);
    return child_here ? parent_value * (1.0f - alpha) + child_value * alpha : parent_value;
}

// Scalar surface of one pixel of fractal_atlas_colourise_kfp_planes
// (renderer.cpp:17520-17553, 17686-17706): the primary tile (the child when
// it fills the frame) everywhere, the child blended in over its rectangle
// with no shortcut at alpha 1; interior flags for the plane pass.
template <bool Exact>
__device__ __forceinline__ float planes_surface_pixel(bool& undecided, const AtlasLaunch& a, const SourceView& parent,
                                                      const SourceView& child, int x, int y) {
    std::uint8_t flags;
    float value;
    if (a.full_child) {
        const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, x, y, undecided);
        flags = c.inside ? 1 : 0;
        value = c.inside ? a.interior_value : encode_sample(a, c.value);
    } else {
        const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
        flags = p.inside ? 1 : 0;
        value = p.inside ? a.interior_value : encode_sample(a, p.value);
        const int cx = x - a.child_left, cy = y - a.child_top;
        if (in_child(a, cx, cy)) {
            const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, cx, cy, undecided);
            flags |= c.inside ? 2 : 0;
            const float child_value = c.inside ? a.interior_value : encode_sample(a, c.value);
            const float alpha = seam_alpha(a, cx, cy);
            value = value * (1.0f - alpha) + child_value * alpha;
        }
    }
    a.inside_out[static_cast<long long>(y) * a.out_width + x] = flags;
    return value;
}

// RGB8 of one pixel (atlas_colourise_impl's per-pixel body).
template <bool Exact>
__device__ __forceinline__ void colour_pixel(bool& undecided, const AtlasLaunch& a, const SourceView& parent, const SourceView& child,
                                             int x, int y, std::uint8_t* dst) {
    const float cap = static_cast<float>(a.palette_iter);
    if (a.full_child) {
        const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, x, y, undecided);
        aurora_colour(a, c.inside ? cap : c.value, dst);
        return;
    }
    const int cx = x - a.child_left, cy = y - a.child_top;
    if (!in_child(a, cx, cy)) {
        const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
        aurora_colour(a, p.inside ? cap : p.value, dst);
        return;
    }
    const Sample c = sample_preserving_interior<Exact>(child, a.child_x, a.child_y, cx, cy, undecided);
    const float alpha = seam_alpha(a, cx, cy);
    if (alpha >= 0.999999f) {
        aurora_colour(a, c.inside ? cap : c.value, dst);
        return;
    }
    const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
    std::uint8_t prgb[3], crgb[3];
    aurora_colour(a, p.inside ? cap : p.value, prgb);
    aurora_colour(a, c.inside ? cap : c.value, crgb);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) dst[ch] = blend_byte(prgb[ch], crgb[ch], alpha);
}

// sample_bilinear_mapped (renderer.cpp:5053-5073): plain float bilinear.
__device__ __forceinline__ float crop_pixel(const AtlasLaunch& a, int x, int y) {
    const int x0 = __ldg(a.parent_x.index0 + x), x1 = __ldg(a.parent_x.index1 + x);
    const float xw = __ldg(a.parent_x.weight + x);
    const int y0 = __ldg(a.parent_y.index0 + y), y1 = __ldg(a.parent_y.index1 + y);
    const float yw = __ldg(a.parent_y.weight + y);
    const float* top = a.parent + static_cast<long long>(y0) * a.parent_width;
    const float* bottom = a.parent + static_cast<long long>(y1) * a.parent_width;
    const float top_value = __ldg(top + x0) * (1.0f - xw) + __ldg(top + x1) * xw;
    const float bottom_value = __ldg(bottom + x0) * (1.0f - xw) + __ldg(bottom + x1) * xw;
    return top_value * (1.0f - yw) + bottom_value * yw;
}

// sample_rgb_bilinear_mapped (renderer.cpp:5262-5298): per channel float
// bilinear, rounded half to even and clamped like rounded_colour_byte (the
// double conversion of a float changes nothing there).
__device__ __forceinline__ void rgb_sample(const std::uint8_t* __restrict__ source, int width, const AtlasAxis& ax,
                                           const AtlasAxis& ay, int x, int y, std::uint8_t* dst) {
    const int x0 = __ldg(ax.index0 + x), x1 = __ldg(ax.index1 + x);
    const float xw = __ldg(ax.weight + x);
    const int y0 = __ldg(ay.index0 + y), y1 = __ldg(ay.index1 + y);
    const float yw = __ldg(ay.weight + y);
    const std::uint8_t* top = source + (static_cast<long long>(y0) * width + x0) * 3;
    const std::uint8_t* top_next = source + (static_cast<long long>(y0) * width + x1) * 3;
    const std::uint8_t* bottom = source + (static_cast<long long>(y1) * width + x0) * 3;
    const std::uint8_t* bottom_next = source + (static_cast<long long>(y1) * width + x1) * 3;
    const float ix = 1.0f - xw, iy = 1.0f - yw;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float t = static_cast<float>(__ldg(top + c)) * ix + static_cast<float>(__ldg(top_next + c)) * xw;
        const float b = static_cast<float>(__ldg(bottom + c)) * ix + static_cast<float>(__ldg(bottom_next + c)) * xw;
        float v = t * iy + b * yw;
        v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
        dst[c] = static_cast<std::uint8_t>(rintf(v));
    }
}

// fractal_atlas_composite_rgb's per-pixel body (renderer.cpp:18572-18617).
__device__ __forceinline__ void rgb_pixel(const AtlasLaunch& a, int x, int y, std::uint8_t* dst) {
    rgb_sample(a.parent_rgb, a.parent_width, a.parent_x, a.parent_y, x, y, dst);
    const int cx = x - a.child_left, cy = y - a.child_top;
    if (!in_child(a, cx, cy)) return;
    std::uint8_t child[3];
    rgb_sample(a.child_rgb, a.child_width, a.child_x, a.child_y, cx, cy, child);
    double alpha = 1.0;
    if (a.feather >= 2) {
        const int ex = cx < a.child_visible_width - 1 - cx ? cx : a.child_visible_width - 1 - cx;
        const int ey = cy < a.child_visible_height - 1 - cy ? cy : a.child_visible_height - 1 - cy;
        const int edge = ex < ey ? ex : ey;
        alpha = edge >= a.feather ? 1.0 : __ldg(a.alpha + edge);
    }
    if (alpha == 1.0) {  // parent * 0 + child * 1 is the child's byte exactly
        dst[0] = child[0];
        dst[1] = child[1];
        dst[2] = child[2];
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        dst[c] = rounded_byte(static_cast<double>(dst[c]) * (1.0 - alpha) + static_cast<double>(child[c]) * alpha);
    }
}

// crop_colourise_impl's per-pixel body (renderer.cpp:19053-19078): interior
// colour for an interior sample, else the palette entry (no cap test).
template <bool Exact>
__device__ __forceinline__ void crop_aurora_pixel(bool& undecided, const AtlasLaunch& a, const SourceView& parent, int x, int y,
                                                  std::uint8_t* dst) {
    const Sample p = sample_preserving_interior<Exact>(parent, a.parent_x, a.parent_y, x, y, undecided);
    if (p.inside) {
        dst[0] = static_cast<std::uint8_t>(a.interior[0]);
        dst[1] = static_cast<std::uint8_t>(a.interior[1]);
        dst[2] = static_cast<std::uint8_t>(a.interior[2]);
        return;
    }
    palette_entry(a, p.value, dst);
}

// One output pixel of any mode: a float (field_out modes) into *value or
// three bytes into rgb.
template <bool Exact, int Mode>
__device__ __forceinline__ void atlas_pixel(const AtlasLaunch& a, const SourceView& parent, const SourceView& child,
                                            int x, int y, bool& undecided, float* value, std::uint8_t* rgb) {
    switch (Mode) {
        case kAtlasKfpSurface: *value = surface_pixel<Exact>(undecided, a, parent, child, x, y); break;
        case kAtlasKfpPlanes: *value = planes_surface_pixel<Exact>(undecided, a, parent, child, x, y); break;
        case kAtlasCropField: *value = crop_pixel(a, x, y); break;
        case kAtlasField: *value = field_pixel<Exact>(undecided, a, parent, child, x, y); break;
        case kAtlasRgb: rgb_pixel(a, x, y, rgb); break;
        case kAtlasCropAurora: crop_aurora_pixel<Exact>(undecided, a, parent, x, y, rgb); break;
        default: colour_pixel<Exact>(undecided, a, parent, child, x, y, rgb); break;
    }
}

// Queues pixel `index` for the exact pass (warp-aggregated append).
__device__ __forceinline__ void queue_exact(const AtlasLaunch& a, bool undecided, unsigned index) {
    const unsigned active = __activemask();
    const unsigned want = __ballot_sync(active, undecided);
    if (!undecided) return;
    const int leader = __ffs(want) - 1;
    const int lane = threadIdx.x & 31;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(a.exact_count, static_cast<unsigned>(__popc(want)));
    base = __shfl_sync(want, base, leader);
    a.exact_pixels[base + __popc(want & ((1u << lane) - 1u))] = index;
}

// The fast pass: four horizontally adjacent pixels per thread, no FP64.
// `quads_per_row` = ceil(width / 4); a row's last quad may be partial.  Full
// quads of a row whose width is a multiple of four store 16 bytes (field) or
// 12 bytes (RGB, three aligned words); everything else stores per pixel.  A
// pixel whose sample could not be decided in double-float is written with a
// placeholder and queued for atlas_exact_kernel, which rewrites it.
template <int Mode>
__global__ void __launch_bounds__(256, (Mode == kAtlasRgb || Mode == kAtlasCropAurora) ? 6 : 8)
    atlas_kernel(const AtlasLaunch a, unsigned quads_per_row,
                                                    unsigned total_quads) {
    const bool vector_rows = (a.out_width & 3) == 0;
    const SourceView parent = parent_view(a), child = child_view(a);
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < total_quads; q += gridDim.x * blockDim.x) {
        const int y = static_cast<int>(q / quads_per_row);
        const int x0 = static_cast<int>(q - static_cast<unsigned>(y) * quads_per_row) * 4;
        const long long row = static_cast<long long>(y) * a.out_width;
        const int n = a.out_width - x0 < 4 ? a.out_width - x0 : 4;
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        std::uint8_t out[12];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            bool undecided = false;
            if (k < n) atlas_pixel<false, Mode>(a, parent, child, x0 + k, y, undecided, v + k, out + 3 * k);
            queue_exact(a, undecided, static_cast<unsigned>(row + x0 + k));
        }
        if (a.field_out) {
            if (vector_rows) {
                __stcs(reinterpret_cast<float4*>(a.field_out + row + x0), make_float4(v[0], v[1], v[2], v[3]));
            } else {
                for (int k = 0; k < n; ++k) a.field_out[row + x0 + k] = v[k];
            }
        } else {
            std::uint8_t* dst = a.rgb + 3 * (row + x0);
            if (vector_rows) {
                std::uint32_t* words = reinterpret_cast<std::uint32_t*>(dst);
                __stcs(words, out[0] | (out[1] << 8) | (out[2] << 16) | (static_cast<std::uint32_t>(out[3]) << 24));
                __stcs(words + 1,
                       out[4] | (out[5] << 8) | (out[6] << 16) | (static_cast<std::uint32_t>(out[7]) << 24));
                __stcs(words + 2,
                       out[8] | (out[9] << 8) | (out[10] << 16) | (static_cast<std::uint32_t>(out[11]) << 24));
            } else {
                for (int k = 0; k < 3 * n; ++k) dst[k] = out[k];
            }
        }
    }
}

// The exact pass: the queued pixels, one per thread, every sample in the
// reference's FP64 form.  Dense warps, so the FP64 pipe runs with all lanes
// active; the list is usually a few hundred pixels, up to a few percent of a
// frame whose axes fall on exact halves (2:1 resampling).
template <int Mode>
__global__ void __launch_bounds__(256) atlas_exact_kernel(const AtlasLaunch a) {
    const SourceView parent = parent_view(a), child = child_view(a);
    const unsigned count = *a.exact_count;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const unsigned index = a.exact_pixels[i];
        const int y = static_cast<int>(index / static_cast<unsigned>(a.out_width));
        const int x = static_cast<int>(index - static_cast<unsigned>(y) * static_cast<unsigned>(a.out_width));
        bool undecided = false;
        float value = 0.0f;
        std::uint8_t rgb[3];
        atlas_pixel<true, Mode>(a, parent, child, x, y, undecided, &value, rgb);
        if (a.field_out) {
            a.field_out[index] = value;
        } else {
            a.rgb[3ull * index] = rgb[0];
            a.rgb[3ull * index + 1] = rgb[1];
            a.rgb[3ull * index + 2] = rgb[2];
        }
    }
}

// One source's bilinear / nearest plane samples at local (x, y) through its
// axes (sample_bilinear_mapped_double, sample_nearest_mapped_*:
// renderer.cpp:5076-5138).  Compiled without FMA contraction: the double
// arithmetic is the reference's operation for operation.
struct PlaneAxes {
    AtlasAxis x, y;
    int width;
};

__device__ __forceinline__ long long nearest_index(const PlaneAxes& s, int x, int y) {
    const int xi = __ldg(s.x.weight + x) < 0.5f ? __ldg(s.x.index0 + x) : __ldg(s.x.index1 + x);
    const int yi = __ldg(s.y.weight + y) < 0.5f ? __ldg(s.y.index0 + y) : __ldg(s.y.index1 + y);
    return static_cast<long long>(yi) * s.width + xi;
}

__device__ __forceinline__ double bilinear_double(const double* __restrict__ src, const PlaneAxes& s, int x, int y,
                                                  bool preserve_negative) {
    const int x0 = __ldg(s.x.index0 + x), x1 = __ldg(s.x.index1 + x);
    const double wx = static_cast<double>(__ldg(s.x.weight + x));
    const int y0 = __ldg(s.y.index0 + y), y1 = __ldg(s.y.index1 + y);
    const double wy = static_cast<double>(__ldg(s.y.weight + y));
    const double* top = src + static_cast<long long>(y0) * s.width;
    const double* bottom = src + static_cast<long long>(y1) * s.width;
    auto ordinary = [preserve_negative](double v) { return preserve_negative && v < 0.0 ? 0.0 : v; };
    const double t = ordinary(__ldg(top + x0)) * (1.0 - wx) + ordinary(__ldg(top + x1)) * wx;
    const double b = ordinary(__ldg(bottom + x0)) * (1.0 - wx) + ordinary(__ldg(bottom + x1)) * wx;
    double value = t * (1.0 - wy) + b * wy;
    if (preserve_negative) {
        const double nearest = __ldg(src + nearest_index(s, x, y));
        if (nearest < 0.0) value = nearest;
    }
    return value;
}

// Double planes: 0 bailout, 1 transition (keeps negative markers), 2 phase,
// 3 de_x, 4 de_y, 5 test1, 6 test2; all but the bailout reset to 0 on
// interior samples.
__global__ void __launch_bounds__(256) atlas_planes_kernel(const AtlasLaunch a, const KfpPlaneSet primary,
                                                           const KfpPlaneSet secondary, const KfpPlaneOutputs out,
                                                           long long target_max_iter) {
    const PlaneAxes ps = a.full_child ? PlaneAxes{a.child_x, a.child_y, a.child_width}
                                      : PlaneAxes{a.parent_x, a.parent_y, a.parent_width};
    const PlaneAxes cs{a.child_x, a.child_y, a.child_width};
    const bool secondary_tile = a.use_child && !a.full_child;
    const long long pixels = static_cast<long long>(a.out_width) * a.out_height;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int y = static_cast<int>(i / a.out_width);
        const int x = static_cast<int>(i - static_cast<long long>(y) * a.out_width);
        const std::uint8_t flags = a.inside_out[i];
        const bool inside = flags & 1;
        const int cx = x - a.child_left, cy = y - a.child_top;
        const bool child_here = secondary_tile && in_child(a, cx, cy);
        const bool child_inside = flags & 2;
        const float alpha = child_here ? seam_alpha(a, cx, cy) : 0.0f;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (out.ints[k] == nullptr) continue;
            long long v = 0;
            if (primary.ints[k] != nullptr) v = inside ? target_max_iter : __ldg(primary.ints[k] + nearest_index(ps, x, y));
            if (child_here && secondary.ints[k] != nullptr) {
                v = child_inside ? target_max_iter : __ldg(secondary.ints[k] + nearest_index(cs, cx, cy));
            }
            out.ints[k][i] = v;
        }
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            if (out.doubles[k] == nullptr) continue;
            const bool preserve = k == 1, reset = k != 0;
            // Interior samples of the reset planes are 0 whatever the
            // interpolation gives, so their FP64 work is skipped.
            double v = 0.0;
            if (primary.doubles[k] != nullptr && !(inside && reset)) {
                v = bilinear_double(primary.doubles[k], ps, x, y, preserve);
            }
            if (child_here && secondary.doubles[k] != nullptr) {
                const double c = child_inside && reset ? 0.0 : bilinear_double(secondary.doubles[k], cs, cx, cy, preserve);
                if (primary.doubles[k] == nullptr) {
                    v = c;
                } else {
                    const double blended = v * (1.0 - static_cast<double>(alpha)) + c * static_cast<double>(alpha);
                    if (preserve) {
                        const double selected = alpha >= 0.5f ? c : v;
                        v = selected < 0.0 ? selected : blended;
                    } else {
                        v = blended;
                    }
                }
            }
            out.doubles[k][i] = v;
        }
    }
}

}  // namespace

cudaError_t launch_atlas_planes(const AtlasLaunch& a, const KfpPlaneSet& primary, const KfpPlaneSet& secondary,
                                const KfpPlaneOutputs& out, long long target_max_iter, cudaStream_t stream) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const long long pixels = static_cast<long long>(a.out_width) * a.out_height;
    long long blocks = (pixels + 255) / 256;
    if (blocks > static_cast<long long>(sms) * 8) blocks = static_cast<long long>(sms) * 8;
    atlas_planes_kernel<<<static_cast<unsigned>(blocks < 1 ? 1 : blocks), 256, 0, stream>>>(a, primary, secondary,
                                                                                            out, target_max_iter);
    return cudaGetLastError();
}

// Entries of each per-frame table: the bilinear axes the mode reads, the
// float edge ramps (interior-preserving modes) or the double alpha table
// (RGB composite); and the four axes' constants.
static void atlas_table_sizes(const AtlasLaunch& a, AtlasTables& t) {
    t.parent_x_size = a.full_child ? 0 : a.out_width;
    t.parent_y_size = a.full_child ? 0 : a.out_height;
    t.child_x_size = a.use_child ? (a.full_child ? a.out_width : a.child_visible_width) : 0;
    t.child_y_size = a.use_child ? (a.full_child ? a.out_height : a.child_visible_height) : 0;
    const bool ramps = a.feather >= 2 && a.mode != kAtlasRgb;
    t.edge_x_size = ramps ? a.child_visible_width : 0;
    t.edge_y_size = ramps ? a.child_visible_height : 0;
    t.alpha_size = a.feather >= 2 && a.mode == kAtlasRgb ? a.feather : 0;
    // Axis constants in the reference's operation order (fill_bilinear_axis:
    // zoom >= 1, crop = source * (1 / zoom), left = (source - crop) / 2,
    // step = crop / destination; the window form: crop = source / zoom).
    const int sources[4] = {a.parent_width, a.parent_height, a.child_width, a.child_height};
    const int sizes[4] = {t.parent_x_size, t.parent_y_size, t.child_x_size, t.child_y_size};
    for (int k = 0; k < 4; ++k) {
        AtlasAxisPlan& plan = t.plan[k];
        const double zoom = std::max(k < 2 ? a.parent_zoom : a.child_zoom, 1.0);
        const double source = static_cast<double>(sources[k]);
        plan.source = sources[k];
        plan.window = k >= 2 && a.mode == kAtlasKfpSurface;
        plan.crop = plan.window ? source / zoom : source * (1.0 / zoom);
        plan.left = (source - plan.crop) * 0.5;
        plan.span = static_cast<double>(sizes[k]);
        plan.step = sizes[k] > 0 ? plan.crop / static_cast<double>(sizes[k]) : 0.0;
    }
}

std::size_t atlas_table_bytes(const AtlasLaunch& a) {
    AtlasTables t{};
    atlas_table_sizes(a, t);
    const std::size_t axes = static_cast<std::size_t>(t.parent_x_size) + t.parent_y_size + t.child_x_size
        + t.child_y_size;
    // Fourteen tables, each padded to 256 bytes, then the exact-pass counter
    // and pixel list (one entry per output pixel at most).
    return axes * 12 + (static_cast<std::size_t>(t.edge_x_size) + t.edge_y_size) * 4
        + static_cast<std::size_t>(t.alpha_size) * 8 + 16 * 256 + 256
        + static_cast<std::size_t>(a.out_width) * a.out_height * 4;
}

namespace {

// Smallest float >= cap - bias: the exact interior threshold for float
// samples.
float interior_limit(int cap, double bias) {
    const double limit = static_cast<double>(cap) - bias;
    float f = static_cast<float>(limit);
    if (static_cast<double>(f) < limit) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

void split(double v, float& hi, float& lo) {
    hi = static_cast<float>(v);
    lo = static_cast<float>(v - static_cast<double>(hi));
}

// encode_render_value (renderer.cpp:119-121) on the host: the float
// nearest to value - bias (exact two-sum, halfway cases by the remainder).
float encode_host(double value, double bias) {
    const double hi = value - bias;
    const double v = hi - value;
    const double lo = (value - (hi - v)) + (-bias - v);
    const float f = static_cast<float>(hi);
    if (lo == 0.0 || !std::isfinite(hi)) return f;
    const float below = static_cast<double>(f) <= hi ? f : std::nextafter(f, -std::numeric_limits<float>::infinity());
    const float above = std::nextafter(below, std::numeric_limits<float>::infinity());
    if (hi != 0.5 * (static_cast<double>(below) + static_cast<double>(above))) return f;
    return lo > 0.0 ? above : below;
}

}  // namespace

cudaError_t launch_atlas(AtlasLaunch& a, void* tables, cudaStream_t stream) {
    a.parent_limit = interior_limit(a.parent_max_iter, a.parent_bias);
    a.child_limit = interior_limit(a.child_max_iter, a.child_bias);
    split(a.parent_bias, a.parent_bias_hi, a.parent_bias_lo);
    split(a.child_bias, a.child_bias_hi, a.child_bias_lo);
    a.output_bias_f = static_cast<float>(a.output_bias);
    a.output_bias_exact = static_cast<double>(a.output_bias_f) == a.output_bias;
    a.interior_value = a.mode == kAtlasKfpSurface || a.mode == kAtlasKfpPlanes
        ? encode_host(static_cast<double>(a.effective_iter), a.output_bias)
        : static_cast<float>(static_cast<double>(a.effective_iter) - a.output_bias);
    auto align = [](std::size_t v) { return (v + 255) / 256 * 256; };
    AtlasTables t{};
    atlas_table_sizes(a, t);
    char* base = static_cast<char*>(tables);
    std::size_t at = 0;
    auto take = [&](std::size_t bytes) {
        char* p = base + at;
        at += align(bytes);
        return p;
    };
    AtlasTables::Axis* axes[4] = {&t.parent_x, &t.parent_y, &t.child_x, &t.child_y};
    const int sizes[4] = {t.parent_x_size, t.parent_y_size, t.child_x_size, t.child_y_size};
    for (int k = 0; k < 4; ++k) {
        axes[k]->i0 = reinterpret_cast<int*>(take(sizes[k] * sizeof(int)));
        axes[k]->i1 = reinterpret_cast<int*>(take(sizes[k] * sizeof(int)));
        axes[k]->w = reinterpret_cast<float*>(take(sizes[k] * sizeof(float)));
    }
    t.edge_x = reinterpret_cast<float*>(take(t.edge_x_size * sizeof(float)));
    t.edge_y = reinterpret_cast<float*>(take(t.edge_y_size * sizeof(float)));
    t.alpha = reinterpret_cast<double*>(take(t.alpha_size * sizeof(double)));
    a.alpha = t.alpha;
    a.exact_count = reinterpret_cast<unsigned*>(take(sizeof(unsigned)));
    a.exact_pixels = reinterpret_cast<unsigned*>(take(static_cast<std::size_t>(a.out_width) * a.out_height * 4));
    a.parent_x = AtlasAxis{t.parent_x.i0, t.parent_x.i1, t.parent_x.w};
    a.parent_y = AtlasAxis{t.parent_y.i0, t.parent_y.i1, t.parent_y.w};
    a.child_x = AtlasAxis{t.child_x.i0, t.child_x.i1, t.child_x.w};
    a.child_y = AtlasAxis{t.child_y.i0, t.child_y.i1, t.child_y.w};
    a.edge_x = t.edge_x;
    a.edge_y = t.edge_y;

    const int entries = t.parent_x_size + t.parent_y_size + t.child_x_size + t.child_y_size + t.edge_x_size
        + t.edge_y_size + t.alpha_size;
    // Always launched: it also clears the exact-pass counter.
    atlas_axes_kernel<<<static_cast<unsigned>(entries > 0 ? (entries + 255) / 256 : 1), 256, 0, stream>>>(a, t);
    cudaError_t status = cudaGetLastError();
    if (status != cudaSuccess) return status;
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const unsigned quads_per_row = static_cast<unsigned>((a.out_width + 3) / 4);
    const unsigned total = quads_per_row * static_cast<unsigned>(a.out_height);
    // One quad per thread: blocks retire as they finish, so uneven pixels
    // (the seam band's second sample, the child rectangle) balance
    // themselves.
    long long blocks = (static_cast<long long>(total) + 255) / 256;
    const unsigned grid = static_cast<unsigned>(blocks < 1 ? 1 : blocks), exact_grid = static_cast<unsigned>(sms) * 2;
    // One instantiation per mode: each gets its own register allocation and
    // no per-pixel mode switch.
    switch (a.mode) {
#define FGB_ATLAS_MODE(M)                                                                    \
        case M:                                                                              \
            atlas_kernel<M><<<grid, 256, 0, stream>>>(a, quads_per_row, total);              \
            status = cudaGetLastError();                                                     \
            if (status != cudaSuccess) return status;                                        \
            atlas_exact_kernel<M><<<exact_grid, 256, 0, stream>>>(a);                         \
            return cudaGetLastError();
        FGB_ATLAS_MODE(kAtlasField)
        FGB_ATLAS_MODE(kAtlasAurora)
        FGB_ATLAS_MODE(kAtlasKfpSurface)
        FGB_ATLAS_MODE(kAtlasCropField)
        FGB_ATLAS_MODE(kAtlasRgb)
        FGB_ATLAS_MODE(kAtlasCropAurora)
        FGB_ATLAS_MODE(kAtlasKfpPlanes)
#undef FGB_ATLAS_MODE
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace fgb
