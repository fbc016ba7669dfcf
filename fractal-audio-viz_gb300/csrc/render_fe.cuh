// Floatexp form (included by render_fe.cu): deep Mandelbrot perturbation with FP32-mantissa / int32-exponent
// deltas, one thread per pixel, plus the shallow mode (plain FP32 perturbation below 1e12).
//
// The decision structure is the plain form's (render_bla_impl,
// renderer.cpp:12673-13583): image-series jump, glitch sentinel, escape,
// rebasing, map_end continuation, cubic/linear BLA with endpoint replay and
// the plain tail once |delta|^2 > 2^-90 and no BLA block applies.  The
// arithmetic is FP32: floatexp (floatexp32.h) while deltas are tiny, plain
// float in the tail.  FP64 stays in the host-side table construction (BLA
// coefficient merging, validity radii) and the orbit downcast; the tables are
// converted once per handle.  Per-field agreement with the FP64 form is
// measured by the bench (count mismatch fraction) and by
// tests/test_gpu_floatexp.py.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device.h"

namespace fgb {
namespace fxk {
namespace {

using namespace f32x;

constexpr float kLn2 = 0.693147180559945309f;
constexpr float kInvLn2 = 1.442695040888963407f;

__device__ __forceinline__ float nan32() { return __int_as_float(0x7fc00000); }

__device__ __forceinline__ float axis_offset(int index, int dimension, int mode) {
    const float origin = mode == 1 ? static_cast<float>(dimension / 2) : static_cast<float>(dimension - 1) * 0.5f;
    return static_cast<float>(index) - origin;
}

__device__ __forceinline__ N1e bailout(int mode) {
    N1e r;
    if (mode == 1) {
        r.m = 0.7450580596923828f;  // 1e8 = 0.745... * 2^27
        r.e = 27;
    } else {
        r.m = 0.5f;
        r.e = 3;
    }
    return r;
}

__device__ __forceinline__ F2e ld_f2e(const F2e* p) { return make(__ldg(&p->x), __ldg(&p->y), __ldg(&p->e)); }
__device__ __forceinline__ N1e ld_n1e(const N1e* p) {
    N1e r;
    r.m = __ldg(&p->m);
    r.e = __ldg(&p->e);
    return r;
}

// Smooth escape value n - log2(ln|z|) from a squared norm (renderer.cpp:8170-8181).
__device__ __forceinline__ float smooth_from_norm(int iteration, const N1e& n, float bias) {
    const float log_mag = 0.5f * (__logf(n.m) + static_cast<float>(n.e) * kLn2);
    if (!(log_mag > 0.0f) || !isfinite(log_mag)) return static_cast<float>(iteration) - bias;
    return (static_cast<float>(iteration) - __logf(log_mag) * kInvLn2) - bias;
}

// The reference forms the pixel norm as R^2 + ((|Z|^2 - R^2) + 2 Re(conj(Z) d)
// + |d|^2) in double (renderer.cpp:8374-8390), so its glitch sentinel and
// rebase test see |Z + d|^2 rounded to a multiple of the last place of R^2:
// 2^-51 for R^2 = 4, 2^-26 for R^2 = 1e8, and exact zero below half of it.
// Near a periodic reference (|Z| close to 0) that zero flags a glitch the
// exact norm would not.  This applies the same quantisation to the FP32 norm
// where it is coarser than the FP32 mantissa.
// Z_i (floatexp) and the record's norm / margin word in two 16-byte loads.
__device__ __forceinline__ void orbit_record(const FxOrbitRec* orbit, int i, F2e& z, N1e& z2) {
    const float4 lo = __ldg(reinterpret_cast<const float4*>(orbit + i));
    const int4 hi = __ldg(reinterpret_cast<const int4*>(orbit + i) + 1);
    z = make(lo.z, lo.w, hi.x);
    z2.m = __int_as_float(hi.y);
    z2.e = hi.z;
}

// A block's head (squared radius, length) in one 16-byte load.
template <typename Step>
__device__ __forceinline__ void block_head(const Step* s, N1e& r2, int& len) {
    const int4 h = __ldg(reinterpret_cast<const int4*>(s));
    r2.m = __int_as_float(h.x);
    r2.e = h.y;
    len = h.z;
}

// The plain-float orbit value Z_i in one 8-byte load (records are 32 bytes
// from a cudaMalloc base, so zr / zi sit 8-byte aligned).
__device__ __forceinline__ float2 orbit_float(const FxOrbitRec* orbit, int i) {
    return __ldg(reinterpret_cast<const float2*>(&orbit[i].zr));
}

__device__ __forceinline__ N1e reference_norm(const N1e& n, int mode) {
    const int place = mode == 1 ? -26 : -51;
    if (n.m == 0.0f || n.e >= place + 24) return n;
    const float units = rintf(ldexpf_fast(n.m, n.e - place));
    return n_norm(units, place);
}

// The aligned power-of-two lookup over a level index in device memory
// (BlaLevels::lookup, renderer.cpp:8645-8684): the longest block starting at
// `start` whose squared radius exceeds |d|^2.
template <typename Step>
__device__ const Step* find_block(const Step* table, const LevelIndex* index, int start, const N1e& dn,
                                  int max_length) {
    if (start <= 0 || max_length <= 0) return nullptr;
    const int levels = __ldg(&index->levels);
    if (levels == 0 || start > __ldg(&index->count[0])) return nullptr;
    int top = 31 - __clz(max_length);
    top = top < levels - 1 ? top : levels - 1;
    const int offset = start - 1;
    for (int level = top; level >= 1; --level) {
        if ((offset & ((1 << level) - 1)) != 0) continue;
        const int at = offset >> level;
        if (at >= __ldg(&index->count[level])) continue;
        const Step* c = table + __ldg(&index->offset[level]) + at;
        N1e r2;
        int len;
        block_head(c, r2, len);
        if (len > 1 && r2.e != 0x3fffffff && n_cmp(dn, r2) < 0) return c;
    }
    return nullptr;
}

__device__ __forceinline__ const FxCubic* find_cubic(const FxParams& p, int start, const N1e& dn, int max_length) {
    return find_block(p.cubic, p.cubic_index, start, dn, max_length);
}

__device__ __forceinline__ const FxLinear* find_linear(const FxParams& p, int start, const N1e& dn,
                                                       int max_length) {
    return find_block(p.linear, p.linear_index, start, dn, max_length);
}

// Cubic bivariate map in Horner form (renderer.cpp:8686-8730).  Not inlined:
// the pixel loop's hot code stays small enough for the instruction cache.
__device__ __noinline__ F2e apply_cubic(const FxCubic* s, const F2e& d, const F2e& c, int order) {
    const F2e k0 = ld_f2e(&s->c[0]);
    const F2e k1 = ld_f2e(&s->c[1]);
    if (order <= 1) return add(mul(k0, d), mul(k1, c));
    const F2e k2 = ld_f2e(&s->c[2]);
    const F2e k3 = ld_f2e(&s->c[3]);
    const F2e k4 = ld_f2e(&s->c[4]);
    if (order == 2) {
        return add(mul(d, add(k0, add(mul(k2, d), mul(k3, c)))), mul(c, add(k1, mul(k4, c))));
    }
    const F2e dcub = add(add(mul(ld_f2e(&s->c[5]), d), mul(ld_f2e(&s->c[6]), c)), k2);
    const F2e ccub = add(k3, mul(ld_f2e(&s->c[7]), c));
    const F2e din = add(k0, add(mul(d, dcub), mul(c, ccub)));
    const F2e cin = add(k1, mul(c, add(k4, mul(ld_f2e(&s->c[8]), c))));
    return add(mul(d, din), mul(c, cin));
}

struct PixelOut {
    float value;
    std::uint32_t count;
    float de_x;  // analytic distance estimate (derivative planes only)
    float de_y;
};

__device__ __forceinline__ PixelOut out_of(float value, std::uint32_t count) {
    return PixelOut{value, count, 0.0f, 0.0f};
}

__device__ __forceinline__ F2e one_f2e() { return make(0.5f, 0.0f, 1); }

// d(z^2 + c)/dc = 2 z dz/dc + 1 for the pixel's total z.
__device__ __forceinline__ F2e derivative_step(const F2e& total, const F2e& derivative) {
    return add(twice(mul(total, derivative)), one_f2e());
}

// render_plane_de (renderer.cpp:7844-7890) in FP32 floatexp: the distance
// estimate |z| ln|z| / (u conj(dz/dc) spacing) with u = z/|z|, as (re, im)
// in pixel-spacing units; zero where it is undefined.
__device__ void plane_de(const F2e& total, const F2e& derivative, const N1e& spacing, float& out_x,
                         float& out_y) {
    out_x = 0.0f;
    out_y = 0.0f;
    if (is_zero(total) || !finite(total) || is_zero(derivative) || !finite(derivative)) return;
    const float mag = hypotf(total.x, total.y);
    const float log_mag = __logf(mag) + static_cast<float>(total.e) * kLn2;
    if (!(log_mag > 0.0f) || !isfinite(log_mag)) return;
    const F2e unit = make(total.x / mag, total.y / mag, 0);
    const F2e den = mul(mul(unit, conj(derivative)), make(spacing.m, 0.0f, spacing.e));
    const float den2 = fmaf(den.x, den.x, den.y * den.y);
    if (!(den2 > 0.0f) || !isfinite(den2)) return;
    const float num = mag * log_mag;
    const int e = total.e - den.e;
    const float rx = ldexpf_fast(num * den.x / den2, e);
    const float ry = ldexpf_fast(-num * den.y / den2, e);
    if (isfinite(rx) && isfinite(ry)) {
        out_x = rx;
        out_y = ry;
    }
}

template <bool Planes>
__device__ __forceinline__ PixelOut escaped(float value, std::uint32_t count, const F2e& total, const F2e& derivative,
                                            const FxParams& p) {
    PixelOut r = out_of(value, count);
    if constexpr (Planes) plane_de(total, derivative, p.pixel_spacing, r.de_x, r.de_y);
    return r;
}

// apply_bla_series_derivative (renderer.cpp:8732-8795): the derivative with
// respect to c through a cubic block, given dd = dd/dc on entry.
__device__ __noinline__ F2e apply_cubic_derivative(const FxCubic* s, const F2e& d, const F2e& c, const F2e& dd, int order) {
    const F2e k0 = ld_f2e(&s->c[0]);
    const F2e k1 = ld_f2e(&s->c[1]);
    if (order <= 1) return add(mul(k0, dd), k1);
    const F2e k2 = ld_f2e(&s->c[2]);
    const F2e k3 = ld_f2e(&s->c[3]);
    const F2e k4 = ld_f2e(&s->c[4]);
    F2e pd = add(k0, add(twice(mul(k2, d)), mul(k3, c)));
    F2e pc = add(k1, add(mul(k3, d), twice(mul(k4, c))));
    if (order >= 3) {
        const F2e k5 = ld_f2e(&s->c[5]);
        const F2e k6 = ld_f2e(&s->c[6]);
        const F2e k7 = ld_f2e(&s->c[7]);
        const F2e k8 = ld_f2e(&s->c[8]);
        const F2e d2 = mul(d, d);
        const F2e c2 = mul(c, c);
        pd = add(pd, add(mul(add(twice(mul(k5, d)), mul(k5, d)), d), add(twice(mul(k6, mul(d, c))), mul(k7, c2))));
        pc = add(pc, add(mul(k6, d2), add(twice(mul(k7, mul(d, c))), mul(add(twice(mul(k8, c)), mul(k8, c)), c))));
    }
    return add(mul(pd, dd), pc);
}

// Plain-float tail (the FP32 counterpart of renderer.cpp:12451-12669).  It is
// the deep pixels' hot loop, so it is inlined into the pixel function: as a
// call it cost a stack frame's worth of register saves per pixel.
template <bool Planes>
__device__ __forceinline__ PixelOut float_tail(const FxParams& p, int iteration, int ref, const F2e& delta, const F2e& dc,
                               F2e derivative) {
    const float dcr = to_float_x(dc), dci = to_float_y(dc);
    float dr = to_float_x(delta), di = to_float_y(delta);
    const float escape2 = p.escape_mode == 1 ? 1.0e8f : 4.0f;
    const float safe2 = escape2 + 1.0e-7f;
    int steps = 0, rebases = 0;
    const bool strict = p.strict != 0;
    const PixelOut unresolved_out = out_of(nan32(), 0u);
    float2 z = orbit_float(p.orbit, ref);
    // The loop runs while iteration < max_iter and ref + 1 < orbit_size and
    // gives up on its 65537th step.  Between rebases ref and iteration
    // advance together, so the steps to the first of those bounds are known
    // up front: a run takes them with one counter, and the step that would
    // exceed the limit is not computed (its output needs only the count).
    while (true) {
        const int room = min(p.max_iter - iteration, p.orbit_size - 1 - ref);
        if (room <= 0) break;
        const int to_limit = 65537 - steps;
        const bool limited = room >= to_limit;
        const int run = limited ? to_limit - 1 : room;
        const float2* next = reinterpret_cast<const float2*>(p.orbit + ref + 1);
        constexpr int kStride = sizeof(FxOrbitRec) / sizeof(float2);
        // A step leaves the run on escape or overflow (a NaN or infinite
        // norm fails m2 <= escape2 as an escaping one does) or to rebase
        // (|Z + d| < |d|): one branch per step, sorted out after the loop.
        int k = 0;
        float tr = 0.0f, ti = 0.0f, m2 = 0.0f;
        bool left_run = false;
#pragma unroll 2
        for (; k < run; ++k) {
            if constexpr (Planes) derivative = derivative_step(norm(z.x + dr, z.y + di, 0), derivative);
            // d' = (2Z + d) d + dc, in FMA form as the shallow mode has it.
            const float ar = fmaf(2.0f, z.x, dr), ai = fmaf(2.0f, z.y, di);
            const float nr = fmaf(dr, ar, fmaf(-di, ai, dcr));
            const float ni = fmaf(2.0f, fmaf(z.x, di, dr * (z.y + di)), dci);
            dr = nr;
            di = ni;
            z = __ldg(next + k * kStride);
            tr = z.x + dr;
            ti = z.y + di;
            m2 = fmaf(tr, tr, ti * ti);
            if (!(m2 <= escape2) | (m2 < fmaf(dr, dr, di * di))) {
                left_run = true;
                break;
            }
        }
        if (left_run) {
            iteration += k + 1;
            if (!(m2 <= escape2)) {
                if (!isfinite(m2)) {
                    return strict ? unresolved_out
                                  : out_of(static_cast<float>(iteration) - p.output_bias,
                                           static_cast<std::uint32_t>(iteration));
                }
                const float mag = sqrtf(fmaxf(m2, safe2));
                return escaped<Planes>((static_cast<float>(iteration) - __logf(__logf(mag)) * kInvLn2) - p.output_bias,
                                       static_cast<std::uint32_t>(iteration), norm(tr, ti, 0), derivative, p);
            }
            dr = tr;
            di = ti;
            ref = 0;
            z = orbit_float(p.orbit, 0);
            if (++rebases > 64) {
                return strict ? unresolved_out
                              : out_of(static_cast<float>(iteration) - p.output_bias,
                                       static_cast<std::uint32_t>(iteration));
            }
            steps += k + 1;
            continue;
        }
        iteration += run;
        if (limited) {
            ++iteration;
            return strict ? unresolved_out
                          : out_of(static_cast<float>(iteration) - p.output_bias, static_cast<std::uint32_t>(iteration));
        }
        break;
    }
    if (iteration < p.max_iter) {
        return strict ? unresolved_out
                      : out_of(static_cast<float>(iteration) - p.output_bias, static_cast<std::uint32_t>(iteration));
    }
    return out_of(static_cast<float>(p.max_iter) - p.output_bias, static_cast<std::uint32_t>(p.max_iter));
}

// Direct recurrence from the total once the pixel has left the reference.
template <bool Planes>
__device__ __noinline__ PixelOut continue_direct(const FxParams& p, F2e total, int iteration, const F2e& dc, F2e derivative) {
    const F2e parameter = add(ld_f2e(&p.orbit[1].z), dc);
    const N1e limit = bailout(p.escape_mode);
    while (iteration < p.max_iter) {
        if constexpr (Planes) derivative = derivative_step(total, derivative);
        total = add(mul(total, total), parameter);
        ++iteration;
        const N1e n = norm2(total);
        if (n_cmp(n, limit) > 0) {
            return escaped<Planes>(smooth_from_norm(iteration, n, p.output_bias), static_cast<std::uint32_t>(iteration),
                                   total, derivative, p);
        }
    }
    return out_of(static_cast<float>(p.max_iter) - p.output_bias, static_cast<std::uint32_t>(p.max_iter));
}

// Shallow mode: a field above 1e-12 of view height renders by plain FP32
// perturbation against the reference orbit, z_n = Z_m + d, from d = 0 at
// iteration 0 (Z_0 = 0), rebasing to the orbit's start (d <- z, m <- 0)
// whenever |z| < |d| or the orbit's valid part ends, with no limit on the
// number of rebases.  The deltas' rounding error is relative to |d|, which
// starts at the pixel's offset from the centre, so the counts equal those
// of the FP64 direct iteration except where FP64 rounding itself decides
// them.  The step is d' = d (2Z + d) + dc written as
//   re: dr (2Zr + dr) - di (2Zi + di) + dcr
//   im: 2 (Zr di + dr (Zi + di)) + dci
// (6 FMA-pipe operations), then |Z + d|^2 for the escape and rebase tests.
template <bool Planes>
__device__ __noinline__ PixelOut shallow_pixel(const FxParams& p, int px, int py) {
    const float xf = axis_offset(px, p.width, p.coordinate_mode) / static_cast<float>(p.width);
    const float yf = -axis_offset(py, p.height, p.coordinate_mode) / static_cast<float>(p.height);
    const float dcr = ldexpf_fast(p.view_width.x * xf, p.view_width.e);
    const float dci = ldexpf_fast(p.view_height.x * yf, p.view_height.e);
    const PixelOut inside = out_of(static_cast<float>(p.max_iter) - p.output_bias,
                                   static_cast<std::uint32_t>(p.max_iter));
    if (p.interior_test) {
        // Main cardioid and period-2 bulb (renderer.cpp:10060-10066), taken
        // only with a margin far above the float error of c = centre + dc,
        // so a culled pixel is interior in FP64 as well; pixels near either
        // boundary are iterated (an interior pixel then reaches the cap).
        const float cx = p.centre_re + dcr, cy = p.centre_im + dci;
        const float xq = cx - 0.25f;
        const float q = fmaf(xq, xq, cy * cy);
        const bool cardioid = q * (q + xq) <= fmaf(0.25f * cy, cy, -1.0e-4f);
        const float xb = cx + 1.0f;
        const bool bulb = fmaf(xb, xb, cy * cy) <= 0.0625f - 1.0e-4f;
        if (cardioid || bulb) return inside;
    }
    const float escape2 = p.escape_mode == 1 ? 1.0e8f : 4.0f;
    const float safe2 = escape2 + 1.0e-7f;
    // Last orbit entry before the reference escapes (map_end) or ends; the
    // host guarantees orbit_size >= 2.
    const int valid = max(1, min(p.map_end, p.orbit_size - 1));
    const float2* orbit = reinterpret_cast<const float2*>(p.orbit);
    constexpr int kStride = sizeof(FxOrbitRec) / sizeof(float2);
    float dr = 0.0f, di = 0.0f;
    float zr = 0.0f, zi = 0.0f;  // Z_0
    F2e derivative = zero();
    // Runs from Z_0: each takes up to `valid` steps (the orbit's last usable
    // entry) or the iterations left, with one counter; a rebase (|Z + d| <
    // |d|, or the run reaching `valid`) starts the next run from Z_0.
    int done = 0;  // iterations completed
    while (done < p.max_iter) {
        const int run = min(valid, p.max_iter - done);
        int k = 1;
        bool rebase = false;
        for (; k <= run; ++k) {
            if constexpr (Planes) derivative = derivative_step(norm(zr + dr, zi + di, 0), derivative);
            const float ar = fmaf(2.0f, zr, dr), ai = fmaf(2.0f, zi, di);
            const float nr = fmaf(dr, ar, fmaf(-di, ai, dcr));
            const float ni = fmaf(2.0f, fmaf(zr, di, dr * (zi + di)), dci);
            dr = nr;
            di = ni;
            const float2 z = __ldg(orbit + static_cast<long long>(k) * kStride);
            zr = z.x;
            zi = z.y;
            const float tr = zr + dr, ti = zi + di;
            const float m2 = fmaf(tr, tr, ti * ti);
            if (m2 > escape2) {
                const int iteration = done + k;
                const float mag = sqrtf(fmaxf(m2, safe2));
                return escaped<Planes>((static_cast<float>(iteration) - __logf(__logf(mag)) * kInvLn2) - p.output_bias,
                                       static_cast<std::uint32_t>(iteration), norm(tr, ti, 0), derivative, p);
            }
            if (m2 < fmaf(dr, dr, di * di) || k == valid) {
                dr = tr;
                di = ti;
                zr = 0.0f;
                zi = 0.0f;
                rebase = true;
                break;
            }
        }
        done += rebase ? k : run;
    }
    return inside;
}

// One Mandelbrot pixel of the floatexp form; shared by the per-field kernel
// and the batched persistent queues.
template <bool Planes>
__device__ __noinline__ PixelOut floatexp_pixel(const FxParams& p, int px, int py) {
    if (p.shallow) return shallow_pixel<Planes>(p, px, py);
    const float xf = axis_offset(px, p.width, p.coordinate_mode) / static_cast<float>(p.width);
    const float yf = -axis_offset(py, p.height, p.coordinate_mode) / static_cast<float>(p.height);
    const F2e dx = norm(p.view_width.x * xf, 0.0f, p.view_width.e);
    const F2e dy = norm(p.view_height.x * yf, 0.0f, p.view_height.e);
    const F2e dc = add(make(dx.x, 0.0f, dx.e), make(0.0f, dy.x, dy.e));

    F2e delta = dc;
    F2e derivative = one_f2e();
    int ref = 1;
    int iteration = 1;
    if (p.series_on && n_cmp(norm2(dc), p.series_r2) <= 0) {
        if (p.series_scaled) {
            // Plain-float Horner on u = dc 2^-scale with the field's
            // prescaled coefficients (|u| <= 1), rescaled once at the end;
            // with planes the derivative sum_k k b_k u^(k-1) alongside.
            const FxSeriesScaled* sc = p.series_scaled;
            const int scale = __ldg(&sc->scale);
            const float ur = ldexpf_fast(p.view_width.x * xf, p.view_width.e - scale);
            const float ui = ldexpf_fast(p.view_height.x * yf, p.view_height.e - scale);
            const int terms = __ldg(&sc->terms);
            // Coefficient pairs in one 8-byte load each (the struct's pairs
            // are 8-byte aligned).
            const float2* b = reinterpret_cast<const float2*>(sc->b);
            const float2 top = __ldg(b + terms - 1);
            float vr = top.x;
            float vi = top.y;
            float wr = 0.0f, wi = 0.0f;  // derivative of the inner polynomial
#pragma unroll 4
            for (int k = terms - 1; k > 1; --k) {
                if constexpr (Planes) {
                    const float nwr = fmaf(wr, ur, fmaf(-wi, ui, vr));
                    const float nwi = fmaf(wr, ui, fmaf(wi, ur, vi));
                    wr = nwr;
                    wi = nwi;
                }
                const float2 bk = __ldg(b + k - 1);
                const float nr = fmaf(vr, ur, fmaf(-vi, ui, bk.x));
                const float ni = fmaf(vr, ui, fmaf(vi, ur, bk.y));
                vr = nr;
                vi = ni;
            }
            const int shift = __ldg(&sc->shift);
            delta = norm(vr * ur - vi * ui, vr * ui + vi * ur, shift);
            if constexpr (Planes) {
                // d/dc [v(u) u] 2^shift = (v + u v'(u)) 2^(shift - scale)
                derivative = norm(vr + (wr * ur - wi * ui), vi + (wr * ui + wi * ur), shift - scale);
            }
        } else {
            F2e value = ld_f2e(&p.series[p.series_terms - 1]);
            F2e poly = zero();
            for (int k = p.series_terms - 1; k > 1; --k) {
                if constexpr (Planes) poly = add(mul(poly, dc), value);
                value = add(mul(value, dc), ld_f2e(&p.series[k - 1]));
            }
            if constexpr (Planes) derivative = add(mul(poly, dc), value);
            delta = mul(value, dc);
        }
        ref = p.series_iteration;
        iteration = p.series_iteration;
    }
    const N1e limit = bailout(p.escape_mode);
    const N1e three = N1e{0.75f, 2};
    PixelOut result = out_of(static_cast<float>(p.max_iter) - p.output_bias, static_cast<std::uint32_t>(p.max_iter));
    bool have_total = false;
    F2e total = zero();
    N1e total_norm = n_norm(0.0f, 0);
    bool no_pixel_bla = false;
    int rebases = 0;
    while (iteration < p.max_iter) {
        if (ref < 0 || ref >= p.orbit_size) {
            result = out_of(static_cast<float>(iteration) - p.output_bias, static_cast<std::uint32_t>(iteration));
            break;
        }
        F2e z;
        N1e z2;
        orbit_record(p.orbit, ref, z, z2);
        if (!have_total) {
            total = add(z, delta);
            total_norm = reference_norm(norm2(total), p.escape_mode);
        }
        have_total = false;
        if (z2.m != 0.0f && z2.e != 0x3fffffff) {
            // Glitch when |Z + d|^2 < 1e-7 |Z|^2.
            const N1e bound = n_norm(z2.m * 1.0e-7f, z2.e);
            if (n_cmp(total_norm, bound) < 0) {
                if (p.allow_recovery && finite(total) && ++rebases <= 64) {
                    delta = total;
                    ref = 0;
                    continue;
                }
                result = out_of(nan32(), 0u);
                break;
            }
        }
        if (n_cmp(total_norm, limit) > 0) {
            result = escaped<Planes>(smooth_from_norm(iteration, total_norm, p.output_bias),
                                     static_cast<std::uint32_t>(iteration), total, derivative, p);
            break;
        }
        const N1e dn = norm2(delta);
        if (n_cmp(total_norm, dn) < 0) {
            if (++rebases > 64) {
                result = continue_direct<Planes>(p, total, iteration, dc, derivative);
                break;
            }
            delta = total;
            ref = 0;
            continue;
        }
        if (p.map_end > 1 && ref >= p.map_end) {
            result = continue_direct<Planes>(p, total, iteration, dc, derivative);
            break;
        }
        const int remaining = p.max_iter - iteration;
        const int order = p.approx_order >= 3 && dn.e < -115 ? (dn.e < -160 ? 1 : 2) : p.approx_order;
        const FxLinear* lin = nullptr;
        const FxCubic* cub = nullptr;
        const bool bla = !p.disable_bla && !no_pixel_bla;
        if (bla) {
            if (order <= 1) {
                lin = find_linear(p, ref, dn, p.max_lin_len < remaining ? p.max_lin_len : remaining);
            } else {
                cub = find_cubic(p, ref, dn, p.max_bla_len < remaining ? p.max_bla_len : remaining);
            }
        }
        const int length = lin ? __ldg(&lin->len) : (cub ? __ldg(&cub->len) : 0);
        if (bla && (length <= 0 || ref + length > p.max_iter) && dn.e > -90) {
            result = float_tail<Planes>(p, iteration, ref, delta, dc, derivative);
            break;
        }
        if (length > 0 && ref + length <= p.max_iter) {
            const F2e previous = delta;
            const F2e previous_derivative = derivative;
            delta = lin ? add(mul(ld_f2e(&lin->a), previous), mul(ld_f2e(&lin->b), dc))
                        : apply_cubic(cub, previous, dc, order);
            const F2e z_end = ld_f2e(&p.orbit[ref + length].z);
            const F2e end = add(z_end, delta);
            const N1e end_norm = reference_norm(norm2(end), p.escape_mode);
            if (!finite(delta) || !finite(end)) {
                delta = previous;
                no_pixel_bla = true;
                continue;
            }
            if (n_cmp(end_norm, three) >= 0) {
                // Replay the block exactly near escape.
                delta = previous;
                bool escaped_here = false;
                for (int k = 0; k < length && iteration < p.max_iter; ++k) {
                    const F2e zk = ld_f2e(&p.orbit[ref].z);
                    if constexpr (Planes) derivative = derivative_step(add(zk, delta), derivative);
                    delta = add(twice(mul(zk, delta)), add(mul(delta, delta), dc));
                    ++ref;
                    ++iteration;
                    total = add(ld_f2e(&p.orbit[ref].z), delta);
                    total_norm = reference_norm(norm2(total), p.escape_mode);
                    if (n_cmp(total_norm, limit) > 0) {
                        result = escaped<Planes>(smooth_from_norm(iteration, total_norm, p.output_bias),
                                                 static_cast<std::uint32_t>(iteration), total, derivative, p);
                        escaped_here = true;
                        break;
                    }
                }
                if (escaped_here) break;
                have_total = true;
            } else {
                if constexpr (Planes) {
                    derivative = lin ? add(mul(ld_f2e(&lin->a), previous_derivative), ld_f2e(&lin->b))
                                     : apply_cubic_derivative(cub, previous, dc, previous_derivative, order);
                }
                ref += length;
                iteration += length;
                total = end;
                total_norm = end_norm;
                have_total = true;
            }
            continue;
        }
        if constexpr (Planes) derivative = derivative_step(total, derivative);
        delta = add(twice(mul(z, delta)), add(mul(delta, delta), dc));
        ++ref;
        ++iteration;
    }
    return result;
}

}  // namespace
}  // namespace fxk
}  // namespace fgb
