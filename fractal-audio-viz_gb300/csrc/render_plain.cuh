// Plain form (included by render_plain_*.cu, one kernel variant each): FP64-mantissa / int32-exponent perturbation of one deep
// Mandelbrot field per launch, one thread per pixel.
//
// The per-pixel procedure restates render_bla_impl (renderer.cpp:12673-13583)
// and render_scaled_double_tail (:12451-12669): image-series jump, glitch
// sentinel, escape with signed margin, Brent cycle test (non-strict only),
// Zhuoran rebasing with the 64-rebase exact fallback, map_end direct
// continuation, cubic / linear / deep-linear BLA lookup with endpoint replay,
// plain-double tail, and the exact step d' = 2 Z d + d^2 + dc.  This file is
// compiled with --fmad=false so every double operation rounds exactly as the
// reference release build does; the derivative (analytic DE) is carried only
// when the caller asked for render planes, because nothing else reads it.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device.h"

namespace fgb {
namespace plain {
namespace {

using namespace fx;

constexpr double kTwoPi = 6.283185307179586476925286766559005768;
constexpr double kLogTwo = 0.693147180559945309417232121458176568;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ double pixel_offset(int index, int dimension, int mode) {
    const double origin = mode == 1 ? static_cast<double>(dimension / 2)
                                    : static_cast<double>(dimension - 1) / 2.0;
    return static_cast<double>(index) - origin;
}

__device__ __forceinline__ float encode(double value, double bias) {
    return static_cast<float>(value - bias);
}

__device__ __forceinline__ float nan_f() { return __int_as_float(0x7fc00000); }

// Local copies of the counters in the reference's RenderStats order.
struct Counters {
    unsigned long long v[kStatsSlots];
};

enum Slot {
    kPixels = 0, kLogical, kBlaBlocks, kLinearBlocks, kCubicBlocks, kExactSteps, kReplaySteps,
    kBlaRetries, kCycleInside, kDoubleTailPixels, kBlaDisabledPixels, kTailSteps, kMaxTailSteps,
    kTailRebases, kTailRebaseFallbacks, kMaxPixelIterations, kSeriesPixels, kSeriesJumps,
    kGlitchCount, kUnresolvedPixels, kDeadlineAborts, kSecondaryReferences, kRenderNs, kHist0
};

template <bool Stats>
struct StatSink {
    Counters c;
    __device__ void init() {
        if constexpr (Stats) {
#pragma unroll
            for (int i = 0; i < kStatsSlots; ++i) c.v[i] = 0;
        }
    }
    __device__ void add(int slot, unsigned long long n = 1) {
        if constexpr (Stats) c.v[slot] += n;
    }
    __device__ void max(int slot, unsigned long long n) {
        if constexpr (Stats) c.v[slot] = c.v[slot] > n ? c.v[slot] : n;
    }
    __device__ void bla_length(int length) {
        if constexpr (Stats) {
            if (length <= 0) return;
            int bucket = 0;
            unsigned int value = static_cast<unsigned int>(length);
            while (value > 1U && bucket < 15) {
                value >>= 1U;
                ++bucket;
            }
            c.v[kHist0 + bucket] += 1;
        }
    }
    // Warp-aggregate then one atomic per warp and slot.
    __device__ void flush(unsigned long long* out) {
        if constexpr (Stats) {
            const unsigned mask = __activemask();
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(mask) - 1;
            for (int i = 0; i < kStatsSlots; ++i) {
                unsigned long long value = c.v[i];
                const bool is_max = i == kMaxTailSteps || i == kMaxPixelIterations;
                for (int offset = 16; offset > 0; offset >>= 1) {
                    const unsigned long long other = __shfl_down_sync(mask, value, offset);
                    const bool valid = (lane + offset) < 32 && ((mask >> (lane + offset)) & 1u);
                    if (valid) value = is_max ? (value > other ? value : other) : value + other;
                }
                // Lanes below the leader are not in the mask; the leader holds
                // the sum of every active lane above it.
                if (lane == leader) {
                    if (is_max) {
                        atomicMax(out + i, value);
                    } else if (value) {
                        atomicAdd(out + i, value);
                    }
                }
            }
        }
    }
};

// ------------------------------------------------------------ planes
__device__ double plane_phase(const Sc& v) {
    const double re = sc_re_d(v);
    const double im = sc_im_d(v);
    if (!is_finite(re) || !is_finite(im)) return 0.0;
    double phase = atan2(im, re) / kTwoPi;
    phase -= floor(phase);
    return is_finite(phase) ? phase : 0.0;
}

// render_plane_de (renderer.cpp:7844-7890).
__device__ bool plane_de(const Sc& total, const Sc& derivative, const Fe& spacing, double& out_re,
                         double& out_im) {
    const double mag = hypot(total.re, total.im);
    if (!(mag > 0.0) || !is_finite(mag)) return false;
    const double log_mag = log(mag) + static_cast<double>(total.e) * kLogTwo;
    if (!(log_mag > 0.0) || !is_finite(log_mag)) return false;
    const double ur = total.re / mag;
    const double ui = total.im / mag;
    const Sc unit = sc_from_fe(fe_from(ur, 0), fe_from(ui, 0));
    const Sc spacing_c = sc_from_fe(spacing, fe_zero());
    const Sc den = sc_mul(unit, sc_mul(sc_conj(derivative), spacing_c));
    const double den2 = den.re * den.re + den.im * den.im;
    if (!(den2 > 0.0) || !is_finite(den2)) return false;
    Sc r = sc_make(mag * log_mag * den.re / den2, -mag * log_mag * den.im / den2,
                   sat_exp(static_cast<long long>(total.e) - den.e));
    sc_normalize(r);
    out_re = sc_re_d(r);
    out_im = sc_im_d(r);
    return is_finite(out_re) && is_finite(out_im);
}

struct PlaneOut {
    std::int64_t* iter;
    double* phase;
    double* dex;
    double* dey;
    double* t1;
    double* t2;

    __device__ void clear(long long i, int max_iter) const {
        iter[i] = max_iter;
        phase[i] = 0.0;
        dex[i] = 0.0;
        dey[i] = 0.0;
        t1[i] = 0.0;
        t2[i] = 0.0;
    }
    __device__ void escape(long long i, int raw, const Sc& total, const Nrm& test1, const Nrm& test2,
                           const Sc& derivative, const Fe& spacing) const {
        iter[i] = raw;
        phase[i] = plane_phase(total);
        double de_re = 0.0, de_im = 0.0;
        if (plane_de(total, derivative, spacing, de_re, de_im)) {
            dex[i] = de_re;
            dey[i] = de_im;
        } else {
            dex[i] = 0.0;
            dey[i] = 0.0;
        }
        t1[i] = nrm_to_d(test1);
        t2[i] = nrm_to_d(test2);
    }
};

__device__ __forceinline__ int kalles_raw(int iteration) { return iteration - 1 > 0 ? iteration - 1 : 0; }

// smooth_escape_value (renderer.cpp:8170-8181), evaluated in double.
__device__ float smooth_escape(int iteration, const Nrm& norm, double bias) {
    if (norm.m == 0.0) return encode(static_cast<double>(iteration), bias);
    const double log_mag = 0.5 * (log(norm.m) + static_cast<double>(norm.e) * kLogTwo);
    if (!(log_mag > 0.0) || !is_finite(log_mag)) return encode(static_cast<double>(iteration), bias);
    return encode(static_cast<double>(iteration) - log(log_mag) / kLogTwo, bias);
}

// ------------------------------------------------------------ BLA lookup
__device__ const CubicStep* lookup_cubic(const PlainParams& p, int start, const Fe& dn, int max_length) {
    if (start <= 0 || max_length <= 0 || !fe_finite(dn)) return nullptr;
    const int levels = p.cubic_index.levels;
    const int base = levels ? p.cubic_index.count[0] : 0;
    if (start > base) return nullptr;
    int highest = 31 - __clz(max_length);
    highest = highest < levels - 1 ? highest : levels - 1;
    const int offset = start - 1;
    for (int level = highest; level >= 0; --level) {
        if ((offset & ((1 << level) - 1)) != 0) continue;
        const int index = offset >> level;
        if (index >= p.cubic_index.count[level]) continue;
        const CubicStep* c = p.cubic + p.cubic_index.offset[level] + index;
        const int len = __ldg(&c->len);
        const Fe r2 = fe_make(__ldg(&c->r2.m), __ldg(&c->r2.e));
        if (len > 1 && fe_finite(r2) && fe_cmp(dn, r2) < 0) return c;
    }
    return nullptr;
}

__device__ const LinearStep* lookup_linear(const PlainParams& p, int start, const Fe& dn, int max_length) {
    if (start <= 0 || max_length <= 0 || !fe_finite(dn)) return nullptr;
    const int levels = p.linear_index.levels;
    const int base = levels ? p.linear_index.count[0] : 0;
    if (start > base) return nullptr;
    int highest = 31 - __clz(max_length);
    highest = highest < levels - 1 ? highest : levels - 1;
    const int offset = start - 1;
    for (int level = highest; level >= 0; --level) {
        if ((offset & ((1 << level) - 1)) != 0) continue;
        const int index = offset >> level;
        if (index >= p.linear_index.count[level]) continue;
        const LinearStep* c = p.linear + p.linear_index.offset[level] + index;
        const int len = __ldg(&c->len);
        const Fe r2 = fe_make(__ldg(&c->r2.m), __ldg(&c->r2.e));
        if (len > 1 && fe_finite(r2) && fe_cmp(dn, r2) < 0) return c;
    }
    return nullptr;
}

__device__ __forceinline__ Sc ld_sc(const Sc* s) { return sc_make(__ldg(&s->re), __ldg(&s->im), __ldg(&s->e)); }

// apply_bla_series (renderer.cpp:8686-8730).
__device__ Sc apply_cubic(const CubicStep* step, const Sc& d, const Sc& c, int order) {
    const Sc k0 = ld_sc(&step->c[0]);
    const Sc k1 = ld_sc(&step->c[1]);
    if (order <= 1) return sc_add(sc_mul(k0, d), sc_mul(k1, c));
    const Sc k2 = ld_sc(&step->c[2]);
    const Sc k3 = ld_sc(&step->c[3]);
    const Sc k4 = ld_sc(&step->c[4]);
    if (order == 2) {
        const Sc d_inner = sc_add(sc_mul(k2, d), sc_mul(k3, c));
        const Sc c_inner = sc_add(k1, sc_mul(k4, c));
        return sc_add(sc_mul(d, sc_add(k0, d_inner)), sc_mul(c, c_inner));
    }
    const Sc k5 = ld_sc(&step->c[5]);
    const Sc k6 = ld_sc(&step->c[6]);
    const Sc k7 = ld_sc(&step->c[7]);
    const Sc k8 = ld_sc(&step->c[8]);
    const Sc d_cubic = sc_add(sc_add(sc_mul(k5, d), sc_mul(k6, c)), k2);
    const Sc c_cubic = sc_add(k3, sc_mul(k7, c));
    const Sc d_inner = sc_add(k0, sc_add(sc_mul(d, d_cubic), sc_mul(c, c_cubic)));
    const Sc c_inner = sc_add(k1, sc_mul(c, sc_add(k4, sc_mul(k8, c))));
    return sc_add(sc_mul(d, d_inner), sc_mul(c, c_inner));
}

// apply_bla_series_derivative (renderer.cpp:8732-8795).
__device__ __noinline__ Sc apply_cubic_derivative(const CubicStep* step, const Sc& d, const Sc& c, const Sc& dd,
                                     int order) {
    const Sc k0 = ld_sc(&step->c[0]);
    const Sc k1 = ld_sc(&step->c[1]);
    if (order <= 1) return sc_add(sc_mul(k0, dd), k1);
    Sc pd = k0;
    Sc pc = k1;
    const Sc k2 = ld_sc(&step->c[2]);
    const Sc k3 = ld_sc(&step->c[3]);
    const Sc k4 = ld_sc(&step->c[4]);
    pd = sc_add(pd, sc_add(sc_twice(sc_mul(k2, d)), sc_mul(k3, c)));
    pc = sc_add(pc, sc_add(sc_mul(k3, d), sc_twice(sc_mul(k4, c))));
    if (order >= 3) {
        const Sc k5 = ld_sc(&step->c[5]);
        const Sc k6 = ld_sc(&step->c[6]);
        const Sc k7 = ld_sc(&step->c[7]);
        const Sc k8 = ld_sc(&step->c[8]);
        const Sc d2 = sc_mul(d, d);
        const Sc c2 = sc_mul(c, c);
        pd = sc_add(pd, sc_add(sc_mul(sc_add(sc_twice(sc_mul(k5, d)), sc_mul(k5, d)), d),
                               sc_add(sc_twice(sc_mul(k6, sc_mul(d, c))), sc_mul(k7, c2))));
        pc = sc_add(pc, sc_add(sc_mul(k6, d2),
                               sc_add(sc_twice(sc_mul(k7, sc_mul(d, c))),
                                      sc_mul(sc_add(sc_twice(sc_mul(k8, c)), sc_mul(k8, c)), c))));
    }
    return sc_add(sc_mul(pd, dd), pc);
}

struct OrbitView {
    const OrbitRec* r;
    __device__ Sc z(int i) const { return ld_sc(&r[i].z); }
    __device__ double zd_re(int i) const { return __ldg(&r[i].zd_re); }
    __device__ double zd_im(int i) const { return __ldg(&r[i].zd_im); }
    __device__ Fe glitch(int i) const { return fe_make(__ldg(&r[i].glitch.m), __ldg(&r[i].glitch.e)); }
    // Signed escape margin |Z_i + d|^2 - R^2 (renderer.cpp:8374-8390) with
    // the reference-only terms read from the record.
    __device__ Fe margin(int i, const Sc& d) const {
        const Fe pr = fe_make(__ldg(&r[i].parts.re.m), __ldg(&r[i].parts.re.e));
        const Fe pi = fe_make(__ldg(&r[i].parts.im.m), __ldg(&r[i].parts.im.e));
        const Fe m0 = fe_make(__ldg(&r[i].margin.m), __ldg(&r[i].margin.e));
        const Fe dr = fe_from(d.re, d.e);
        const Fe di = fe_from(d.im, d.e);
        const Fe cross = fe_mul(fe_add(fe_mul(pr, dr), fe_mul(pi, di)), 2.0);
        return fe_add(fe_add(m0, cross), fe_add(fe_sqr(dr), fe_sqr(di)));
    }
};

// Exact scaled recurrence from the reconstructed total once the pixel has
// left the compact reference (renderer.cpp:13053-13146 and 13155-13250).
template <bool Planes, bool Stats>
__device__ __noinline__ void exact_continuation(const PlainParams& p, const OrbitView& orbit, long long index,
                                   const Sc& dc, Sc total, Nrm total_norm, Sc derivative, int& iteration,
                                   StatSink<Stats>& st, unsigned& ticks, unsigned long long deadline_ns,
                                   float& out_value, std::uint32_t& out_count, bool& deadline,
                                   const PlaneOut& planes) {
    const Sc parameter = sc_add(orbit.z(1), dc);
    Sc tortoise = sc_zero();
    int power = 1, length = 0;
    bool ready = false;
    const int cycle_min = p.strict_cycle ? 2048 : 512;
    const int cycle_margin = p.strict_cycle ? 78 : 60;
    bool escaped = false;
    while (iteration < p.max_iter) {
        if (deadline_ns && ((ticks++ & 255U) == 0U) && global_ns() >= deadline_ns) {
            out_value = nan_f();
            out_count = 0;
            deadline = true;
            st.add(kDeadlineAborts);
            st.add(kUnresolvedPixels);
            return;
        }
        const Nrm prior = total_norm;
        if constexpr (Planes) derivative = sc_add(sc_twice(sc_mul(total, derivative)), sc_one());
        total = sc_add(sc_mul(total, total), parameter);
        ++iteration;
        st.add(kLogical);
        st.add(kExactSteps);
        total_norm = sc_norm2(total);
        if (nrm_outside(total_norm, p.escape_mode)) {
            out_value = smooth_escape(iteration, total_norm, p.output_bias);
            out_count = static_cast<std::uint32_t>(iteration);
            if constexpr (Planes) planes.escape(index, kalles_raw(iteration), total, total_norm, prior,
                                                derivative, p.pixel_spacing);
            escaped = true;
            break;
        }
        if (p.cycle) {
            if (iteration >= cycle_min && (iteration & 31) == 0 && nrm_cmp(total_norm, nrm_make(0.75, 2)) < 0) {
                if (!ready) {
                    tortoise = total;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    const Nrm dist = sc_norm2(sc_sub(total, tortoise));
                    const int scale_e = total_norm.e > 0 ? total_norm.e : 0;
                    if (dist.m == 0.0 || dist.e <= scale_e - cycle_margin) {
                        out_value = encode(static_cast<double>(p.max_iter), p.output_bias);
                        out_count = static_cast<std::uint32_t>(p.max_iter);
                        escaped = true;
                        break;
                    }
                    if (++length >= power) {
                        tortoise = total;
                        power = power * 2 < (1 << 20) ? power * 2 : (1 << 20);
                        length = 0;
                    }
                }
            }
        }
    }
    if (!escaped) {
        out_value = encode(static_cast<double>(p.max_iter), p.output_bias);
        out_count = static_cast<std::uint32_t>(p.max_iter);
    }
}

// render_scaled_double_tail (renderer.cpp:12451-12669).  Returns true when
// the tail was pathological (too many steps or rebases).
template <bool Planes, bool Stats>
__device__ __noinline__ bool double_tail(const PlainParams& p, const OrbitView& orbit, long long index, const Sc& dc,
                            int& iteration, int& ref, const Sc& delta_in, Sc& derivative,
                            const Nrm& initial_norm, StatSink<Stats>& st, unsigned& ticks,
                            unsigned long long deadline_ns, float& out_value, std::uint32_t& out_count, bool& deadline,
                            bool& unresolved, const PlaneOut& planes) {
    const int kMaxTailRebases = 64;
    const int kMaxTailSteps = 65536;
    const double dc_re = sc_re_d(dc);
    const double dc_im = scale2(dc.im, dc.e);
    const double escape2 = escape_r2_d(p.escape_mode);
    const double safe_escape2 = escape2 + 1.0e-7;
    double dr = sc_re_d(delta_in);
    double di = scale2(delta_in.im, delta_in.e);
    out_value = encode(static_cast<double>(p.max_iter), p.output_bias);
    out_count = static_cast<std::uint32_t>(p.max_iter);
    double tort_re = 0.0, tort_im = 0.0;
    int power = 1, length = 0, tail_steps = 0, tail_iterations = 0, tail_rebases = 0;
    Nrm previous = initial_norm;
    bool ready = false;
    const bool strict = p.strict != 0;
    while (iteration < p.max_iter && ref >= 0 && ref + 1 < p.orbit_size) {
        if (deadline_ns && ((ticks++ & 255U) == 0U) && global_ns() >= deadline_ns) {
            out_value = nan_f();
            out_count = 0;
            deadline = true;
            unresolved = true;
            st.add(kDeadlineAborts);
            st.add(kUnresolvedPixels);
            return false;
        }
        const double zr = orbit.zd_re(ref);
        const double zi = orbit.zd_im(ref);
        if constexpr (Planes) {
            Sc prior = sc_make(zr + dr, zi + di, 0);
            sc_normalize(prior);
            derivative = sc_add(sc_twice(sc_mul(prior, derivative)), sc_one());
        }
        const double lin_re = 2.0 * (zr * dr - zi * di);
        const double lin_im = 2.0 * (zr * di + zi * dr);
        const double sq_re = dr * dr - di * di;
        const double sq_im = 2.0 * dr * di;
        dr = lin_re + sq_re + dc_re;
        di = lin_im + sq_im + dc_im;
        ++ref;
        ++iteration;
        if (++tail_iterations > kMaxTailSteps) {
            st.add(kTailRebaseFallbacks);
            st.add(kUnresolvedPixels);
            unresolved = true;
            out_value = strict ? nan_f() : encode(static_cast<double>(iteration), p.output_bias);
            out_count = strict ? 0u : static_cast<std::uint32_t>(iteration);
            return true;
        }
        st.add(kLogical);
        st.add(kExactSteps);
        const double tr = orbit.zd_re(ref) + dr;
        const double ti = orbit.zd_im(ref) + di;
        const double mag2 = tr * tr + ti * ti;
        if (!is_finite(mag2)) {
            unresolved = true;
            st.add(kGlitchCount);
            st.add(kUnresolvedPixels);
            out_value = strict ? nan_f() : encode(static_cast<double>(iteration), p.output_bias);
            out_count = strict ? 0u : static_cast<std::uint32_t>(iteration);
            return false;
        }
        if (mag2 > escape2) {
            const double magnitude = sqrt(dmax(mag2, safe_escape2));
            out_value = static_cast<float>(
                (static_cast<double>(iteration) - log(log(magnitude)) / kLogTwo) - p.output_bias);
            out_count = static_cast<std::uint32_t>(iteration);
            if constexpr (Planes) {
                Sc escaped = sc_make(tr, ti, 0);
                sc_normalize(escaped);
                planes.escape(index, kalles_raw(iteration), escaped, nrm_from_d(mag2), previous, derivative,
                              p.pixel_spacing);
            }
            return false;
        }
        previous = nrm_from_d(mag2);
        const double dmag2 = dr * dr + di * di;
        ++tail_steps;
        if (p.cycle) {
            if (tail_steps >= 64 && (tail_steps & 31) == 0) {
                if (!ready) {
                    tort_re = tr;
                    tort_im = ti;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    const double cr = tr - tort_re;
                    const double ci = ti - tort_im;
                    const double dist2 = cr * cr + ci * ci;
                    const int cycle_min = p.strict_cycle ? 2048 : 512;
                    const double tol = p.strict_cycle ? 1.0e-24 : 1.0e-18;
                    if (iteration >= cycle_min && mag2 < 3.0 && dist2 <= tol * dmax(1.0, mag2)) {
                        if constexpr (Planes) planes.clear(index, p.max_iter);
                        return false;
                    }
                    if (++length >= power) {
                        tort_re = tr;
                        tort_im = ti;
                        power = power * 2 < (1 << 20) ? power * 2 : (1 << 20);
                        length = 0;
                    }
                }
            }
        }
        if (mag2 < dmag2) {
            dr = tr;
            di = ti;
            ref = 0;
            tail_steps = 0;
            ready = false;
            st.add(kTailRebases);
            if (++tail_rebases > kMaxTailRebases) {
                st.add(kTailRebaseFallbacks);
                st.add(kUnresolvedPixels);
                unresolved = true;
                out_value = strict ? nan_f() : encode(static_cast<double>(iteration), p.output_bias);
                out_count = strict ? 0u : static_cast<std::uint32_t>(iteration);
                if constexpr (Planes) planes.clear(index, p.max_iter);
                return true;
            }
        }
    }
    if (iteration < p.max_iter) {
        unresolved = true;
        st.add(kUnresolvedPixels);
        out_value = strict ? nan_f() : encode(static_cast<double>(iteration), p.output_bias);
        out_count = strict ? 0u : static_cast<std::uint32_t>(iteration);
        if constexpr (Planes) planes.clear(index, p.max_iter);
    }
    return false;
}

template <bool Planes, bool Stats>
__global__ void __launch_bounds__(128) plain_mandelbrot_kernel(const PlainParams p) {
    const long long total_pixels = static_cast<long long>(p.width) * p.height;
    const long long index = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (index >= total_pixels) return;
    const int py = static_cast<int>(index / p.width);
    const int px = static_cast<int>(index - static_cast<long long>(py) * p.width);
    const OrbitView orbit{p.orbit};
    const PlaneOut planes{p.p_iter, p.p_phase, p.p_dex, p.p_dey, p.p_t1, p.p_t2};
    StatSink<Stats> st;
    st.init();
    st.add(kPixels);

    // Pixel offsets (renderer.cpp:12764-12783): the view span times the
    // signed pixel-centre fraction, both in FloatExp.
    // A point render takes dc from its list (renderer.cpp:12838-12842).
    const double x_fraction = pixel_offset(px, p.width, p.coordinate_mode) / static_cast<double>(p.width);
    const double y_fraction = -pixel_offset(py, p.height, p.coordinate_mode) / static_cast<double>(p.height);
    const Sc dc = p.points ? sc_make(p.points[index].re, p.points[index].im, p.points[index].e)
                           : sc_from_fe(fe_mul(p.view_width, x_fraction), fe_mul(p.view_height, y_fraction));
    const unsigned long long deadline_ns = p.deadline_base ? *p.deadline_base + p.budget_ns : 0ull;
    if constexpr (Planes) planes.clear(index, p.max_iter);
    Sc delta = dc;
    Sc derivative = sc_one();
    int ref = 1;
    int iteration = 1;
    if (p.series_on && nrm_cmp(sc_norm2(dc), p.series_r2) <= 0) {
        // Horner evaluation of the image series (renderer.cpp:8594-8639).
        Sc value = ld_sc(&p.series[p.series_terms - 1]);
        Sc poly_derivative = sc_zero();
        for (int k = p.series_terms - 1; k > 1; --k) {
            if constexpr (Planes) poly_derivative = sc_add(sc_mul(poly_derivative, dc), value);
            value = sc_add(sc_mul(value, dc), ld_sc(&p.series[k - 1]));
        }
        if constexpr (Planes) derivative = sc_add(sc_mul(poly_derivative, dc), value);
        delta = sc_mul(value, dc);
        ref = p.series_iteration;
        iteration = p.series_iteration;
        st.add(kSeriesPixels);
        st.add(kSeriesJumps, static_cast<unsigned long long>(iteration));
    }

    float out_value = 0.0f;
    std::uint32_t out_count = 0;
    bool escaped = false;
    bool have_total = false;
    Sc total = sc_zero();
    Nrm total_norm = nrm_make(0.0, 0);
    Nrm prev_total_norm = nrm_make(0.0, 0);
    Fe margin = fe_zero();
    Sc tortoise = sc_zero();
    int power = 1, length = 0;
    bool ready = false;
    bool pixel_disable_bla = false;
    int rebases = 0;
    unsigned ticks = 0;
    bool timed_out = false;
    bool unresolved = false;
    const int cycle_min = p.strict_cycle ? 2048 : 512;
    const int cycle_margin = p.strict_cycle ? 78 : 60;

    while (iteration < p.max_iter) {
        if (deadline_ns && ((ticks++ & 255U) == 0U) && global_ns() >= deadline_ns) {
            out_value = nan_f();
            out_count = 0;
            timed_out = true;
            unresolved = true;
            st.add(kDeadlineAborts);
            st.add(kUnresolvedPixels);
            break;
        }
        if (ref < 0 || ref >= p.orbit_size) {
            out_value = encode(static_cast<double>(iteration), p.output_bias);
            out_count = static_cast<std::uint32_t>(iteration);
            if constexpr (Planes) planes.escape(index, kalles_raw(iteration), total, total_norm, prev_total_norm,
                                                derivative, p.pixel_spacing);
            escaped = true;
            break;
        }
        if (!have_total) {
            total = sc_add(orbit.z(ref), delta);
            margin = orbit.margin(ref, delta);
            total_norm = nrm_from_margin(margin, p.escape_mode);
        }
        have_total = false;
        // Glitch sentinel (renderer.cpp:12938-12988).
        const Fe glitch = orbit.glitch(ref);
        if (glitch.m != 0.0 && fe_cmp(fe_make(total_norm.m, total_norm.e), glitch) < 0) {
            st.add(kGlitchCount);
            if (p.exact_flags) {
                // Strict point renders repair the pixel exactly (MPFR, on
                // the host) before any rebase (renderer.cpp:12944-12966).
                p.exact_flags[index] = 1;
                out_value = nan_f();
                out_count = 0;
                escaped = true;  // finished by the repair, as in the reference
                break;
            }
            if (p.allow_recovery && sc_finite(total) && ++rebases <= 64) {
                delta = total;
                ref = 0;
                have_total = false;
                continue;
            }
            out_value = nan_f();
            out_count = 0;
            unresolved = true;
            st.add(kUnresolvedPixels);
            break;
        }
        if (nrm_outside(total_norm, p.escape_mode) || fe_cmp(margin, fe_zero()) > 0) {
            out_value = smooth_escape(iteration, total_norm, p.output_bias);
            out_count = static_cast<std::uint32_t>(iteration);
            if constexpr (Planes) planes.escape(index, kalles_raw(iteration), total, total_norm, prev_total_norm,
                                                derivative, p.pixel_spacing);
            escaped = true;
            break;
        }
        if (p.cycle) {
            if (iteration >= cycle_min && (iteration & 31) == 0 && nrm_cmp(total_norm, nrm_make(0.75, 2)) < 0) {
                if (!ready) {
                    tortoise = total;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    const Nrm dist = sc_norm2(sc_sub(total, tortoise));
                    const int scale_e = total_norm.e > 0 ? total_norm.e : 0;
                    if (dist.m == 0.0 || dist.e <= scale_e - cycle_margin) {
                        st.add(kCycleInside);
                        out_value = encode(static_cast<double>(p.max_iter), p.output_bias);
                        out_count = static_cast<std::uint32_t>(p.max_iter);
                        escaped = true;
                        break;
                    }
                    if (++length >= power) {
                        tortoise = total;
                        power = power * 2 < (1 << 20) ? power * 2 : (1 << 20);
                        length = 0;
                    }
                }
            }
        }
        // Rebase when |Z + d| < |d| (renderer.cpp:13047-13153).
        const Nrm delta_norm = sc_norm2(delta);
        if (nrm_cmp(total_norm, delta_norm) < 0) {
            if (++rebases > 64) {
                exact_continuation<Planes, Stats>(p, orbit, index, dc, total, total_norm, derivative,
                                                         iteration, st, ticks, deadline_ns, out_value,
                                                         out_count, timed_out, planes);
                if (timed_out) unresolved = true;
                escaped = !timed_out;
                break;
            }
            delta = total;
            ref = 0;
            continue;
        }
        if (p.map_end > 1 && ref >= p.map_end) {
            exact_continuation<Planes, Stats>(p, orbit, index, dc, total, total_norm, derivative,
                                                     iteration, st, ticks, deadline_ns, out_value, out_count,
                                                     timed_out, planes);
            if (timed_out) unresolved = true;
            escaped = !timed_out;
            break;
        }
        const Fe dn = fe_make(delta_norm.m, delta_norm.e);
        const int remaining = p.max_iter - iteration;
        const int order = p.approx_order >= 3 && delta_norm.e < -115 ? (delta_norm.e < -160 ? 1 : 2)
                                                                     : p.approx_order;
        const LinearStep* lin = nullptr;
        const CubicStep* cub = nullptr;
        const bool bla_allowed = !p.disable_bla && !pixel_disable_bla;
        if (bla_allowed) {
            if (order <= 1) {
                lin = lookup_linear(p, ref, dn, p.max_lin_len < remaining ? p.max_lin_len : remaining);
            } else {
                cub = lookup_cubic(p, ref, dn, p.max_bla_len < remaining ? p.max_bla_len : remaining);
            }
        }
        const int map_length = lin ? __ldg(&lin->len) : (cub ? __ldg(&cub->len) : 0);
        if (bla_allowed && (map_length <= 0 || ref + map_length > p.max_iter) && delta_norm.e > -90) {
            st.add(kDoubleTailPixels);
            const int tail_start = iteration;
            const bool pathological = double_tail<Planes, Stats>(
                p, orbit, index, dc, iteration, ref, delta, derivative, total_norm, st, ticks, deadline_ns,
                out_value, out_count, timed_out, unresolved, planes);
            if (timed_out || unresolved) break;
            const unsigned long long steps = iteration > tail_start ? iteration - tail_start : 0;
            st.add(kTailSteps, steps);
            st.max(kMaxTailSteps, steps);
            if (pathological) {
                delta = dc;
                if constexpr (Planes) derivative = sc_one();
                ref = 1;
                iteration = 1;
                have_total = false;
                pixel_disable_bla = true;
                continue;
            }
            escaped = true;
            break;
        }
        if (map_length > 0 && ref + map_length <= p.max_iter) {
            st.add(kBlaBlocks);
            st.add(lin ? kLinearBlocks : kCubicBlocks);
            st.add(kSeriesJumps);
            st.bla_length(map_length);
            const Sc prev_delta = delta;
            const Sc prev_derivative = derivative;
            const int prev_ref = ref;
            const int prev_iteration = iteration;
            if (lin) {
                const Sc a = ld_sc(&lin->a);
                const Sc b = ld_sc(&lin->b);
                delta = sc_add(sc_mul(a, prev_delta), sc_mul(b, dc));
                if constexpr (Planes) derivative = sc_add(sc_mul(a, prev_derivative), b);
            } else {
                delta = apply_cubic(cub, prev_delta, dc, order);
                if constexpr (Planes) derivative = apply_cubic_derivative(cub, prev_delta, dc, prev_derivative, order);
            }
            ref += map_length;
            iteration += map_length;
            const Sc endpoint = sc_add(orbit.z(ref), delta);
            const Fe end_margin = orbit.margin(ref, delta);
            const Nrm endpoint_norm = nrm_from_margin(end_margin, p.escape_mode);
            if (!sc_finite(delta) || !sc_finite(endpoint)) {
                delta = prev_delta;
                derivative = prev_derivative;
                ref = prev_ref;
                iteration = prev_iteration;
                st.add(kBlaRetries);
                if (!pixel_disable_bla) st.add(kBlaDisabledPixels);
                pixel_disable_bla = true;
                have_total = false;
                continue;
            }
            if (nrm_cmp(endpoint_norm, nrm_make(0.75, 2)) >= 0) {
                // Replay the block one exact step at a time near escape.
                delta = prev_delta;
                derivative = prev_derivative;
                ref = prev_ref;
                iteration = prev_iteration;
                Sc replay_total = sc_zero();
                Nrm replay_norm = nrm_make(0.0, 0);
                Fe replay_margin = fe_zero();
                bool retry = false;
                for (int k = 0; k < map_length && iteration < p.max_iter; ++k) {
                    if (deadline_ns && ((ticks++ & 255U) == 0U) && global_ns() >= deadline_ns) {
                        out_value = nan_f();
                        out_count = 0;
                        timed_out = true;
                        unresolved = true;
                        st.add(kDeadlineAborts);
                        st.add(kUnresolvedPixels);
                        break;
                    }
                    const Sc z = orbit.z(ref);
                    if constexpr (Planes) {
                        const Sc prior = sc_add(z, delta);
                        derivative = sc_add(sc_twice(sc_mul(prior, derivative)), sc_one());
                    }
                    delta = sc_add(sc_twice(sc_mul(z, delta)), sc_add(sc_mul(delta, delta), dc));
                    ++ref;
                    ++iteration;
                    st.add(kReplaySteps);
                    st.add(kLogical);
                    replay_total = sc_add(orbit.z(ref), delta);
                    replay_margin = orbit.margin(ref, delta);
                    replay_norm = nrm_from_margin(replay_margin, p.escape_mode);
                    if (!sc_finite(delta) || !sc_finite(replay_total)) {
                        retry = true;
                        break;
                    }
                    if (nrm_outside(replay_norm, p.escape_mode) || fe_cmp(replay_margin, fe_zero()) > 0) {
                        out_value = smooth_escape(iteration, replay_norm, p.output_bias);
                        out_count = static_cast<std::uint32_t>(iteration);
                        if constexpr (Planes) planes.escape(index, kalles_raw(iteration), replay_total, replay_norm,
                                                            total_norm, derivative, p.pixel_spacing);
                        escaped = true;
                        break;
                    }
                }
                if (timed_out || escaped) break;
                if (retry) {
                    delta = prev_delta;
                    derivative = prev_derivative;
                    ref = prev_ref;
                    iteration = prev_iteration;
                    st.add(kBlaRetries);
                    if (!pixel_disable_bla) st.add(kBlaDisabledPixels);
                    pixel_disable_bla = true;
                    have_total = false;
                    continue;
                }
                total = replay_total;
                total_norm = replay_norm;
                margin = replay_margin;
                prev_total_norm = total_norm;
                have_total = true;
            } else {
                total = endpoint;
                total_norm = endpoint_norm;
                margin = end_margin;
                prev_total_norm = total_norm;
                have_total = true;
                st.add(kLogical, static_cast<unsigned long long>(map_length));
            }
            continue;
        }
        // One exact perturbation step.
        const Sc z = orbit.z(ref);
        const Nrm prior_norm = total_norm;
        if constexpr (Planes) {
            const Sc prior = sc_add(z, delta);
            derivative = sc_add(sc_twice(sc_mul(prior, derivative)), sc_one());
        }
        delta = sc_add(sc_twice(sc_mul(z, delta)), sc_add(sc_mul(delta, delta), dc));
        ++ref;
        ++iteration;
        prev_total_norm = prior_norm;
        st.add(kLogical);
        st.add(kExactSteps);
    }
    if (!escaped && !timed_out && !unresolved) {
        out_value = encode(static_cast<double>(p.max_iter), p.output_bias);
        out_count = static_cast<std::uint32_t>(p.max_iter);
    }
    st.max(kMaxPixelIterations, static_cast<unsigned long long>(iteration > 0 ? iteration : 0));
    p.out[index] = out_value;
    if (p.counts) p.counts[index] = out_count;
    st.flush(p.stats);
}

}  // namespace
}  // namespace plain

template <bool Planes, bool Stats>
cudaError_t launch_plain_variant(const PlainParams& p, cudaStream_t stream) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const dim3 block(128);
    const dim3 grid(static_cast<unsigned>((pixels + 127) / 128));
    plain::plain_mandelbrot_kernel<Planes, Stats><<<grid, block, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace fgb
