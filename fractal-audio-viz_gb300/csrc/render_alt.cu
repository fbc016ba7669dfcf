// Plain form for julia / burning-ship / tricorn: FP64-mantissa perturbation
// with the formula-aware real 2x2 linear BLA, one thread per pixel.
//
// Restates render_alternate_reference_impl and alternate_delta_step
// (renderer.cpp:11933-12448): the image series for Julia, the signed escape
// margin built on the MPFR margin of each reference step, block acceptance
// only when the endpoint stays inside (else an exact replay), the Burning
// Ship axis-crossing step in FloatExp components, the exact scaled formula
// step once the reference orbit ends, and the Jacobian carried for the
// analytic-DE plane.  Compiled with --fmad=false like the Mandelbrot plain
// form, so results match the reference release build bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device.h"

namespace fgb {
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
    const double origin = mode == 1 ? static_cast<double>(dimension / 2) : static_cast<double>(dimension - 1) / 2.0;
    return static_cast<double>(index) - origin;
}

__device__ __forceinline__ float nan_f() { return __int_as_float(0x7fc00000); }

__device__ __forceinline__ Sc ld_sc(const Sc* s) { return sc_make(__ldg(&s->re), __ldg(&s->im), __ldg(&s->e)); }
__device__ __forceinline__ Fe ld_fe(const Fe* f) { return fe_make(__ldg(&f->m), __ldg(&f->e)); }

__device__ float smooth_escape(int iteration, const Nrm& norm, double bias) {
    if (norm.m == 0.0) return static_cast<float>(static_cast<double>(iteration) - bias);
    const double log_mag = 0.5 * (log(norm.m) + static_cast<double>(norm.e) * kLogTwo);
    if (!(log_mag > 0.0) || !is_finite(log_mag)) return static_cast<float>(static_cast<double>(iteration) - bias);
    return static_cast<float>((static_cast<double>(iteration) - log(log_mag) / kLogTwo) - bias);
}

// Real Jacobian [xa xb; ya yb] of the pixel map (renderer.cpp:7912-8073).
struct Jac {
    Fe xa, xb, ya, yb;
};

__device__ Jac jac_identity() { return Jac{fe_from(1.0, 0), fe_zero(), fe_zero(), fe_from(1.0, 0)}; }

__device__ Jac jac_holomorphic(const Sc& d) {
    const Fe re = fe_from(d.re, d.e);
    const Fe im = fe_from(d.im, d.e);
    return Jac{re, fe_neg(im), im, re};
}

__device__ Jac jac_step(int formula, const Sc& total, const Jac& p, bool parameter_plane) {
    const Fe re = fe_from(total.re, total.e);
    const Fe im = fe_from(total.im, total.e);
    Fe m00, m01, m10, m11;
    if (formula == kFormulaTricorn) {
        m00 = fe_mul(re, 2.0);
        m01 = fe_mul(im, -2.0);
        m10 = fe_mul(im, -2.0);
        m11 = fe_mul(re, -2.0);
    } else if (formula == kFormulaBurningShip) {
        const Fe ar = fe_abs(re), ai = fe_abs(im);
        const double rs = re.m < 0.0 ? -1.0 : 1.0;
        const double is = im.m < 0.0 ? -1.0 : 1.0;
        m00 = fe_mul(ar, 2.0 * rs);
        m01 = fe_mul(ai, -2.0 * is);
        m10 = fe_mul(ai, 2.0 * rs);
        m11 = fe_mul(ar, 2.0 * is);
    } else {
        m00 = fe_mul(re, 2.0);
        m01 = fe_mul(im, -2.0);
        m10 = fe_mul(im, 2.0);
        m11 = fe_mul(re, 2.0);
    }
    const Fe one = parameter_plane ? fe_from(1.0, 0) : fe_zero();
    return Jac{fe_add(fe_add(fe_mul(m00, p.xa), fe_mul(m01, p.ya)), one),
               fe_add(fe_add(fe_mul(m00, p.xb), fe_mul(m01, p.yb)), fe_zero()),
               fe_add(fe_add(fe_mul(m10, p.xa), fe_mul(m11, p.ya)), fe_zero()),
               fe_add(fe_add(fe_mul(m10, p.xb), fe_mul(m11, p.yb)), one)};
}

__device__ Jac jac_bla(const AltStep* s, const Jac& p, bool parameter_plane) {
    Fe c[8];
    for (int k = 0; k < 8; ++k) c[k] = ld_fe(&s->c[k]);
    return Jac{fe_add(fe_add(fe_mul(c[0], p.xa), fe_mul(c[1], p.ya)), parameter_plane ? c[4] : fe_zero()),
               fe_add(fe_add(fe_mul(c[0], p.xb), fe_mul(c[1], p.yb)), parameter_plane ? c[5] : fe_zero()),
               fe_add(fe_add(fe_mul(c[2], p.xa), fe_mul(c[3], p.ya)), parameter_plane ? c[6] : fe_zero()),
               fe_add(fe_add(fe_mul(c[2], p.xb), fe_mul(c[3], p.yb)), parameter_plane ? c[7] : fe_zero())};
}

// render_plane_de_matrix (renderer.cpp:7936-7990).
__device__ bool de_matrix(const Sc& total, const Jac& j, const Fe& spacing, double& ox, double& oy) {
    const double mag = hypot(total.re, total.im);
    if (!(mag > 0.0) || !is_finite(mag)) return false;
    const double lm = log(mag) + static_cast<double>(total.e) * kLogTwo;
    if (!(lm > 0.0) || !is_finite(lm)) return false;
    const double ur = total.re / mag, ui = total.im / mag;
    const Fe sxa = fe_mul(j.xa, spacing), sxb = fe_mul(j.xb, spacing);
    const Fe sya = fe_mul(j.ya, spacing), syb = fe_mul(j.yb, spacing);
    const Fe dr = fe_add(fe_mul(sxa, ur), fe_mul(sya, ui));
    const Fe di = fe_add(fe_mul(sxb, ur), fe_mul(syb, ui));
    const Fe d2 = fe_add(fe_sqr(dr), fe_sqr(di));
    if (fe_is_zero(d2) || !fe_finite(d2)) return false;
    const Fe num = fe_from(mag * lm, total.e);
    const Fe rr = fe_div(fe_mul(num, dr), d2);
    const Fe ri = fe_div(fe_neg(fe_mul(num, di)), d2);
    ox = scale2(rr.m, rr.e);
    oy = scale2(ri.m, ri.e);
    return is_finite(ox) && is_finite(oy);
}

struct Planes {
    std::int64_t* iter;
    double *phase, *dex, *dey, *t1, *t2;
    __device__ void clear(long long i, int max_iter) const {
        iter[i] = max_iter;
        phase[i] = dex[i] = dey[i] = t1[i] = t2[i] = 0.0;
    }
    __device__ void escape(long long i, int raw, const Sc& total, const Nrm& test2, const Jac& j,
                           const Fe& spacing) const {
        iter[i] = raw;
        const double re = sc_re_d(total), im = sc_im_d(total);
        double ph = 0.0;
        if (is_finite(re) && is_finite(im)) {
            ph = atan2(im, re) / kTwoPi;
            ph -= floor(ph);
            if (!is_finite(ph)) ph = 0.0;
        }
        phase[i] = ph;
        double ox = 0.0, oy = 0.0;
        if (de_matrix(total, j, spacing, ox, oy)) {
            dex[i] = ox;
            dey[i] = oy;
        } else {
            dex[i] = 0.0;
            dey[i] = 0.0;
        }
        t1[i] = nrm_to_d(sc_norm2(total));
        t2[i] = nrm_to_d(test2);
    }
};

// Signed escape margin from the MPFR margin of step i (renderer.cpp:8427-8443).
__device__ Fe alt_margin(const AltParams& p, int i, const Sc& d) {
    const OrbitRec* r = p.orbit + i;
    const Fe m0 = ld_fe(&r->margin);
    const Fe zr = fe_make(__ldg(&r->parts.re.m), __ldg(&r->parts.re.e));
    const Fe zi = fe_make(__ldg(&r->parts.im.m), __ldg(&r->parts.im.e));
    const Fe cross = fe_mul(fe_add(fe_mul(zr, fe_from(d.re, d.e)), fe_mul(zi, fe_from(d.im, d.e))), 2.0);
    const Nrm dn = sc_norm2(d);
    return fe_add(fe_add(m0, cross), fe_make(dn.m, dn.e));
}

// alternate_delta_step (renderer.cpp:11933-12034).
__device__ Sc alt_step(const AltParams& p, int i, const Sc& d, const Sc& pd) {
    const Sc z = ld_sc(&p.orbit[i].z);
    if (p.formula == kFormulaTricorn) {
        const Sc zc = sc_conj(z), dcj = sc_conj(d);
        return sc_add(sc_twice(sc_mul(zc, dcj)), sc_add(sc_mul(dcj, dcj), pd));
    }
    if (p.formula == kFormulaBurningShip) {
        const Fe rr = fe_from(z.re, z.e), ri = fe_from(z.im, z.e);
        const Fe dr = fe_from(d.re, d.e), di = fe_from(d.im, d.e);
        const Fe ar = fe_abs(rr), ai = fe_abs(ri);
        const Fe tr = fe_add(rr, dr), ti = fe_add(ri, di);
        const bool cross_r = (fe_cmp(rr, fe_zero()) >= 0) != (fe_cmp(tr, fe_zero()) >= 0);
        const bool cross_i = (fe_cmp(ri, fe_zero()) >= 0) != (fe_cmp(ti, fe_zero()) >= 0);
        if (cross_r || cross_i) {
            const Fe atr = fe_abs(tr), ati = fe_abs(ti);
            const Sc zn = ld_sc(&p.orbit[i + 1].z);
            const Fe por = fe_sub(fe_from(p.parameter.re, p.parameter.e), fe_from(zn.re, zn.e));
            const Fe poi = fe_sub(fe_from(p.parameter.im, p.parameter.e), fe_from(zn.im, zn.e));
            const Fe nr = fe_add(fe_sub(fe_sqr(atr), fe_sqr(ati)), fe_add(por, fe_from(pd.re, pd.e)));
            const Fe ni = fe_add(fe_mul(fe_mul(atr, ati), 2.0), fe_add(poi, fe_from(pd.im, pd.e)));
            return sc_from_fe(nr, ni);
        }
        const double rs = rr.m < 0.0 ? -1.0 : 1.0;
        const double is = ri.m < 0.0 ? -1.0 : 1.0;
        const Fe lr = fe_sub(fe_mul(fe_mul(ar, dr), 2.0 * rs), fe_mul(fe_mul(ai, di), 2.0 * is));
        const Fe li = fe_add(fe_mul(fe_mul(ar, di), 2.0 * is), fe_mul(fe_mul(ai, dr), 2.0 * rs));
        const Fe sr = fe_sub(fe_sqr(dr), fe_sqr(di));
        const Fe si = fe_mul(fe_mul(dr, di), 2.0 * rs * is);
        return sc_from_fe(fe_add(fe_add(lr, sr), fe_from(pd.re, pd.e)), fe_add(fe_add(li, si), fe_from(pd.im, pd.e)));
    }
    return sc_add(sc_twice(sc_mul(z, d)), sc_add(sc_mul(d, d), pd));
}

// scaled_formula_step (renderer.cpp:11917-11931).
__device__ Sc formula_step(int formula, const Sc& v, const Sc& c) {
    if (formula == kFormulaBurningShip) {
        const Sc a = sc_make(fabs_(v.re), fabs_(v.im), v.e);
        return sc_add(sc_mul(a, a), c);
    }
    const Sc sq = formula == kFormulaTricorn ? sc_mul(sc_conj(v), sc_conj(v)) : sc_mul(v, v);
    return sc_add(sq, c);
}

// AlternateLinearBlaLevels::lookup (renderer.cpp:8536-8567).
__device__ const AltStep* alt_lookup(const AltParams& p, int start, const Fe& dn, const Fe& pn, int max_length) {
    if (p.alt_index.levels == 0 || start < p.alt_start || max_length <= 0 || !fe_finite(dn) || !fe_finite(pn)) {
        return nullptr;
    }
    const int offset = start - p.alt_start;
    if (offset < 0 || offset >= p.alt_index.count[0]) return nullptr;
    int top = 31 - __clz(max_length);
    top = top < p.alt_index.levels - 1 ? top : p.alt_index.levels - 1;
    // Only blocks of two or more steps are taken, and they start at even
    // offsets.  At one start the radii never grow with the level (a merge
    // keeps at most its first half's radius, times 1 - 2^-40; an unpaired
    // entry is copied), so a delta outside the two-step block's finite
    // radius is outside every longer block's too: one load settles the
    // common case of a delta too large for any block, with the same result
    // as the full top-down search.
    if (top < 1 || (offset & 1) != 0) return nullptr;
    if ((offset >> 1) < p.alt_index.count[1]) {
        const Fe r2 = ld_fe(&p.alt[p.alt_index.offset[1] + (offset >> 1)].r2);
        if (fe_finite(r2) && fe_cmp(dn, r2) >= 0) return nullptr;
    }
    for (int level = top; level >= 1; --level) {
        if ((offset & ((1 << level) - 1)) != 0) continue;
        const int index = offset >> level;
        if (index >= p.alt_index.count[level]) continue;
        const AltStep* s = p.alt + p.alt_index.offset[level] + index;
        const Fe r2 = ld_fe(&s->r2);
        if (__ldg(&s->len) > 1 && fe_finite(r2) && fe_cmp(dn, r2) < 0 && fe_cmp(pn, p.alt_input_radius2) <= 0) return s;
    }
    return nullptr;
}

__device__ Sc apply_alt(const AltStep* s, const Sc& d, const Sc& c) {
    const Fe dr = fe_from(d.re, d.e), di = fe_from(d.im, d.e);
    const Fe cr = fe_from(c.re, c.e), ci = fe_from(c.im, c.e);
    Fe k[8];
    for (int j = 0; j < 8; ++j) k[j] = ld_fe(&s->c[j]);
    const Fe rr = fe_add(fe_add(fe_mul(k[0], dr), fe_mul(k[1], di)), fe_add(fe_mul(k[4], cr), fe_mul(k[5], ci)));
    const Fe ri = fe_add(fe_add(fe_mul(k[2], dr), fe_mul(k[3], di)), fe_add(fe_mul(k[6], cr), fe_mul(k[7], ci)));
    return sc_from_fe(rr, ri);
}

// One pixel's state between steps, so a lane can park it and carry on
// later (the lane-refill queue below) or run it to the end at once.
template <bool WithPlanes>
struct AltLane {
    long long index;
    Sc dc, pd, delta, total, tortoise;
    Fe pn;
    Nrm total_norm, palette_norm;
    Jac jac;
    int ref, it, power, length, hits;
    unsigned ticks;
    bool ready;
};

__device__ __forceinline__ void alt_store(const AltParams& p, long long index, float out, std::uint32_t count) {
    p.out[index] = out;
    if (p.counts) p.counts[index] = count;
}

// Start pixel `index`: coordinates, Julia series jump, first escape test.
// Returns true when the pixel is finished (its outputs written).
template <bool WithPlanes>
__device__ __forceinline__ bool alt_begin(const AltParams& p, long long index, AltLane<WithPlanes>& s) {
    const int py = static_cast<int>(index / p.width);
    const int px = static_cast<int>(index - static_cast<long long>(py) * p.width);
    const Planes planes{p.p_iter, p.p_phase, p.p_dex, p.p_dey, p.p_t1, p.p_t2};
    if constexpr (WithPlanes) planes.clear(index, p.max_iter);
    const double xf = pixel_offset(px, p.width, p.coordinate_mode) / static_cast<double>(p.width);
    const double yf = -pixel_offset(py, p.height, p.coordinate_mode) / static_cast<double>(p.height);
    s.index = index;
    s.dc = p.points ? sc_make(p.points[index].re, p.points[index].im, p.points[index].e)
                    : sc_from_fe(fe_mul(p.view_width, xf), fe_mul(p.view_height, yf));
    const bool julia = p.formula == kFormulaJulia;
    s.pd = julia ? sc_zero() : s.dc;
    const Nrm pnorm = sc_norm2(s.pd);
    s.pn = fe_make(pnorm.m, pnorm.e);
    s.delta = s.dc;
    s.jac = jac_identity();
    s.ref = julia ? 0 : 1;
    s.it = julia ? 0 : 1;
    if (p.series_on && nrm_cmp(sc_norm2(s.dc), p.series_r2) <= 0) {
        Sc value = ld_sc(&p.series[p.series_terms - 1]);
        Sc poly = sc_zero();
        for (int k = p.series_terms - 1; k > 1; --k) {
            poly = sc_add(sc_mul(poly, s.dc), value);
            value = sc_add(sc_mul(value, s.dc), ld_sc(&p.series[k - 1]));
        }
        const Sc derivative = sc_add(sc_mul(poly, s.dc), value);
        s.delta = sc_mul(value, s.dc);
        if constexpr (WithPlanes) s.jac = jac_holomorphic(derivative);
        s.ref = p.series_iteration;
        s.it = p.series_iteration;
    }
    s.ticks = 0;
    s.total = sc_add(ld_sc(&p.orbit[s.ref].z), s.delta);
    s.total_norm = nrm_from_margin(alt_margin(p, s.ref, s.delta), p.escape_mode);
    s.palette_norm = WithPlanes ? sc_norm2(s.total) : nrm_make(0.0, 0);
    if (nrm_outside(s.total_norm, p.escape_mode)) {
        if constexpr (WithPlanes) {
            planes.escape(index, julia ? s.it : (s.it - 1 > 0 ? s.it - 1 : 0), s.total, nrm_make(0.0, 0), s.jac,
                          p.pixel_spacing);
        }
        alt_store(p, index, smooth_escape(s.it, s.total_norm, p.output_bias), static_cast<std::uint32_t>(s.it));
        return true;
    }
    s.tortoise = sc_zero();
    s.power = 1;
    s.length = 0;
    s.hits = 0;
    s.ready = false;
    return false;
}

// One turn of the per-pixel loop: a formula step past the orbit's end, a
// BLA block (or its exact replay), or one exact perturbation step with the
// escape and cycle tests.  Returns true when the pixel is finished.
template <bool WithPlanes>
__device__ __forceinline__ bool alt_advance(const AltParams& p, AltLane<WithPlanes>& s, unsigned long long deadline,
                            int max_block) {
    const Planes planes{p.p_iter, p.p_phase, p.p_dex, p.p_dey, p.p_t1, p.p_t2};
    const long long index = s.index;
    const bool julia = p.formula == kFormulaJulia;
    auto raw_iteration = [&](int n) { return julia ? n : (n - 1 > 0 ? n - 1 : 0); };
    if (s.it >= p.max_iter) {
        if constexpr (WithPlanes) planes.clear(index, p.max_iter);
        alt_store(p, index, static_cast<float>(static_cast<double>(p.max_iter) - p.output_bias),
                  static_cast<std::uint32_t>(p.max_iter));
        return true;
    }
    if (deadline && ((s.ticks++ & 255U) == 0U) && global_ns() >= deadline) {
        alt_store(p, index, nan_f(), 0u);
        return true;
    }
    const int next = s.ref + 1;
    if (next >= p.orbit_size) {
        const Sc parameter = julia ? p.parameter : sc_add(p.parameter, s.dc);
        const Nrm prev_palette = s.palette_norm;
        if constexpr (WithPlanes) s.jac = jac_step(p.formula, s.total, s.jac, !julia);
        s.total = formula_step(p.formula, s.total, parameter);
        ++s.it;
        s.total_norm = sc_norm2(s.total);
        if (nrm_outside(s.total_norm, p.escape_mode)) {
            if constexpr (WithPlanes) {
                planes.escape(index, raw_iteration(s.it), s.total, prev_palette, s.jac, p.pixel_spacing);
            }
            alt_store(p, index, smooth_escape(s.it, s.total_norm, p.output_bias), static_cast<std::uint32_t>(s.it));
            return true;
        }
        if constexpr (WithPlanes) s.palette_norm = sc_norm2(s.total);
        return false;
    }
    const Nrm dnorm = sc_norm2(s.delta);
    const int remaining = p.max_iter - s.it;
    const AltStep* step = !p.disable_bla
        ? alt_lookup(p, s.ref, fe_make(dnorm.m, dnorm.e), s.pn, max_block < remaining ? max_block : remaining)
        : nullptr;
    if (step != nullptr && s.ref + __ldg(&step->len) < p.orbit_size) {
        const int len = __ldg(&step->len);
        const int end = s.ref + len;
        const Sc cand = apply_alt(step, s.delta, s.pd);
        const Fe cmargin = alt_margin(p, end, cand);
        const Nrm cnorm = nrm_from_margin(cmargin, p.escape_mode);
        const Sc ctotal = sc_add(ld_sc(&p.orbit[end].z), cand);
        const bool bad = !sc_finite(cand) || !fe_finite(cmargin) || !sc_finite(ctotal)
            || fe_cmp(cmargin, fe_zero()) > 0 || nrm_cmp(cnorm, nrm_make(0.75, 2)) >= 0;
        if (!bad) {
            s.delta = cand;
            if constexpr (WithPlanes) s.jac = jac_bla(step, s.jac, !julia);
            s.ref = end;
            s.it += len;
            s.total = ctotal;
            s.total_norm = cnorm;
            if constexpr (WithPlanes) s.palette_norm = sc_norm2(s.total);
            return false;
        }
        for (int k = 0; k < len && s.it < p.max_iter; ++k) {
            const Nrm prev_palette = s.palette_norm;
            if constexpr (WithPlanes) {
                const Sc prior = sc_add(ld_sc(&p.orbit[s.ref].z), s.delta);
                s.jac = jac_step(p.formula, prior, s.jac, !julia);
            }
            s.delta = alt_step(p, s.ref, s.delta, s.pd);
            ++s.ref;
            ++s.it;
            if (!sc_finite(s.delta)) {
                alt_store(p, index, p.strict ? nan_f() : static_cast<float>(static_cast<double>(s.it) - p.output_bias),
                          p.strict ? 0u : static_cast<std::uint32_t>(s.it));
                return true;
            }
            const Fe margin = alt_margin(p, s.ref, s.delta);
            s.total_norm = nrm_from_margin(margin, p.escape_mode);
            s.total = sc_add(ld_sc(&p.orbit[s.ref].z), s.delta);
            if (fe_cmp(margin, fe_zero()) > 0 || nrm_outside(s.total_norm, p.escape_mode)) {
                if constexpr (WithPlanes) {
                    planes.escape(index, raw_iteration(s.it), s.total, prev_palette, s.jac, p.pixel_spacing);
                }
                alt_store(p, index, smooth_escape(s.it, s.total_norm, p.output_bias),
                          static_cast<std::uint32_t>(s.it));
                return true;
            }
            if constexpr (WithPlanes) s.palette_norm = sc_norm2(s.total);
        }
        return false;
    }
    const Nrm prev_palette = s.palette_norm;
    if constexpr (WithPlanes) {
        const Sc prior = sc_add(ld_sc(&p.orbit[s.ref].z), s.delta);
        s.jac = jac_step(p.formula, prior, s.jac, !julia);
    }
    s.delta = alt_step(p, s.ref, s.delta, s.pd);
    s.ref = next;
    ++s.it;
    if (!sc_finite(s.delta)) {
        alt_store(p, index, p.strict ? nan_f() : static_cast<float>(static_cast<double>(s.it) - p.output_bias),
                  p.strict ? 0u : static_cast<std::uint32_t>(s.it));
        return true;
    }
    const Fe margin = alt_margin(p, s.ref, s.delta);
    s.total_norm = nrm_from_margin(margin, p.escape_mode);
    s.total = sc_add(ld_sc(&p.orbit[s.ref].z), s.delta);
    if (fe_cmp(margin, fe_zero()) > 0 || nrm_outside(s.total_norm, p.escape_mode)) {
        if constexpr (WithPlanes) planes.escape(index, raw_iteration(s.it), s.total, prev_palette, s.jac, p.pixel_spacing);
        alt_store(p, index, smooth_escape(s.it, s.total_norm, p.output_bias), static_cast<std::uint32_t>(s.it));
        return true;
    }
    if constexpr (WithPlanes) s.palette_norm = sc_norm2(s.total);
    // Bounded cycle confirmed three times (non-strict renders only).
    if (p.cycle && s.it >= 2048 && (s.it & 31) == 0 && nrm_cmp(s.total_norm, nrm_make(0.75, 2)) < 0) {
        if (!s.ready) {
            s.tortoise = s.total;
            s.power = 1;
            s.length = 0;
            s.hits = 0;
            s.ready = true;
        } else {
            const Nrm dist = sc_norm2(sc_sub(s.total, s.tortoise));
            const int scale_e = s.total_norm.e > 0 ? s.total_norm.e : 0;
            if (dist.m == 0.0 || dist.e <= scale_e - 78) {
                if (++s.hits >= 3) {
                    if constexpr (WithPlanes) planes.clear(index, p.max_iter);
                    alt_store(p, index, static_cast<float>(static_cast<double>(p.max_iter) - p.output_bias),
                              static_cast<std::uint32_t>(p.max_iter));
                    return true;
                }
            } else {
                s.hits = 0;
            }
            if (++s.length >= s.power) {
                s.tortoise = s.total;
                s.power = s.power * 2 < (1 << 20) ? s.power * 2 : (1 << 20);
                s.length = 0;
            }
        }
    }
    return false;
}

__device__ __forceinline__ int alt_max_block(const AltParams& p) {
    return p.max_lin_len < 2 ? 2 : (p.max_lin_len > kMaxSafeLinearBlaLength ? kMaxSafeLinearBlaLength : p.max_lin_len);
}

__device__ __forceinline__ unsigned long long alt_deadline(const AltParams& p) {
    return p.deadline_base ? *p.deadline_base + p.budget_ns : 0ull;
}

// One thread per pixel (point lists).
template <bool WithPlanes>
__global__ void __launch_bounds__(128) alt_kernel(const AltParams p) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const long long index = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (index >= pixels) return;
    const unsigned long long deadline = alt_deadline(p);
    const int max_block = alt_max_block(p);
    AltLane<WithPlanes> s;
    bool done = alt_begin<WithPlanes>(p, index, s);
    while (!done) done = alt_advance<WithPlanes>(p, s, deadline, max_block);
}

// Lane-refill queue for Julia fields.  GB300 issues an FP64 warp
// instruction at the same cost whatever the number of active lanes, and a
// Julia view (the dynamic plane, crossed by the Julia set) mixes a few very
// long orbits with many short ones: 99 % of pixels under 100 iterations,
// some at the cap, so a warp that keeps a lane per pixel runs mostly empty.
// Persistent warps instead keep every lane busy: each lane holds one
// pixel's state, the warp runs kAltRound turns of the loop, and lanes whose
// pixel finished take new ones (claimed for the whole warp with one atomic
// on the launch's counter) once at least kAltRefill of them wait, or when
// none has work left.  Parameter-plane views (burning ship, tricorn) have
// escape times close together; there lanes that start together stay on the
// same branch of the loop, and one thread per pixel is faster (measured:
// 1.47 s against 2.23 s for a 3840x2160 burning-ship field at 1e94).
constexpr int kAltRound = 16;
constexpr int kAltRefill = 8;

template <bool WithPlanes>
__global__ void __launch_bounds__(128) alt_queue_kernel(const AltParams p, unsigned long long* counter) {
    constexpr unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const unsigned long long deadline = alt_deadline(p);
    const int max_block = alt_max_block(p);
    AltLane<WithPlanes> s;
    bool have = false;
    bool drained = false;
    while (true) {
        if (!drained) {
            unsigned need = __ballot_sync(kFull, !have);
            while (__popc(need) >= kAltRefill) {
                const unsigned n = static_cast<unsigned>(__popc(need));
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(counter, static_cast<unsigned long long>(n));
                base = __shfl_sync(kFull, base, 0);
                if (!have) {
                    const long long index = static_cast<long long>(base) + __popc(need & ((1u << lane) - 1u));
                    if (index < pixels) have = !alt_begin<WithPlanes>(p, index, s);
                }
                if (static_cast<long long>(base) + n >= pixels) {
                    drained = true;
                    break;
                }
                need = __ballot_sync(kFull, !have);
            }
        }
        if (!__any_sync(kFull, have)) {
            if (drained) break;
            continue;
        }
        // One copy of the loop body: unrolled, the turns would multiply the
        // kernel's code and miss in the instruction cache.
#pragma unroll 1
        for (int k = 0; k < kAltRound; ++k) {
            if (have && alt_advance<WithPlanes>(p, s, deadline, max_block)) have = false;
        }
    }
}

template <bool WithPlanes>
int alt_queue_blocks() {
    static int blocks = 0;
    if (blocks == 0) {
        int per_sm = 0, sms = 0, device = 0;
        cudaGetDevice(&device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, alt_queue_kernel<WithPlanes>, 128, 0);
        blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    return blocks;
}

}  // namespace

cudaError_t launch_plain_alternate(const AltParams& p, bool planes, bool stats, unsigned long long* queue_counter,
                                   cudaStream_t stream) {
    (void)stats;
    const long long pixels = static_cast<long long>(p.width) * p.height;
    if (queue_counter != nullptr && p.points == nullptr && p.formula == kFormulaJulia) {
        const cudaError_t cleared = cudaMemsetAsync(queue_counter, 0, sizeof(unsigned long long), stream);
        if (cleared != cudaSuccess) return cleared;
        // A field smaller than the persistent grid needs no more warps than pixels / 32.
        const long long needed = (pixels + 127) / 128;
        if (planes) {
            const long long grid = std::min<long long>(alt_queue_blocks<true>(), needed);
            alt_queue_kernel<true><<<static_cast<unsigned>(grid), 128, 0, stream>>>(p, queue_counter);
        } else {
            const long long grid = std::min<long long>(alt_queue_blocks<false>(), needed);
            alt_queue_kernel<false><<<static_cast<unsigned>(grid), 128, 0, stream>>>(p, queue_counter);
        }
        return cudaGetLastError();
    }
    const dim3 grid(static_cast<unsigned>((pixels + 127) / 128));
    if (planes) {
        alt_kernel<true><<<grid, 128, 0, stream>>>(p);
    } else {
        alt_kernel<false><<<grid, 128, 0, stream>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace fgb
