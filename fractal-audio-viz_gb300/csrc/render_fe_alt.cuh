// Floatexp form for julia / burning-ship / tricorn: FP32-mantissa /
// int32-exponent perturbation with the formula-aware real 2x2 linear BLA.
//
// The decision structure is the plain form's (render_alt.cu, itself
// render_alternate_reference_impl and alternate_delta_step,
// renderer.cpp:11933-12448): the image series for Julia, the signed escape
// margin built on each reference step's MPFR margin, block acceptance only
// when the endpoint stays inside (else an exact replay), the Burning Ship
// axis-crossing step, the exact formula step once the reference orbit ends,
// and the Jacobian carried for the analytic distance estimate when the
// caller asked for derivative planes.  The arithmetic is FP32 floatexp; the
// tables come from the FP64 ones converted once per handle.  Only strict
// renders without cycle detection or time budget take this form.
#pragma once

#include "render_fe.cuh"

namespace fgb {
namespace fxk {
namespace {

__device__ __forceinline__ R1e ld_r1e(const R1e* p) { return r_make(__ldg(&p->m), __ldg(&p->e)); }

// Signed escape margin |Z_i + d|^2 - R^2 = m_i + 2 Re(conj(Z_i) d) + |d|^2
// with m_i = |Z_i|^2 - R^2 from the MPFR orbit (renderer.cpp:8427-8443).
__device__ R1e alt_margin(const FxParams& p, int i, const F2e& d) {
    const FxOrbitRec* r = p.orbit + i;
    const R1e m0 = r_make(__ldg(&r->z2.m), __ldg(&r->z2.e));
    if (is_zero(d)) return m0;
    const F2e z = ld_f2e(&r->z);
    const R1e cross = is_zero(z) ? r_zero() : r_norm(2.0f * fmaf(z.x, d.x, z.y * d.y), z.e + d.e);
    const N1e dn = norm2(d);
    return r_add(r_add(m0, cross), r_make(dn.m, dn.e));
}

// R^2 + margin as a norm (negative rounding residue clamps to zero).
__device__ __forceinline__ N1e norm_from_margin(const R1e& margin, int mode) {
    const N1e limit = bailout(mode);
    const R1e n = r_add(r_make(limit.m, limit.e), margin);
    return n.m > 0.0f ? n_from_r(n) : n_norm(0.0f, 0);
}

// alternate_delta_step (renderer.cpp:11933-12034) in FP32 floatexp.
__device__ F2e alt_step(const FxParams& p, int i, const F2e& d, const F2e& pd) {
    const F2e z = ld_f2e(&p.orbit[i].z);
    if (p.formula == kFormulaTricorn) {
        const F2e zc = conj(z), dcj = conj(d);
        return add(twice(mul(zc, dcj)), add(mul(dcj, dcj), pd));
    }
    if (p.formula == kFormulaBurningShip) {
        const R1e rr = r_re(z), ri = r_im(z);
        const R1e dr = r_re(d), di = r_im(d);
        const R1e ar = r_abs(rr), ai = r_abs(ri);
        const R1e tr = r_add(rr, dr), ti = r_add(ri, di);
        const bool cross_r = (r_sign(rr) >= 0) != (r_sign(tr) >= 0);
        const bool cross_i = (r_sign(ri) >= 0) != (r_sign(ti) >= 0);
        if (cross_r || cross_i) {
            // The pixel's orbit crosses an axis: step it through |.| exactly
            // and re-subtract the next reference value.
            const R1e atr = r_abs(tr), ati = r_abs(ti);
            const F2e zn = ld_f2e(&p.orbit[i + 1].z);
            const R1e por = r_sub(r_re(p.parameter), r_re(zn));
            const R1e poi = r_sub(r_im(p.parameter), r_im(zn));
            const R1e nr = r_add(r_sub(r_mul(atr, atr), r_mul(ati, ati)), r_add(por, r_re(pd)));
            const R1e ni = r_add(r_scale(r_mul(atr, ati), 2.0f), r_add(poi, r_im(pd)));
            return from_r(nr, ni);
        }
        const float rs = rr.m < 0.0f ? -1.0f : 1.0f;
        const float is = ri.m < 0.0f ? -1.0f : 1.0f;
        const R1e lr = r_sub(r_scale(r_mul(ar, dr), 2.0f * rs), r_scale(r_mul(ai, di), 2.0f * is));
        const R1e li = r_add(r_scale(r_mul(ar, di), 2.0f * is), r_scale(r_mul(ai, dr), 2.0f * rs));
        const R1e sr = r_sub(r_mul(dr, dr), r_mul(di, di));
        const R1e si = r_scale(r_mul(dr, di), 2.0f * rs * is);
        return from_r(r_add(r_add(lr, sr), r_re(pd)), r_add(r_add(li, si), r_im(pd)));
    }
    return add(twice(mul(z, d)), add(mul(d, d), pd));
}

// scaled_formula_step (renderer.cpp:11917-11931): the exact map once the
// reference orbit has ended.
__device__ F2e formula_step(int formula, const F2e& v, const F2e& c) {
    if (formula == kFormulaBurningShip) {
        const F2e a = make(fabsf(v.x), fabsf(v.y), v.e);
        return add(mul(a, a), c);
    }
    const F2e sq = formula == kFormulaTricorn ? mul(conj(v), conj(v)) : mul(v, v);
    return add(sq, c);
}

// AlternateLinearBlaLevels::lookup (renderer.cpp:8536-8567).
__device__ const FxAltStep* alt_lookup(const FxParams& p, int start, const N1e& dn, const N1e& pn, int max_length) {
    const LevelIndex* index = p.linear_index;
    const int levels = __ldg(&index->levels);
    if (levels == 0 || start < p.alt_start || max_length <= 0 || dn.e == 0x3fffffff || pn.e == 0x3fffffff) {
        return nullptr;
    }
    const int offset = start - p.alt_start;
    if (offset < 0 || offset >= __ldg(&index->count[0])) return nullptr;
    int top = 31 - __clz(max_length);
    top = top < levels - 1 ? top : levels - 1;
    // One load settles a delta too large for any block: radii never grow
    // with the level at one start (see the FP64 lookup), and the FP32 radii
    // are the FP64 ones rounded to nearest, which keeps their order.
    if (top < 1 || (offset & 1) != 0) return nullptr;
    if ((offset >> 1) < __ldg(&index->count[1])) {
        const N1e r2 = ld_n1e(&p.alt[__ldg(&index->offset[1]) + (offset >> 1)].r2);
        if (r2.e != 0x3fffffff && n_cmp(dn, r2) >= 0) return nullptr;
    }
    for (int level = top; level >= 1; --level) {
        if ((offset & ((1 << level) - 1)) != 0) continue;
        const int at = offset >> level;
        if (at >= __ldg(&index->count[level])) continue;
        const FxAltStep* s = p.alt + __ldg(&index->offset[level]) + at;
        const N1e r2 = ld_n1e(&s->r2);
        if (__ldg(&s->len) > 1 && r2.e != 0x3fffffff && n_cmp(dn, r2) < 0 && n_cmp(pn, p.alt_input_radius2) <= 0) {
            return s;
        }
    }
    return nullptr;
}

__device__ F2e apply_alt(const FxAltStep* s, const F2e& d, const F2e& c) {
    const R1e dr = r_re(d), di = r_im(d), cr = r_re(c), ci = r_im(c);
    R1e k[8];
    for (int j = 0; j < 8; ++j) k[j] = ld_r1e(&s->c[j]);
    const R1e rr = r_add(r_add(r_mul(k[0], dr), r_mul(k[1], di)), r_add(r_mul(k[4], cr), r_mul(k[5], ci)));
    const R1e ri = r_add(r_add(r_mul(k[2], dr), r_mul(k[3], di)), r_add(r_mul(k[6], cr), r_mul(k[7], ci)));
    return from_r(rr, ri);
}

// Real Jacobian [xa xb; ya yb] of the pixel map (renderer.cpp:7912-8073).
struct Jac {
    R1e xa, xb, ya, yb;
};

__device__ __forceinline__ Jac jac_identity() { return Jac{r_make(0.5f, 1), r_zero(), r_zero(), r_make(0.5f, 1)}; }

__device__ __forceinline__ Jac jac_holomorphic(const F2e& d) {
    const R1e re = r_re(d), im = r_im(d);
    return Jac{re, r_neg(im), im, re};
}

__device__ Jac jac_step(int formula, const F2e& total, const Jac& p, bool parameter_plane) {
    const R1e re = r_re(total), im = r_im(total);
    R1e m00, m01, m10, m11;
    if (formula == kFormulaTricorn) {
        m00 = r_scale(re, 2.0f);
        m01 = r_scale(im, -2.0f);
        m10 = r_scale(im, -2.0f);
        m11 = r_scale(re, -2.0f);
    } else if (formula == kFormulaBurningShip) {
        const R1e ar = r_abs(re), ai = r_abs(im);
        const float rs = re.m < 0.0f ? -1.0f : 1.0f;
        const float is = im.m < 0.0f ? -1.0f : 1.0f;
        m00 = r_scale(ar, 2.0f * rs);
        m01 = r_scale(ai, -2.0f * is);
        m10 = r_scale(ai, 2.0f * rs);
        m11 = r_scale(ar, 2.0f * is);
    } else {
        m00 = r_scale(re, 2.0f);
        m01 = r_scale(im, -2.0f);
        m10 = r_scale(im, 2.0f);
        m11 = r_scale(re, 2.0f);
    }
    const R1e one = parameter_plane ? r_make(0.5f, 1) : r_zero();
    return Jac{r_add(r_add(r_mul(m00, p.xa), r_mul(m01, p.ya)), one), r_add(r_mul(m00, p.xb), r_mul(m01, p.yb)),
               r_add(r_mul(m10, p.xa), r_mul(m11, p.ya)), r_add(r_add(r_mul(m10, p.xb), r_mul(m11, p.yb)), one)};
}

__device__ Jac jac_bla(const FxAltStep* s, const Jac& p, bool parameter_plane) {
    R1e c[8];
    for (int k = 0; k < 8; ++k) c[k] = ld_r1e(&s->c[k]);
    return Jac{r_add(r_add(r_mul(c[0], p.xa), r_mul(c[1], p.ya)), parameter_plane ? c[4] : r_zero()),
               r_add(r_add(r_mul(c[0], p.xb), r_mul(c[1], p.yb)), parameter_plane ? c[5] : r_zero()),
               r_add(r_add(r_mul(c[2], p.xa), r_mul(c[3], p.ya)), parameter_plane ? c[6] : r_zero()),
               r_add(r_add(r_mul(c[2], p.xb), r_mul(c[3], p.yb)), parameter_plane ? c[7] : r_zero())};
}

// render_plane_de_matrix (renderer.cpp:7936-7990).
__device__ void de_matrix(const F2e& total, const Jac& j, const N1e& spacing, float& ox, float& oy) {
    ox = 0.0f;
    oy = 0.0f;
    if (is_zero(total) || !finite(total)) return;
    const float mag = hypotf(total.x, total.y);
    const float lm = __logf(mag) + static_cast<float>(total.e) * kLn2;
    if (!(lm > 0.0f) || !isfinite(lm)) return;
    const R1e ur = r_norm(total.x / mag, 0), ui = r_norm(total.y / mag, 0);
    const R1e s = r_make(spacing.m, spacing.e);
    const R1e sxa = r_mul(j.xa, s), sxb = r_mul(j.xb, s), sya = r_mul(j.ya, s), syb = r_mul(j.yb, s);
    const R1e dr = r_add(r_mul(sxa, ur), r_mul(sya, ui));
    const R1e di = r_add(r_mul(sxb, ur), r_mul(syb, ui));
    const R1e d2 = r_add(r_mul(dr, dr), r_mul(di, di));
    if (d2.m == 0.0f || !r_finite(d2)) return;
    const float num = mag * lm;
    const float rx = ldexpf_fast(num * dr.m / d2.m, total.e + dr.e - d2.e);
    const float ry = ldexpf_fast(-num * di.m / d2.m, total.e + di.e - d2.e);
    if (isfinite(rx) && isfinite(ry)) {
        ox = rx;
        oy = ry;
    }
}

template <bool Planes>
__device__ __noinline__ PixelOut alt_pixel(const FxParams& p, int px, int py) {
    const float xf = axis_offset(px, p.width, p.coordinate_mode) / static_cast<float>(p.width);
    const float yf = -axis_offset(py, p.height, p.coordinate_mode) / static_cast<float>(p.height);
    const F2e dx = norm(p.view_width.x * xf, 0.0f, p.view_width.e);
    const F2e dy = norm(p.view_height.x * yf, 0.0f, p.view_height.e);
    const F2e dc = add(make(dx.x, 0.0f, dx.e), make(0.0f, dy.x, dy.e));
    const bool julia = p.formula == kFormulaJulia;
    const F2e pd = julia ? zero() : dc;
    const N1e pn = norm2(pd);
    F2e delta = dc;
    Jac jac = jac_identity();
    int ref = julia ? 0 : 1;
    int it = julia ? 0 : 1;
    if (p.series_on && n_cmp(norm2(dc), p.series_r2) <= 0) {
        F2e value = ld_f2e(&p.series[p.series_terms - 1]);
        F2e poly = zero();
        for (int k = p.series_terms - 1; k > 1; --k) {
            if constexpr (Planes) poly = add(mul(poly, dc), value);
            value = add(mul(value, dc), ld_f2e(&p.series[k - 1]));
        }
        if constexpr (Planes) jac = jac_holomorphic(add(mul(poly, dc), value));
        delta = mul(value, dc);
        ref = p.series_iteration;
        it = p.series_iteration;
    }
    const bool strict = p.strict != 0;
    const N1e three = N1e{0.75f, 2};
    auto escape_out = [&](int n, const N1e& norm_value, const F2e& total) {
        PixelOut r = out_of(smooth_from_norm(n, norm_value, p.output_bias), static_cast<std::uint32_t>(n));
        if constexpr (Planes) de_matrix(total, jac, p.pixel_spacing, r.de_x, r.de_y);
        return r;
    };
    auto unresolved = [&](int n) {
        return strict ? out_of(nan32(), 0u) : out_of(static_cast<float>(n) - p.output_bias, static_cast<std::uint32_t>(n));
    };
    F2e total = add(ld_f2e(&p.orbit[ref].z), delta);
    N1e total_norm = norm_from_margin(alt_margin(p, ref, delta), p.escape_mode);
    const N1e limit = bailout(p.escape_mode);
    if (n_cmp(total_norm, limit) > 0) return escape_out(it, total_norm, total);
    const int max_block = p.max_lin_len < 2 ? 2 : (p.max_lin_len > kMaxSafeLinearBlaLength ? kMaxSafeLinearBlaLength
                                                                                          : p.max_lin_len);
    while (it < p.max_iter) {
        const int next = ref + 1;
        if (next >= p.orbit_size) {
            const F2e parameter = julia ? p.parameter : add(p.parameter, dc);
            if constexpr (Planes) jac = jac_step(p.formula, total, jac, !julia);
            total = formula_step(p.formula, total, parameter);
            ++it;
            total_norm = norm2(total);
            if (n_cmp(total_norm, limit) > 0) return escape_out(it, total_norm, total);
            continue;
        }
        const N1e dnorm = norm2(delta);
        const int remaining = p.max_iter - it;
        const FxAltStep* step = !p.disable_bla
            ? alt_lookup(p, ref, dnorm, pn, max_block < remaining ? max_block : remaining)
            : nullptr;
        if (step != nullptr && ref + __ldg(&step->len) < p.orbit_size) {
            const int len = __ldg(&step->len);
            const int end = ref + len;
            const F2e cand = apply_alt(step, delta, pd);
            const R1e cmargin = alt_margin(p, end, cand);
            const N1e cnorm = norm_from_margin(cmargin, p.escape_mode);
            const F2e ctotal = add(ld_f2e(&p.orbit[end].z), cand);
            const bool bad = !finite(cand) || !r_finite(cmargin) || !finite(ctotal) || cmargin.m > 0.0f
                || n_cmp(cnorm, three) >= 0;
            if (!bad) {
                delta = cand;
                if constexpr (Planes) jac = jac_bla(step, jac, !julia);
                ref = end;
                it += len;
                total = ctotal;
                total_norm = cnorm;
                continue;
            }
            for (int k = 0; k < len && it < p.max_iter; ++k) {
                if constexpr (Planes) jac = jac_step(p.formula, add(ld_f2e(&p.orbit[ref].z), delta), jac, !julia);
                delta = alt_step(p, ref, delta, pd);
                ++ref;
                ++it;
                if (!finite(delta)) return unresolved(it);
                const R1e margin = alt_margin(p, ref, delta);
                total_norm = norm_from_margin(margin, p.escape_mode);
                total = add(ld_f2e(&p.orbit[ref].z), delta);
                if (margin.m > 0.0f || n_cmp(total_norm, limit) > 0) return escape_out(it, total_norm, total);
            }
            continue;
        }
        if constexpr (Planes) jac = jac_step(p.formula, total, jac, !julia);
        delta = alt_step(p, ref, delta, pd);
        ref = next;
        ++it;
        if (!finite(delta)) return unresolved(it);
        const R1e margin = alt_margin(p, ref, delta);
        total_norm = norm_from_margin(margin, p.escape_mode);
        total = add(ld_f2e(&p.orbit[ref].z), delta);
        if (margin.m > 0.0f || n_cmp(total_norm, limit) > 0) return escape_out(it, total_norm, total);
    }
    return out_of(static_cast<float>(p.max_iter) - p.output_bias, static_cast<std::uint32_t>(p.max_iter));
}

// Every field kind of the floatexp form: Mandelbrot (deep or shallow mode)
// or another formula, with or without derivative planes.
__device__ __forceinline__ PixelOut field_pixel(const FxParams& p, int px, int py) {
    if (p.formula == kFormulaMandelbrot) return p.de_x ? floatexp_pixel<true>(p, px, py) : floatexp_pixel<false>(p, px, py);
    return p.de_x ? alt_pixel<true>(p, px, py) : alt_pixel<false>(p, px, py);
}

// Renders one pixel and stores every output the field asks for.
__device__ __forceinline__ void render_pixel(const FxParams& p, int px, int py) {
    const PixelOut r = field_pixel(p, px, py);
    const long long local = static_cast<long long>(py) * p.width + px;
    p.out[local] = r.value;
    if (p.counts) p.counts[local] = r.count;
    if (p.de_x) {
        p.de_x[local] = static_cast<double>(r.de_x);
        p.de_y[local] = static_cast<double>(r.de_y);
    }
}

// The pixel's count alone (probe samples).
__device__ __forceinline__ std::uint32_t pixel_count(const FxParams& p, int px, int py) {
    return p.formula == kFormulaMandelbrot ? floatexp_pixel<false>(p, px, py).count : alt_pixel<false>(p, px, py).count;
}

}  // namespace
}  // namespace fxk
}  // namespace fgb
