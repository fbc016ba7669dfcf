// BLA table arithmetic shared by the host builder and the GPU builder.
//
// One definition of every table formula, compiled for both sides without
// floating-point contraction, so the GPU-built hierarchies are bit-identical
// to the host-built ones (and to the reference's, renderer.cpp:11336-11869).
#pragma once

#include "reference.h"
#include "scaled.h"

namespace fgb {

struct BuilderCubic {
    fx::Fec c[9];  // A B C D E F G H I
    fx::Fe r2;
    int len;
    int pad;
};

struct BuilderLinear {
    fx::Fec a;
    fx::Fec b;
    fx::Fe r2;
    int len;
    int pad;
};

// 2^-38 relative perturbation budget of a single step (renderer.cpp:11644).
FX_HD fx::Fe bla_tolerance() { return fx::fe_from(0x1p-38, 0); }

// Radius of a composed map y(x(.)) given x's linear coefficient norms
// (renderer.cpp:11528-11540, 11588-11603, 11380-11390).
FX_HD fx::Fe merged_radius(const fx::Fe& x_r2, const fx::Fe& y_r2, const fx::Fe& x_a, const fx::Fe& x_b,
                           const fx::Fe& input_radius) {
    fx::Fe r = fx::fe_sqrt(x_r2);
    const fx::Fe remaining = fx::fe_sub(fx::fe_sqrt(y_r2), fx::fe_mul(x_b, input_radius));
    if (fx::fe_cmp(remaining, fx::fe_zero()) > 0 && fx::fe_cmp(x_a, fx::fe_zero()) > 0) {
        r = fx::fe_min(r, fx::fe_div(remaining, x_a));
    } else {
        r = fx::fe_zero();
    }
    return r;
}

// Single-step cubic map at reference index `start` (renderer.cpp:11645-11669).
FX_HD BuilderCubic cubic_base(const fx::Fec& ref) {
    BuilderCubic s;
    const fx::Fec zero = fx::fec_make(fx::fe_zero(), fx::fe_zero());
    for (int k = 0; k < 9; ++k) s.c[k] = zero;
    s.c[0] = fx::fec_scale(ref, fx::fe_from(2.0, 0));
    s.c[1] = fx::fec_make(fx::fe_from(1.0, 0), fx::fe_zero());
    s.c[2] = fx::fec_make(fx::fe_from(1.0, 0), fx::fe_zero());
    s.r2 = fx::fe_sqr(fx::fe_mul(bla_tolerance(), fx::fe_sqrt(fx::fec_norm2(ref))));
    s.len = 1;
    s.pad = 0;
    return s;
}

FX_HD BuilderLinear linear_base(const fx::Fec& ref) {
    BuilderLinear s;
    s.a = fx::fec_scale(ref, fx::fe_from(2.0, 0));
    s.b = fx::fec_make(fx::fe_from(1.0, 0), fx::fe_zero());
    s.r2 = fx::fe_sqr(fx::fe_mul(bla_tolerance(), fx::fe_sqrt(fx::fec_norm2(ref))));
    s.len = 1;
    s.pad = 0;
    return s;
}

// merge_bla (renderer.cpp:11528-11586): y(x(d, c), c) truncated at degree 3.
FX_HD BuilderCubic merge_cubic(const BuilderCubic& y, const BuilderCubic& x, const fx::Fe& input_radius) {
    using namespace fx;
    const Fe x_a = fe_sqrt(fec_norm2(x.c[0]));
    const Fe x_b = fe_sqrt(fec_norm2(x.c[1]));
    const Fe radius = merged_radius(x.r2, y.r2, x_a, x_b, input_radius);
    const Fe two = fe_from(2.0, 0);
    const Fe three = fe_from(3.0, 0);
    const Fec &xA = x.c[0], &xB = x.c[1], &xC = x.c[2], &xD = x.c[3], &xE = x.c[4];
    const Fec &yA = y.c[0], &yB = y.c[1], &yC = y.c[2], &yD = y.c[3], &yE = y.c[4], &yF = y.c[5], &yG = y.c[6],
              &yH = y.c[7], &yI = y.c[8];
    const Fec x_a2 = fec_mul(xA, xA);
    const Fec x_ab = fec_mul(xA, xB);
    const Fec x_b2 = fec_mul(xB, xB);
    const Fec x_a3 = fec_mul(x_a2, xA);
    const Fec x_a2b = fec_mul(x_a2, xB);
    const Fec x_ab2 = fec_mul(xA, x_b2);
    const Fec x_b3 = fec_mul(x_b2, xB);
    BuilderCubic r;
    r.c[0] = fec_mul(yA, xA);
    r.c[1] = fec_add(fec_mul(yA, xB), yB);
    r.c[2] = fec_add(fec_mul(yA, xC), fec_mul(yC, x_a2));
    r.c[3] = fec_add(fec_add(fec_mul(yA, xD), fec_mul(yC, fec_scale(x_ab, two))), fec_mul(yD, xA));
    r.c[4] = fec_add(fec_add(fec_mul(yA, xE), fec_mul(yC, x_b2)), fec_add(fec_mul(yD, xB), yE));
    r.c[5] = fec_add(fec_add(fec_mul(yA, x.c[5]), fec_mul(yC, fec_scale(fec_mul(xA, xC), two))), fec_mul(yF, x_a3));
    r.c[6] = fec_add(
        fec_add(fec_add(fec_mul(yA, x.c[6]), fec_mul(yC, fec_scale(fec_add(fec_mul(xA, xD), fec_mul(xB, xC)), two))),
                fec_add(fec_mul(yD, xC), fec_mul(yF, fec_scale(x_a2b, three)))),
        fec_mul(yG, x_a2));
    r.c[7] = fec_add(
        fec_add(fec_add(fec_mul(yA, x.c[7]), fec_mul(yC, fec_scale(fec_add(fec_mul(xA, xE), fec_mul(xB, xD)), two))),
                fec_add(fec_mul(yD, xD), fec_mul(yF, fec_scale(x_ab2, three)))),
        fec_add(fec_mul(yG, fec_scale(x_ab, two)), fec_mul(yH, xA)));
    r.c[8] = fec_add(fec_add(fec_add(fec_mul(yA, x.c[8]), fec_mul(yC, fec_scale(fec_mul(xB, xE), two))),
                             fec_add(fec_mul(yD, xE), fec_mul(yF, x_b3))),
                     fec_add(fec_mul(yG, x_b2), fec_add(fec_mul(yH, xB), yI)));
    r.r2 = fe_sqr(radius);
    r.len = x.len + y.len;
    r.pad = 0;
    return r;
}

// merge_linear_bla (renderer.cpp:11588-11610).
FX_HD BuilderLinear merge_linear(const BuilderLinear& y, const BuilderLinear& x, const fx::Fe& input_radius) {
    using namespace fx;
    const Fe x_a = fe_sqrt(fec_norm2(x.a));
    const Fe x_b = fe_sqrt(fec_norm2(x.b));
    const Fe radius = merged_radius(x.r2, y.r2, x_a, x_b, input_radius);
    BuilderLinear r;
    r.a = fec_mul(y.a, x.a);
    r.b = fec_add(fec_mul(y.a, x.b), y.b);
    r.r2 = fe_sqr(radius);
    r.len = x.len + y.len;
    r.pad = 0;
    return r;
}

// compact_bla_step / compact_linear_bla_step (renderer.cpp:8645-8684).
FX_HD CubicStep compact_cubic(const BuilderCubic& s) {
    bool finite = fx::fe_finite(s.r2);
    CubicStep r;
    for (int k = 0; k < 9; ++k) {
        finite = finite && fx::fec_finite(s.c[k]);
        r.c[k] = fx::sc_from_fe(s.c[k].re, s.c[k].im);
    }
    r.r2 = finite ? s.r2 : fx::fe_zero();
    r.len = s.len;
    r.pad = 0;
    return r;
}

FX_HD LinearStep compact_linear(const BuilderLinear& s) {
    const bool finite = fx::fe_finite(s.r2) && fx::fec_finite(s.a) && fx::fec_finite(s.b);
    LinearStep r;
    r.a = fx::sc_from_fe(s.a.re, s.a.im);
    r.b = fx::sc_from_fe(s.b.re, s.b.im);
    r.r2 = finite ? s.r2 : fx::fe_zero();
    r.len = s.len;
    r.pad = 0;
    return r;
}

// retarget_bla_radius (renderer.cpp:11776-11801): a composed radius from the
// compact render coefficients, with a 2^-40 inward bias.
FX_HD fx::Fe retarget_radius(const fx::Fe& x_r2, const fx::Fe& y_r2, const fx::Sc& x_a, const fx::Sc& x_b,
                             const fx::Fe& input_radius) {
    const fx::Nrm na = fx::sc_norm2(x_a);
    const fx::Nrm nb = fx::sc_norm2(x_b);
    const fx::Fe a = fx::fe_sqrt(fx::fe_make(na.m, na.e));
    const fx::Fe b = fx::fe_sqrt(fx::fe_make(nb.m, nb.e));
    fx::Fe r = merged_radius(x_r2, y_r2, a, b, input_radius);
    r = fx::fe_mul(r, 1.0 - 0x1p-40);
    return fx::fe_sqr(r);
}

FX_HD fx::Fe alt_matrix_norm(const fx::Fe* c) {
    fx::Fe sum = fx::fe_zero();
    for (int k = 0; k < 4; ++k) sum = fx::fe_add(sum, fx::fe_sqr(c[k]));
    return fx::fe_sqrt(sum);
}

// merge_alternate_linear_bla (renderer.cpp:11352-11393).
FX_HD AltStep merge_alt(const AltStep& y, const AltStep& x, const fx::Fe& input_radius) {
    using namespace fx;
    const Fe* yc = y.c;
    const Fe* xc = x.c;
    AltStep r;
    r.c[0] = fe_add(fe_mul(yc[0], xc[0]), fe_mul(yc[1], xc[2]));
    r.c[1] = fe_add(fe_mul(yc[0], xc[1]), fe_mul(yc[1], xc[3]));
    r.c[2] = fe_add(fe_mul(yc[2], xc[0]), fe_mul(yc[3], xc[2]));
    r.c[3] = fe_add(fe_mul(yc[2], xc[1]), fe_mul(yc[3], xc[3]));
    r.c[4] = fe_add(fe_add(fe_mul(yc[0], xc[4]), fe_mul(yc[1], xc[6])), yc[4]);
    r.c[5] = fe_add(fe_add(fe_mul(yc[0], xc[5]), fe_mul(yc[1], xc[7])), yc[5]);
    r.c[6] = fe_add(fe_add(fe_mul(yc[2], xc[4]), fe_mul(yc[3], xc[6])), yc[6]);
    r.c[7] = fe_add(fe_add(fe_mul(yc[2], xc[5]), fe_mul(yc[3], xc[7])), yc[7]);
    Fe radius = merged_radius(x.r2, y.r2, alt_matrix_norm(xc), alt_matrix_norm(xc + 4), input_radius);
    radius = fe_mul(radius, 1.0 - 0x1p-40);
    r.r2 = fe_sqr(radius);
    r.len = x.len + y.len;
    r.pad = 0;
    return r;
}

// Single-step 2x2 map (renderer.cpp:11428-11485).
FX_HD AltStep alt_base(const fx::Fec& ref, int formula) {
    using namespace fx;
    const Fe two = fe_from(2.0, 0);
    const Fe& re = ref.re;
    const Fe& im = ref.im;
    AltStep s;
    for (int j = 0; j < 8; ++j) s.c[j] = fe_zero();
    if (formula == kFormulaTricorn) {
        s.c[0] = fe_mul(re, two);
        s.c[1] = fe_mul(im, -2.0);
        s.c[2] = fe_mul(im, -2.0);
        s.c[3] = fe_mul(re, -2.0);
    } else if (formula == kFormulaBurningShip) {
        const Fe ar = fe_abs(re);
        const Fe ai = fe_abs(im);
        const double rs = re.m < 0.0 ? -1.0 : 1.0;
        const double is = im.m < 0.0 ? -1.0 : 1.0;
        s.c[0] = fe_mul(ar, 2.0 * rs);
        s.c[1] = fe_mul(ai, -2.0 * is);
        s.c[2] = fe_mul(ai, 2.0 * rs);
        s.c[3] = fe_mul(ar, 2.0 * is);
    } else {
        s.c[0] = fe_mul(re, two);
        s.c[1] = fe_mul(im, -2.0);
        s.c[2] = fe_mul(im, two);
        s.c[3] = fe_mul(re, two);
    }
    if (formula != kFormulaJulia) {
        s.c[4] = fe_from(1.0, 0);
        s.c[7] = fe_from(1.0, 0);
    }
    const Fe mag = fe_sqrt(fec_norm2(ref));
    const Fe one = fe_from(1.0, 0);
    Fe radius = fe_mul(bla_tolerance(), fe_cmp(mag, one) > 0 ? mag : one);
    if (formula == kFormulaBurningShip) {
        if (fe_is_zero(re) || fe_is_zero(im)) {
            radius = fe_zero();
        } else {
            const Fe quarter = fe_from(0.25, 0);
            radius = fe_min(radius, fe_mul(fe_abs(re), quarter));
            radius = fe_min(radius, fe_mul(fe_abs(im), quarter));
        }
    }
    s.r2 = fe_sqr(radius);
    s.len = 1;
    s.pad = 0;
    return s;
}

}  // namespace fgb
