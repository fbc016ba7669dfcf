// Extended-exponent arithmetic shared by the host table builders and the
// plain FP64 device kernels.
//
// Semantics follow the reference's FloatExp / ScaledComplex / ScaledNorm
// (renderer.cpp:7532-7824 and 8190-8475): a double mantissa normalised to
// [0.5, 1) with an int exponent, a complex pair sharing one exponent, the
// same one-shift fast paths, the same 60-exponent cut-off in aligned sums
// and the same comparison rules.  Every operation is written so that it
// performs the same IEEE-754 double operations in the same order as the
// reference release build, which has no fused multiply-add: device code that
// includes this header is compiled with --fmad=false and host code with
// -ffp-contract=off.  The frexp/ldexp replacements below are exact
// bit-level operations with one correctly rounded step for subnormal
// results, i.e. the same values glibc's frexp/scalbn return.
#pragma once

#include <cstdint>
#include <climits>
#include <cmath>

#ifdef __CUDACC__
#define FX_HD __host__ __device__ __forceinline__
#else
#define FX_HD inline
#endif

namespace fx {

FX_HD std::uint64_t bits_of(double v) {
#ifdef __CUDA_ARCH__
    return static_cast<std::uint64_t>(__double_as_longlong(v));
#else
    std::uint64_t b;
    __builtin_memcpy(&b, &v, sizeof b);
    return b;
#endif
}

FX_HD double from_bits(std::uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(static_cast<long long>(b));
#else
    double v;
    __builtin_memcpy(&v, &b, sizeof v);
    return v;
#endif
}

FX_HD bool is_finite(double v) { return (bits_of(v) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull; }
FX_HD bool is_nan(double v) { return v != v; }
FX_HD double fabs_(double v) { return from_bits(bits_of(v) & 0x7fffffffffffffffull); }
FX_HD double copysign_(double mag, double sign) {
    return from_bits((bits_of(mag) & 0x7fffffffffffffffull) | (bits_of(sign) & 0x8000000000000000ull));
}
FX_HD int imax(int a, int b) { return a > b ? a : b; }
FX_HD int imin(int a, int b) { return a < b ? a : b; }
FX_HD double dmax(double a, double b) { return a < b ? b : a; }

// x * 2^n with a single round-to-nearest-even step (glibc scalbn semantics).
FX_HD double scale2(double x, int n) {
    std::uint64_t b = bits_of(x);
    int be = static_cast<int>((b >> 52) & 0x7ff);
    if (be == 0x7ff || (b << 1) == 0) return x;  // inf, nan, +-0
    if (be == 0) {
        // Subnormal input: lift it into the normal range exactly first.
        x = x * 18014398509481984.0;  // 2^54
        b = bits_of(x);
        be = static_cast<int>((b >> 52) & 0x7ff);
        n -= 54;
    }
    if (n > 4096) n = 4096;
    if (n < -4096) n = -4096;
    const int ne = be + n;
    if (ne >= 1 && ne <= 2046) {
        return from_bits((b & ~(0x7ffull << 52)) | (static_cast<std::uint64_t>(ne) << 52));
    }
    if (ne > 2046) return copysign_(from_bits(0x7ff0000000000000ull), x);
    // Subnormal or zero result: move the value to the smallest normal binade
    // (exact), then apply the remaining power of two in one multiplication,
    // which is the only rounding.
    const double y = from_bits((b & ~(0x7ffull << 52)) | (1ull << 52));
    const int r = ne - 1;  // <= -1
    if (r < -54) return copysign_(0.0, x);
    return y * from_bits(static_cast<std::uint64_t>(1023 + r) << 52);
}

// frexp: mantissa in [0.5, 1) and exponent; zero/inf/nan returned unchanged
// with exponent 0.
FX_HD double split2(double x, int* e) {
    std::uint64_t b = bits_of(x);
    int be = static_cast<int>((b >> 52) & 0x7ff);
    if (be == 0x7ff || (b << 1) == 0) { *e = 0; return x; }
    int bias = 0;
    if (be == 0) {
        x = x * 18014398509481984.0;  // 2^54, exact
        b = bits_of(x);
        be = static_cast<int>((b >> 52) & 0x7ff);
        bias = 54;
    }
    *e = be - 1022 - bias;
    return from_bits((b & ~(0x7ffull << 52)) | (0x3feull << 52));
}

FX_HD int sat_exp(long long v) {
    if (v > static_cast<long long>(INT_MAX)) return INT_MAX;
    if (v < static_cast<long long>(INT_MIN)) return INT_MIN;
    return static_cast<int>(v);
}

// ---------------------------------------------------------------- FloatExp
struct Fe {
    double m;
    int e;
};

FX_HD Fe fe_make(double m, int e) { Fe r; r.m = m; r.e = e; return r; }
FX_HD Fe fe_zero() { return fe_make(0.0, 0); }
FX_HD bool fe_finite(const Fe& a) { return is_finite(a.m); }
FX_HD bool fe_is_zero(const Fe& a) { return a.m == 0.0; }

// FloatExp::from_parts (renderer.cpp:7551-7561).
FX_HD Fe fe_from(double value, int exponent) {
    if (value == 0.0 || is_nan(value)) return fe_make(value, 0);
    int shift = 0;
    const double n = split2(value, &shift);
    return fe_make(n, sat_exp(static_cast<long long>(exponent) + shift));
}

FX_HD Fe fe_neg(const Fe& a) { return fe_make(-a.m, a.e); }
FX_HD Fe fe_abs(const Fe& a) { return fe_make(fabs_(a.m), a.e); }

// fe_add (renderer.cpp:8197-8235).
FX_HD Fe fe_add(const Fe& a, const Fe& b) {
    if (a.m == 0.0) return b;
    if (b.m == 0.0) return a;
    const Fe* hi = &a;
    const Fe* lo = &b;
    if (b.e > a.e) { hi = &b; lo = &a; }
    const long long diff = static_cast<long long>(hi->e) - lo->e;
    if (diff > 60) return *hi;
    const double m = hi->m + scale2(lo->m, -static_cast<int>(diff));
    if (m == 0.0 || !is_finite(m)) return fe_from(m, hi->e);
    const double mag = fabs_(m);
    if (mag >= 1.0) return fe_make(m * 0.5, sat_exp(static_cast<long long>(hi->e) + 1));
    if (mag >= 0.5) return fe_make(m, hi->e);
    int shift = 0;
    const double n = split2(m, &shift);
    return fe_make(n, sat_exp(static_cast<long long>(hi->e) + shift));
}

FX_HD Fe fe_sub(const Fe& a, const Fe& b) { return fe_add(a, fe_neg(b)); }

// fe_mul (renderer.cpp:8241-8266).
FX_HD Fe fe_mul(const Fe& a, const Fe& b) {
    if (a.m == 0.0 || b.m == 0.0) return fe_zero();
    const double m = a.m * b.m;
    if (!is_finite(m)) return fe_from(m, 0);
    const double mag = fabs_(m);
    const long long es = static_cast<long long>(a.e) + b.e;
    if (mag >= 1.0) return fe_make(m * 0.5, sat_exp(es + 1));
    if (mag < 0.5) return fe_make(m * 2.0, sat_exp(es - 1));
    return fe_make(m, sat_exp(es));
}

FX_HD Fe fe_mul(const Fe& a, double b) { return fe_mul(a, fe_from(b, 0)); }

// fe_div (renderer.cpp:8272-8291).
FX_HD Fe fe_div(const Fe& a, const Fe& b) {
    if (a.m == 0.0) return fe_zero();
    const double m = a.m / b.m;
    if (!is_finite(m)) return fe_from(m, 0);
    const double mag = fabs_(m);
    const long long ed = static_cast<long long>(a.e) - b.e;
    if (mag >= 1.0) return fe_make(m * 0.5, sat_exp(ed + 1));
    if (mag < 0.5) return fe_make(m * 2.0, sat_exp(ed - 1));
    return fe_make(m, sat_exp(ed));
}

FX_HD Fe fe_sqr(const Fe& a) { return fe_mul(a, a); }

// fe_sqrt (renderer.cpp:8297-8315).
FX_HD Fe fe_sqrt(const Fe& a) {
    if (a.m == 0.0) return a;
    long long e = a.e;
    double m = a.m;
    if (m < 0.0 || !is_finite(m)) return fe_from(sqrt(m), 0);
    if (e % 2 != 0) {
        m *= 2.0;
        --e;
        return fe_make(sqrt(m) * 0.5, sat_exp(e / 2 + 1));
    }
    return fe_make(sqrt(m), sat_exp(e / 2));
}

// fe_compare (renderer.cpp:8317-8340).
FX_HD int fe_cmp(const Fe& a, const Fe& b) {
    if (!fe_finite(a)) return fe_finite(b) ? 1 : 0;
    if (!fe_finite(b)) return -1;
    if (a.m == 0.0) return b.m == 0.0 ? 0 : -1;
    if (b.m == 0.0) return a.m > 0.0 ? 1 : -1;
    if (a.m < 0.0 && b.m >= 0.0) return -1;
    if (a.m >= 0.0 && b.m < 0.0) return 1;
    const bool negative = a.m < 0.0;
    if (a.e != b.e) {
        const int r = a.e < b.e ? -1 : 1;
        return negative ? -r : r;
    }
    return (a.m > b.m) - (a.m < b.m);
}

FX_HD Fe fe_min(const Fe& a, const Fe& b) { return fe_cmp(a, b) <= 0 ? a : b; }

struct Fec {
    Fe re;
    Fe im;
};

FX_HD Fec fec_make(const Fe& re, const Fe& im) { Fec r; r.re = re; r.im = im; return r; }
FX_HD Fec fec_add(const Fec& a, const Fec& b) { return fec_make(fe_add(a.re, b.re), fe_add(a.im, b.im)); }
FX_HD Fec fec_sub(const Fec& a, const Fec& b) { return fec_make(fe_sub(a.re, b.re), fe_sub(a.im, b.im)); }
FX_HD Fec fec_mul(const Fec& a, const Fec& b) {
    return fec_make(fe_sub(fe_mul(a.re, b.re), fe_mul(a.im, b.im)),
                    fe_add(fe_mul(a.re, b.im), fe_mul(a.im, b.re)));
}
FX_HD Fec fec_scale(const Fec& a, const Fe& b) { return fec_make(fe_mul(a.re, b), fe_mul(a.im, b)); }
FX_HD Fe fec_norm2(const Fec& a) { return fe_add(fe_sqr(a.re), fe_sqr(a.im)); }
FX_HD bool fec_finite(const Fec& a) { return fe_finite(a.re) && fe_finite(a.im); }

// Escape threshold as FloatExp: 4 (classic) or 1e8 (Kalles high bailout).
FX_HD Fe escape_r2_fe(int mode) { return mode == 1 ? fe_from(1.0e8, 0) : fe_from(4.0, 0); }
FX_HD double escape_r2_d(int mode) { return mode == 1 ? 1.0e8 : 4.0; }

// |R + D|^2 - R_escape^2 in FloatExp (renderer.cpp:8374-8390).
FX_HD Fe fec_escape_margin(const Fec& r, const Fec& d, int mode) {
    const Fe cross = fe_mul(fe_add(fe_mul(r.re, d.re), fe_mul(r.im, d.im)), 2.0);
    const Fe ref_margin = fe_sub(fec_norm2(r), escape_r2_fe(mode));
    return fe_add(fe_add(ref_margin, cross), fec_norm2(d));
}

// ---------------------------------------------------------- ScaledComplex
struct Sc {
    double re;
    double im;
    int e;
};

struct Nrm {
    double m;
    int e;
};

FX_HD Sc sc_make(double re, double im, int e) { Sc r; r.re = re; r.im = im; r.e = e; return r; }
FX_HD Sc sc_zero() { return sc_make(0.0, 0.0, 0); }
FX_HD Sc sc_one() { return sc_make(1.0, 0.0, 0); }
FX_HD bool sc_is_zero(const Sc& a) { return a.re == 0.0 && a.im == 0.0; }
FX_HD bool sc_finite(const Sc& a) { return is_finite(a.re) && is_finite(a.im); }
FX_HD Nrm nrm_make(double m, int e) { Nrm r; r.m = m; r.e = e; return r; }

// ScaledComplex::normalize (renderer.cpp:7611-7656).
FX_HD void sc_normalize(Sc& v) {
    const double mag = dmax(fabs_(v.re), fabs_(v.im));
    if (mag == 0.0) { v.re = 0.0; v.im = 0.0; v.e = 0; return; }
    if (mag >= 2.0) {
        int shift = 0;
        (void)split2(mag, &shift);
        v.re = scale2(v.re, -shift);
        v.im = scale2(v.im, -shift);
        v.e = sat_exp(static_cast<long long>(v.e) + shift);
        return;
    }
    if (mag >= 1.0) {
        v.re *= 0.5;
        v.im *= 0.5;
        v.e = sat_exp(static_cast<long long>(v.e) + 1);
        return;
    }
    if (mag >= 0.5) return;
    if (mag >= 0.25) {
        v.re *= 2.0;
        v.im *= 2.0;
        v.e = sat_exp(static_cast<long long>(v.e) - 1);
        return;
    }
    int shift = 0;
    (void)split2(mag, &shift);
    v.re = scale2(v.re, -shift);
    v.im = scale2(v.im, -shift);
    v.e = sat_exp(static_cast<long long>(v.e) + shift);
}

// ScaledComplex::from_float_exp (renderer.cpp:7658-7675).
FX_HD Sc sc_from_fe(const Fe& re, const Fe& im) {
    if (re.m == 0.0 && im.m == 0.0) return sc_zero();
    const int common = imax(re.e, im.e);
    const long long rd = static_cast<long long>(re.e) - common;
    const long long id = static_cast<long long>(im.e) - common;
    Sc r = sc_make(rd < -1074 ? 0.0 : scale2(re.m, static_cast<int>(rd)),
                   id < -1074 ? 0.0 : scale2(im.m, static_cast<int>(id)), common);
    sc_normalize(r);
    return r;
}

// sc_add (renderer.cpp:7678-7698).
FX_HD Sc sc_add(const Sc& a, const Sc& b) {
    if (a.re == 0.0 && a.im == 0.0) return b;
    if (b.re == 0.0 && b.im == 0.0) return a;
    const Sc* hi = &a;
    const Sc* lo = &b;
    if (b.e > a.e) { hi = &b; lo = &a; }
    const long long diff = static_cast<long long>(hi->e) - lo->e;
    if (diff > 60) return *hi;
    const int d = static_cast<int>(diff);
    Sc r = sc_make(hi->re + scale2(lo->re, -d), hi->im + scale2(lo->im, -d), hi->e);
    sc_normalize(r);
    return r;
}

FX_HD Sc sc_neg(const Sc& a) { return sc_make(-a.re, -a.im, a.e); }
FX_HD Sc sc_conj(const Sc& a) { return sc_make(a.re, -a.im, a.e); }
FX_HD Sc sc_sub(const Sc& a, const Sc& b) { return sc_add(a, sc_neg(b)); }

// sc_mul (renderer.cpp:7712-7722).
FX_HD Sc sc_mul(const Sc& a, const Sc& b) {
    if ((a.re == 0.0 && a.im == 0.0) || (b.re == 0.0 && b.im == 0.0)) return sc_zero();
    Sc r = sc_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re,
                   sat_exp(static_cast<long long>(a.e) + b.e));
    sc_normalize(r);
    return r;
}

// sc_double (renderer.cpp:7724-7733): exact doubling through the exponent.
FX_HD Sc sc_twice(const Sc& a) {
    if (a.re == 0.0 && a.im == 0.0) return sc_zero();
    return sc_make(a.re, a.im, sat_exp(static_cast<long long>(a.e) + 1));
}

// sc_norm_squared (renderer.cpp:7740-7770).
FX_HD Nrm sc_norm2(const Sc& a) {
    const double inf = from_bits(0x7ff0000000000000ull);
    if (!sc_finite(a)) return nrm_make(inf, INT_MAX);
    const double n = a.re * a.re + a.im * a.im;
    if (n == 0.0) return nrm_make(0.0, 0);
    if (!is_finite(n)) return nrm_make(inf, INT_MAX);
    const long long se = 2LL * a.e;
    if (n >= 1.0) {
        const long long e = se + 1;
        if (e > INT_MAX) return nrm_make(inf, INT_MAX);
        return nrm_make(n * 0.5, static_cast<int>(e));
    }
    if (n < 0.5) {
        const long long e = se - 1;
        if (e < INT_MIN) return nrm_make(0.0, 0);
        return nrm_make(n * 2.0, static_cast<int>(e));
    }
    if (se > INT_MAX) return nrm_make(inf, INT_MAX);
    if (se < INT_MIN) return nrm_make(0.0, 0);
    return nrm_make(n, static_cast<int>(se));
}

// sc_compare_norm (renderer.cpp:7772-7781).
FX_HD int nrm_cmp(const Nrm& a, const Nrm& b) {
    if (!is_finite(a.m)) return is_finite(b.m) ? 1 : 0;
    if (!is_finite(b.m)) return -1;
    if (a.m == 0.0 && b.m == 0.0) return 0;
    if (a.m == 0.0) return -1;
    if (b.m == 0.0) return a.m > 0.0 ? 1 : -1;
    if (a.e != b.e) return a.e < b.e ? -1 : 1;
    return (a.m > b.m) - (a.m < b.m);
}

FX_HD bool nrm_outside(const Nrm& n, int mode) {
    const Fe t = escape_r2_fe(mode);
    return nrm_cmp(n, nrm_make(t.m, t.e)) > 0;
}

FX_HD double sc_re_d(const Sc& a) { return scale2(a.re, a.e); }
FX_HD double sc_im_d(const Sc& a) { return scale2(a.im, a.e); }

// scaled_norm_to_double / scaled_norm_from_double (renderer.cpp:7801-7823).
FX_HD double nrm_to_d(const Nrm& n) {
    if (n.m == 0.0) return 0.0;
    const double dbl_max = 1.7976931348623157e308;
    if (!is_finite(n.m)) return dbl_max;
    const double v = scale2(n.m, n.e);
    return is_finite(v) ? dmax(0.0, v) : dbl_max;
}

FX_HD Nrm nrm_from_d(double v) {
    if (!(v > 0.0) || !is_finite(v)) {
        return v > 0.0 ? nrm_make(1.7976931348623157e308, 0) : nrm_make(0.0, 0);
    }
    int e = 0;
    const double m = split2(v, &e);
    return nrm_make(m, e);
}

FX_HD Fe sc_part_fe(const Sc& v, bool imaginary) { return fe_from(imaginary ? v.im : v.re, v.e); }
FX_HD Fec sc_to_fec(const Sc& v) { return fec_make(sc_part_fe(v, false), sc_part_fe(v, true)); }

// Signed escape margin |Z + d|^2 - R^2 (renderer.cpp:8400-8425).
FX_HD Fe sc_escape_margin(const Sc& ref, const Sc& d, int mode) {
    return fec_escape_margin(sc_to_fec(ref), sc_to_fec(d), mode);
}

// sc_norm_squared_with_delta given the margin (renderer.cpp:8445-8453).
FX_HD Nrm nrm_from_margin(const Fe& margin, int mode) {
    const Fe n = fe_add(escape_r2_fe(mode), margin);
    return nrm_make(n.m, n.e);
}

}  // namespace fx
