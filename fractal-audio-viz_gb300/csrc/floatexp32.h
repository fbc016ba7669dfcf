// FP32-mantissa / int32-exponent complex arithmetic for the floatexp form.
//
// A value is (x + i y) * 2^e with max(|x|, |y|) in [0.5, 1), or zero.  All
// scaling is integer exponent arithmetic on the float bit patterns, so a
// complex multiply costs four FP32 multiplies, two adds and a handful of
// integer operations, against the reference's FP64 ScaledComplex
// (renderer.cpp:7605-7736) whose doubles run at 1/64 of the FP32 rate on
// GB300.  Accuracy is that of FP32 (24-bit mantissa); the range is that of
// the int32 exponent, so deltas far below 1e-38 stay representable.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define F32_HD __host__ __device__ __forceinline__
#else
#define F32_HD inline
#endif

namespace f32x {

struct F2e {
    float x;
    float y;
    int e;
};

struct N1e {  // non-negative real (a squared norm), m in [0.5, 1) or zero
    float m;
    int e;
};

F32_HD int f_bits(float v) {
#ifdef __CUDA_ARCH__
    return __float_as_int(v);
#else
    int b;
    __builtin_memcpy(&b, &v, sizeof b);
    return b;
#endif
}

F32_HD float f_from_bits(int b) {
#ifdef __CUDA_ARCH__
    return __int_as_float(b);
#else
    float v;
    __builtin_memcpy(&v, &b, sizeof v);
    return v;
#endif
}

// 2^k as a float for k in [-126, 127].
F32_HD float pow2f(int k) { return f_from_bits((k + 127) << 23); }

// Multiply by 2^k for any k, saturating to 0 / inf outside the float range.
F32_HD float ldexpf_fast(float v, int k) {
    if (k > 127) {
        v *= pow2f(127);
        k -= 127;
        if (k > 127) k = 127;
    } else if (k < -126) {
        v *= pow2f(-126);
        k += 126;
        if (k < -126) return v * 0.0f;
    }
    return v * pow2f(k);
}

F32_HD F2e make(float x, float y, int e) {
    F2e r;
    r.x = x;
    r.y = y;
    r.e = e;
    return r;
}

F32_HD F2e zero() { return make(0.0f, 0.0f, 0); }

// Normalise so that max(|x|, |y|) is in [0.5, 1).
F32_HD F2e norm(float x, float y, int e) {
    const int bx = f_bits(x) & 0x7fffffff;
    const int by = f_bits(y) & 0x7fffffff;
    int b = bx > by ? bx : by;
    if (b == 0) return zero();
    if (b >= 0x7f800000) return make(x, y, e);  // inf / nan propagate
    int be = b >> 23;
    if (be == 0) {  // subnormal maximum: lift by 2^24 first
        x *= 16777216.0f;
        y *= 16777216.0f;
        e -= 24;
        const int cx = f_bits(x) & 0x7fffffff, cy = f_bits(y) & 0x7fffffff;
        b = cx > cy ? cx : cy;
        be = b >> 23;
    }
    const int shift = be - 126;  // in [-125, 128]
    if (shift == 0) return make(x, y, e);
    if (shift <= 126) {
        const float s = pow2f(-shift);
        return make(x * s, y * s, e + shift);
    }
    const float s = pow2f(-126);
    const float t = pow2f(126 - shift);
    return make(x * s * t, y * s * t, e + shift);
}

F32_HD bool is_zero(const F2e& a) { return a.x == 0.0f && a.y == 0.0f; }
F32_HD bool finite(const F2e& a) {
    return (f_bits(a.x) & 0x7f800000) != 0x7f800000 && (f_bits(a.y) & 0x7f800000) != 0x7f800000;
}

F32_HD F2e add(const F2e& a, const F2e& b) {
    if (is_zero(a)) return b;
    if (is_zero(b)) return a;
    const F2e& hi = b.e > a.e ? b : a;
    const F2e& lo = b.e > a.e ? a : b;
    const int d = hi.e - lo.e;
    if (d > 40) return hi;
    const float s = pow2f(-d);
    return norm(hi.x + lo.x * s, hi.y + lo.y * s, hi.e);
}

F32_HD F2e neg(const F2e& a) { return make(-a.x, -a.y, a.e); }
F32_HD F2e sub(const F2e& a, const F2e& b) { return add(a, neg(b)); }

F32_HD F2e mul(const F2e& a, const F2e& b) {
    if (is_zero(a) || is_zero(b)) return zero();
    return norm(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x, a.e + b.e);
}

F32_HD F2e twice(const F2e& a) { return is_zero(a) ? a : make(a.x, a.y, a.e + 1); }


F32_HD N1e n_norm(float m, int e) {
    if (m == 0.0f) {
        N1e r;
        r.m = 0.0f;
        r.e = 0;
        return r;
    }
    const int b = f_bits(m) & 0x7fffffff;
    N1e r;
    if (b >= 0x7f800000) {
        r.m = m;
        r.e = 0x3fffffff;
        return r;
    }
    const int be = b >> 23;  // m is a sum of squares of values in [0, 1): be >= 1 unless tiny
    if (be == 0) {
        r.m = m;
        r.e = e;
        return r;
    }
    const int shift = be - 126;
    r.m = m * pow2f(-shift);
    r.e = e + shift;
    return r;
}

// |a|^2 as a normalised real.
F32_HD N1e norm2(const F2e& a) {
    if (is_zero(a)) return n_norm(0.0f, 0);
    return n_norm(a.x * a.x + a.y * a.y, 2 * a.e);
}

F32_HD int n_cmp(const N1e& a, const N1e& b) {
    if (a.m == 0.0f && b.m == 0.0f) return 0;
    if (a.m == 0.0f) return -1;
    if (b.m == 0.0f) return 1;
    if (a.e != b.e) return a.e < b.e ? -1 : 1;
    return (a.m > b.m) - (a.m < b.m);
}

// Signed real (m * 2^e, |m| in [0.5, 1), or zero): the components of the
// alternate formulas' 2x2 maps, escape margins and Jacobians.
struct R1e {
    float m;
    int e;
};

F32_HD R1e r_make(float m, int e) {
    R1e r;
    r.m = m;
    r.e = e;
    return r;
}

F32_HD R1e r_zero() { return r_make(0.0f, 0); }

F32_HD R1e r_norm(float m, int e) {
    if (m == 0.0f) return r_zero();
    int b = f_bits(m) & 0x7fffffff;
    if (b >= 0x7f800000) return r_make(m, 0x3fffffff);
    int be = b >> 23;
    if (be == 0) {  // subnormal: lift by 2^24 first
        m *= 16777216.0f;
        e -= 24;
        b = f_bits(m) & 0x7fffffff;
        be = b >> 23;
    }
    const int shift = be - 126;
    return shift == 0 ? r_make(m, e) : r_make(m * pow2f(-shift), e + shift);
}

F32_HD bool r_finite(const R1e& a) { return (f_bits(a.m) & 0x7f800000) != 0x7f800000; }
F32_HD R1e r_neg(const R1e& a) { return r_make(-a.m, a.e); }
F32_HD R1e r_abs(const R1e& a) { return r_make(a.m < 0.0f ? -a.m : a.m, a.e); }

F32_HD R1e r_add(const R1e& a, const R1e& b) {
    if (a.m == 0.0f) return b;
    if (b.m == 0.0f) return a;
    const R1e& hi = b.e > a.e ? b : a;
    const R1e& lo = b.e > a.e ? a : b;
    const int d = hi.e - lo.e;
    if (d > 40) return hi;
    return r_norm(hi.m + lo.m * pow2f(-d), hi.e);
}

F32_HD R1e r_sub(const R1e& a, const R1e& b) { return r_add(a, r_neg(b)); }

F32_HD R1e r_mul(const R1e& a, const R1e& b) {
    if (a.m == 0.0f || b.m == 0.0f) return r_zero();
    return r_norm(a.m * b.m, a.e + b.e);
}

// a * s for a small constant s (2, -2, +-1).
F32_HD R1e r_scale(const R1e& a, float s) { return a.m == 0.0f ? a : r_norm(a.m * s, a.e); }

F32_HD int r_sign(const R1e& a) { return (a.m > 0.0f) - (a.m < 0.0f); }

// Signed comparison.
F32_HD int r_cmp(const R1e& a, const R1e& b) {
    const int sa = r_sign(a), sb = r_sign(b);
    if (sa != sb) return sa < sb ? -1 : 1;
    if (sa == 0) return 0;
    if (a.e != b.e) return (a.e < b.e ? -1 : 1) * sa;
    return (a.m > b.m) - (a.m < b.m);
}

F32_HD R1e r_re(const F2e& z) { return r_norm(z.x, z.e); }
F32_HD R1e r_im(const F2e& z) { return r_norm(z.y, z.e); }

// Complex value from two reals (shared exponent, then normalised).
F32_HD F2e from_r(const R1e& re, const R1e& im) {
    if (re.m == 0.0f && im.m == 0.0f) return zero();
    if (re.m == 0.0f) return norm(0.0f, im.m, im.e);
    if (im.m == 0.0f) return norm(re.m, 0.0f, re.e);
    const int e = re.e > im.e ? re.e : im.e;
    const int dr = re.e - e, di = im.e - e;
    return norm(dr < -126 ? 0.0f : re.m * pow2f(dr), di < -126 ? 0.0f : im.m * pow2f(di), e);
}

F32_HD N1e n_from_r(const R1e& a) {
    N1e r;
    r.m = a.m;
    r.e = a.e;
    return r;
}

F32_HD F2e conj(const F2e& a) { return make(a.x, -a.y, a.e); }

// Plain float value of a (0 when below the float range, +-inf above).
F32_HD float to_float_x(const F2e& a) { return ldexpf_fast(a.x, a.e); }
F32_HD float to_float_y(const F2e& a) { return ldexpf_fast(a.y, a.e); }

F32_HD F2e from_float(float x, float y) { return norm(x, y, 0); }

}  // namespace f32x
