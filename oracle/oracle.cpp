// ORACLE - test infrastructure only.
//
// A CPU restatement of the reference's hot path (haaakez/fractal-audio-viz,
// renderer.cpp), exporting the same renderer.h C ABI so the parity tests can
// drive it exactly like the reference build and like the GB300 library.  It
// exists because the reference cannot be compiled where the GPU runs; it is
// pinned against the reference itself by tests/test_oracle_port.py, which
// requires bit-identical fields and counts on every golden case.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library.  The product never does.
//
// Compiled with -ffp-contract=off (oracle/Makefile): every double operation
// rounds on its own, as in the reference release build.  MPFR comes from the
// system runtime through shim/mpfr.h.
//
// Section map (reference file:line):
//   extended-exponent numbers   renderer.cpp:7532-7824, 8190-8475
//   reference orbit             renderer.cpp:10640-10922
//   image series                renderer.cpp:11162-11334
//   BLA hierarchies             renderer.cpp:11528-11769, retarget 11776-11868
//   deep Mandelbrot pixel loop  renderer.cpp:12451-13583
//   direct renderer             renderer.cpp:10054-10135, 10281-10438
//   aurora colour               renderer.cpp:4788-4923, 5210-5237, 13771-13826
//   atlas compositor            renderer.cpp:4931-5003, 5141-5244, 17969-18304,
//                               18697-18888, 19138-19430
#include <omp.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <sstream>
#include <locale>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "shim/mpfr.h"
#include "fractal_gb300.h"

namespace oracle {

using std::int64_t;

thread_local std::string error_text;

struct Oops : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ------------------------------------------------------------ numbers
// frexp / ldexp with the library's exact results, decided on the bit
// pattern for normal doubles (a multiply by an exact power of two rounds
// once, as ldexp does); zeros, subnormals, infinities, NaNs and extreme
// scales go to the library.  They keep the hot loops free of libm calls.
inline double frexp2(double v, int* e) {
    std::uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    const int biased = static_cast<int>((b >> 52) & 0x7ff);
    if (biased == 0 || biased == 0x7ff) return std::frexp(v, e);
    *e = biased - 1022;
    b = (b & ~(0x7ffULL << 52)) | (1022ULL << 52);
    double r;
    std::memcpy(&r, &b, sizeof r);
    return r;
}

inline double ldexp2(double v, int k) {
    if (k < -1022 || k > 1023) return std::ldexp(v, k);
    const std::uint64_t b = static_cast<std::uint64_t>(k + 1023) << 52;
    double scale;
    std::memcpy(&scale, &b, sizeof scale);
    return v * scale;
}

int clamp_exp(long long v) {
    return v > INT_MAX ? INT_MAX : (v < INT_MIN ? INT_MIN : static_cast<int>(v));
}

struct FE {  // mantissa in [0.5,1) times 2^e
    double m = 0.0;
    int e = 0;
};

FE fe(double value, int exponent) {
    if (value == 0.0 || std::isnan(value)) return {value, 0};
    int s = 0;
    double n = frexp2(value, &s);
    return {n, clamp_exp(static_cast<long long>(exponent) + s)};
}

bool ok(const FE& a) { return std::isfinite(a.m); }

FE neg(const FE& a) { return {-a.m, a.e}; }
FE absv(const FE& a) { return {std::fabs(a.m), a.e}; }

FE add(const FE& a, const FE& b) {
    if (a.m == 0.0) return b;
    if (b.m == 0.0) return a;
    const FE& big = b.e > a.e ? b : a;
    const FE& small = b.e > a.e ? a : b;
    long long gap = static_cast<long long>(big.e) - small.e;
    if (gap > 60) return big;
    double m = big.m + ldexp2(small.m, -static_cast<int>(gap));
    if (m == 0.0 || !std::isfinite(m)) return fe(m, big.e);
    double am = std::fabs(m);
    if (am >= 1.0) return {m * 0.5, clamp_exp(static_cast<long long>(big.e) + 1)};
    if (am >= 0.5) return {m, big.e};
    int s = 0;
    double n = frexp2(m, &s);
    return {n, clamp_exp(static_cast<long long>(big.e) + s)};
}

FE sub(const FE& a, const FE& b) { return add(a, neg(b)); }

FE mul(const FE& a, const FE& b) {
    if (a.m == 0.0 || b.m == 0.0) return {};
    double m = a.m * b.m;
    if (!std::isfinite(m)) return fe(m, 0);
    long long e = static_cast<long long>(a.e) + b.e;
    double am = std::fabs(m);
    if (am >= 1.0) return {m * 0.5, clamp_exp(e + 1)};
    if (am < 0.5) return {m * 2.0, clamp_exp(e - 1)};
    return {m, clamp_exp(e)};
}

FE mul(const FE& a, double b) { return mul(a, fe(b, 0)); }

FE divide(const FE& a, const FE& b) {
    if (a.m == 0.0) return {};
    double m = a.m / b.m;
    if (!std::isfinite(m)) return fe(m, 0);
    long long e = static_cast<long long>(a.e) - b.e;
    double am = std::fabs(m);
    if (am >= 1.0) return {m * 0.5, clamp_exp(e + 1)};
    if (am < 0.5) return {m * 2.0, clamp_exp(e - 1)};
    return {m, clamp_exp(e)};
}

FE sq(const FE& a) { return mul(a, a); }

FE root(const FE& a) {
    if (a.m == 0.0) return a;
    if (a.m < 0.0 || !std::isfinite(a.m)) return fe(std::sqrt(a.m), 0);
    long long e = a.e;
    if (e % 2 != 0) return {std::sqrt(a.m * 2.0) * 0.5, clamp_exp((e - 1) / 2 + 1)};
    return {std::sqrt(a.m), clamp_exp(e / 2)};
}

int cmp(const FE& a, const FE& b) {
    if (!ok(a)) return ok(b) ? 1 : 0;
    if (!ok(b)) return -1;
    if (a.m == 0.0) return b.m == 0.0 ? 0 : -1;
    if (b.m == 0.0) return a.m > 0.0 ? 1 : -1;
    bool an = a.m < 0.0, bn = b.m < 0.0;
    if (an && !bn) return -1;
    if (!an && bn) return 1;
    if (a.e != b.e) return (a.e < b.e ? -1 : 1) * (an ? -1 : 1);
    return (a.m > b.m) - (a.m < b.m);
}

FE lesser(const FE& a, const FE& b) { return cmp(a, b) <= 0 ? a : b; }

struct FC {
    FE r, i;
};

FC cadd(const FC& a, const FC& b) { return {add(a.r, b.r), add(a.i, b.i)}; }
FC csub(const FC& a, const FC& b) { return {sub(a.r, b.r), sub(a.i, b.i)}; }
FC cmul(const FC& a, const FC& b) {
    return {sub(mul(a.r, b.r), mul(a.i, b.i)), add(mul(a.r, b.i), mul(a.i, b.r))};
}
FC cscale(const FC& a, const FE& s) { return {mul(a.r, s), mul(a.i, s)}; }
FE cnorm(const FC& a) { return add(sq(a.r), sq(a.i)); }
bool cok(const FC& a) { return ok(a.r) && ok(a.i); }

FE bailout(int mode) { return mode == 1 ? fe(1.0e8, 0) : fe(4.0, 0); }

FE margin_fc(const FC& z, const FC& d, int mode) {
    FE cross = mul(add(mul(z.r, d.r), mul(z.i, d.i)), 2.0);
    return add(add(sub(cnorm(z), bailout(mode)), cross), cnorm(d));
}

struct SC {  // shared-exponent complex
    double x = 0.0, y = 0.0;
    int e = 0;
};

void fix(SC& v) {
    double big = std::max(std::fabs(v.x), std::fabs(v.y));
    if (big == 0.0) {
        v = {};
        return;
    }
    int s = 0;
    if (big >= 2.0 || big < 0.25) {
        frexp2(big, &s);
        v.x = ldexp2(v.x, -s);
        v.y = ldexp2(v.y, -s);
        v.e = clamp_exp(static_cast<long long>(v.e) + s);
    } else if (big >= 1.0) {
        v.x *= 0.5;
        v.y *= 0.5;
        v.e = clamp_exp(static_cast<long long>(v.e) + 1);
    } else if (big < 0.5) {
        v.x *= 2.0;
        v.y *= 2.0;
        v.e = clamp_exp(static_cast<long long>(v.e) - 1);
    }
}

SC from_fc(const FE& r, const FE& i) {
    if (r.m == 0.0 && i.m == 0.0) return {};
    int top = std::max(r.e, i.e);
    long long dr = static_cast<long long>(r.e) - top, di = static_cast<long long>(i.e) - top;
    SC v{dr < -1074 ? 0.0 : ldexp2(r.m, static_cast<int>(dr)),
         di < -1074 ? 0.0 : ldexp2(i.m, static_cast<int>(di)), top};
    fix(v);
    return v;
}

bool zero(const SC& a) { return a.x == 0.0 && a.y == 0.0; }
bool sok(const SC& a) { return std::isfinite(a.x) && std::isfinite(a.y); }

SC sadd(const SC& a, const SC& b) {
    if (zero(a)) return b;
    if (zero(b)) return a;
    const SC& big = b.e > a.e ? b : a;
    const SC& small = b.e > a.e ? a : b;
    long long gap = static_cast<long long>(big.e) - small.e;
    if (gap > 60) return big;
    SC v{big.x + ldexp2(small.x, -static_cast<int>(gap)), big.y + ldexp2(small.y, -static_cast<int>(gap)),
         big.e};
    fix(v);
    return v;
}

SC sneg(const SC& a) { return {-a.x, -a.y, a.e}; }
SC sconj(const SC& a) { return {a.x, -a.y, a.e}; }
SC ssub(const SC& a, const SC& b) { return sadd(a, sneg(b)); }

SC smul(const SC& a, const SC& b) {
    if (zero(a) || zero(b)) return {};
    SC v{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x, clamp_exp(static_cast<long long>(a.e) + b.e)};
    fix(v);
    return v;
}

SC stwice(const SC& a) {
    if (zero(a)) return {};
    return {a.x, a.y, clamp_exp(static_cast<long long>(a.e) + 1)};
}

const SC ONE{1.0, 0.0, 0};

struct NM {
    double m = 0.0;
    int e = 0;
};

NM norm(const SC& a) {
    const double inf = std::numeric_limits<double>::infinity();
    if (!sok(a)) return {inf, INT_MAX};
    double n = a.x * a.x + a.y * a.y;
    if (n == 0.0) return {};
    if (!std::isfinite(n)) return {inf, INT_MAX};
    long long e = 2LL * a.e;
    if (n >= 1.0) return e + 1 > INT_MAX ? NM{inf, INT_MAX} : NM{n * 0.5, static_cast<int>(e + 1)};
    if (n < 0.5) return e - 1 < INT_MIN ? NM{} : NM{n * 2.0, static_cast<int>(e - 1)};
    if (e > INT_MAX) return {inf, INT_MAX};
    if (e < INT_MIN) return {};
    return {n, static_cast<int>(e)};
}

int ncmp(const NM& a, const NM& b) {
    if (!std::isfinite(a.m)) return std::isfinite(b.m) ? 1 : 0;
    if (!std::isfinite(b.m)) return -1;
    if (a.m == 0.0 && b.m == 0.0) return 0;
    if (a.m == 0.0) return -1;
    if (b.m == 0.0) return a.m > 0.0 ? 1 : -1;
    if (a.e != b.e) return a.e < b.e ? -1 : 1;
    return (a.m > b.m) - (a.m < b.m);
}

bool escaped_norm(const NM& n, int mode) {
    FE t = bailout(mode);
    return ncmp(n, NM{t.m, t.e}) > 0;
}

double sx(const SC& a) { return ldexp2(a.x, a.e); }
double sy(const SC& a) { return ldexp2(a.y, a.e); }

FC to_fc(const SC& a) { return {fe(a.x, a.e), fe(a.y, a.e)}; }

FE margin_sc(const SC& z, const SC& d, int mode) { return margin_fc(to_fc(z), to_fc(d), mode); }

NM norm_with_margin(const FE& margin, int mode) {
    FE n = add(bailout(mode), margin);
    return {n.m, n.e};
}

double norm_double(const NM& n) {
    if (n.m == 0.0) return 0.0;
    if (!std::isfinite(n.m)) return std::numeric_limits<double>::max();
    double v = ldexp2(n.m, n.e);
    return std::isfinite(v) ? std::max(0.0, v) : std::numeric_limits<double>::max();
}

NM norm_of_double(double v) {
    if (!(v > 0.0) || !std::isfinite(v)) return v > 0.0 ? NM{std::numeric_limits<double>::max(), 0} : NM{};
    int e = 0;
    double m = frexp2(v, &e);
    return {m, e};
}

constexpr long double LN2 = 0.693147180559945309417232121458176568L;
constexpr double TAU = 6.283185307179586476925286766559005768;

// ------------------------------------------------------------ reference
struct Cubic {
    std::array<SC, 9> k;
    FE r2;
    int len = 1;
};
struct Linear {
    SC a, b;
    FE r2;
    int len = 1;
};

struct Reference {
    std::vector<FC> builder;  // FloatExp orbit, kept for reusable roots
    std::vector<SC> z;
    std::vector<double> zr, zi;
    std::vector<std::vector<Cubic>> cubic;
    std::vector<std::vector<Linear>> linear, deep;
    FE radius, deep_radius;
    int map_end = 0;
    bool series_on = false;
    int series_order = 0, series_it = 1;
    FE series_r2;
    std::vector<SC> series;
    int max_iter = 0, series_request = 8;
    long double xc = 0, yc = 0;
    int formula = 0, escape_mode = 0, coordinate_mode = 0;
    double jr = 0, ji = 0;
    long bits = 0;
    std::uint64_t ns[3] = {0, 0, 0};
};

std::mutex table_mutex;
std::unordered_map<std::uintptr_t, std::shared_ptr<Reference>> table;
std::uintptr_t next_id = 0x1000;

bool text_ok(const char* s) {
    if (!s) return false;
    for (std::size_t i = 0; i <= 50000; ++i)
        if (s[i] == '\0') return true;
    return false;
}

long double parse_ld(const char* s, const char* what) {
    if (!text_ok(s)) throw Oops("native coordinate text is too long or null");
    std::istringstream in(s);
    in.imbue(std::locale::classic());
    long double v = 0;
    in >> v;
    bool good = !in.fail();
    in >> std::ws;
    if (!good || !in.eof() || !std::isfinite(v)) throw Oops(std::string("invalid ") + what + " coordinate");
    return v;
}

FE fe_of(mpfr_srcptr v) {
    long e = 0;
    double m = mpfr_get_d_2exp(&e, v, MPFR_RNDN);
    if (!std::isfinite(m)) return {m, 0};
    if (e > INT_MAX) return {std::copysign(std::numeric_limits<double>::infinity(), m), 0};
    if (e < INT_MIN) return {};
    return fe(m, static_cast<int>(e));
}

FE zoom_of(const char* s, long bits) {
    if (!text_ok(s)) throw Oops("native zoom text is too long or null");
    mpfr_t v;
    mpfr_init2(v, bits);
    int st = mpfr_set_str(v, s, 10, MPFR_RNDN);
    if (st != 0 || mpfr_sgn(v) <= 0 || !mpfr_number_p(v)) {
        mpfr_clear(v);
        throw Oops("invalid deep Mandelbrot zoom");
    }
    FE r = fe_of(v);
    mpfr_clear(v);
    if (!ok(r) || r.m == 0.0) throw Oops("deep Mandelbrot zoom is outside the native exponent range");
    long double lz = (std::log(std::fabs(static_cast<long double>(r.m))) + r.e * LN2) / std::log(10.0L);
    if (!std::isfinite(lz) || lz < -300.0L || lz > 9800.0L) throw Oops("deep Mandelbrot zoom is outside the supported range");
    return r;
}

double height_factor(int mode) { return mode == 1 ? 4.0 : 2.8; }

double axis(int index, int size, int mode) {
    double origin = mode == 1 ? static_cast<double>(size / 2) : static_cast<double>(size - 1) / 2.0;
    return static_cast<double>(index) - origin;
}

void orbit(Reference& R, const char* xs, const char* ys, const char* zs, int max_iter, int bits) {
    bits = std::max(128, bits);
    mpfr_t cx, cy, zoom, rad, zr, zi, nr, ni, t, n2, mg;
    mpfr_t* all[] = {&cx, &cy, &zoom, &rad, &zr, &zi, &nr, &ni, &t, &n2, &mg};
    for (auto* p : all) mpfr_init2(*p, bits);
    auto cleanup = [&] {
        for (auto* p : all) mpfr_clear(*p);
    };
    if (mpfr_set_str(cx, xs, 10, MPFR_RNDN) != 0 || mpfr_set_str(cy, ys, 10, MPFR_RNDN) != 0) {
        cleanup();
        throw Oops("invalid MPFR Mandelbrot centre");
    }
    if (mpfr_set_str(zoom, zs, 10, MPFR_RNDN) == 0 && mpfr_sgn(zoom) > 0) {
        mpfr_set_d(rad, height_factor(R.coordinate_mode), MPFR_RNDN);
        mpfr_div(rad, rad, zoom, MPFR_RNDN);
        R.radius = fe_of(rad);
    } else {
        R.radius = fe(1.0, 0);
    }
    mpfr_set_zero(zr, 0);
    mpfr_set_zero(zi, 0);
    R.bits = bits;
    R.max_iter = max_iter;
    R.builder.clear();
    FE re = fe_of(zr), im = fe_of(zi);
    for (int i = 0; i <= max_iter; ++i) {
        if (!ok(re) || !ok(im)) break;
        R.builder.push_back({re, im});
        // z <- z^2 + c
        mpfr_mul(nr, zr, zr, MPFR_RNDN);
        mpfr_mul(t, zi, zi, MPFR_RNDN);
        mpfr_sub(nr, nr, t, MPFR_RNDN);
        mpfr_mul(ni, zr, zi, MPFR_RNDN);
        mpfr_mul_ui(ni, ni, 2, MPFR_RNDN);
        mpfr_add(nr, nr, cx, MPFR_RNDN);
        mpfr_add(ni, ni, cy, MPFR_RNDN);
        mpfr_set(zr, nr, MPFR_RNDN);
        mpfr_set(zi, ni, MPFR_RNDN);
        re = fe_of(zr);
        im = fe_of(zi);
    }
    cleanup();
    if (R.builder.empty()) throw Oops("reference orbit lost finite state at iteration zero");
    R.map_end = static_cast<int>(R.builder.size()) - 1;
    for (std::size_t i = 1; i < R.builder.size(); ++i) {
        if (cmp(cnorm(R.builder[i]), bailout(R.escape_mode)) > 0) {
            R.map_end = static_cast<int>(i);
            break;
        }
    }
    const std::size_t n = R.builder.size();
    R.z.resize(n);
    R.zr.resize(n);
    R.zi.resize(n);
    for (std::size_t i = 0; i < n; ++i) {
        R.z[i] = from_fc(R.builder[i].r, R.builder[i].i);
        R.zr[i] = ldexp2(R.z[i].x, R.z[i].e);
        R.zi[i] = ldexp2(R.z[i].y, R.z[i].e);
    }
}

FC poly(const std::vector<FC>& k, const FC& dc) {
    if (k.size() <= 1) return {};
    FC r = k.back();
    for (std::size_t i = k.size() - 1; i > 1; --i) r = cadd(cmul(r, dc), k[i - 1]);
    return cmul(r, dc);
}

void image_series(Reference& R, const std::vector<FC>& orb) {
    R.series_on = false;
    R.series.clear();
    R.series_it = 1;
    R.series_order = 0;
    R.series_r2 = {};
    if (orb.size() < 16 || R.max_iter < 8) return;
    const int order = std::clamp(R.series_request, 8, 32);
    const int last = std::max(2, std::clamp(R.map_end, 2, static_cast<int>(orb.size()) - 1) - 1);
    if (R.radius.m == 0.0 || !ok(R.radius)) return;
    const FE pr = mul(R.radius, 1.5), dg = mul(pr, 0.7071067811865476), in = mul(pr, 0.47), z0{};
    const FC probes[12] = {{pr, z0}, {neg(pr), z0}, {z0, pr}, {z0, neg(pr)}, {dg, dg}, {neg(dg), dg},
                           {dg, neg(dg)}, {neg(dg), neg(dg)}, {in, mul(in, 0.63)}, {neg(in), mul(in, 0.63)},
                           {mul(in, 0.63), in}, {mul(in, 0.63), neg(in)}};
    std::vector<FC> k(static_cast<std::size_t>(order + 1)), nk(k.size()), keep;
    FC exact[12] = {};
    const FE two = fe(2.0, 0), tol = fe(ldexp2(1.0, -38), 0), floor2 = sq(pr);
    int best = 1;
    for (int it = 0; it < last; ++it) {
        const FC& Z = orb[static_cast<std::size_t>(it)];
        for (int t = 1; t <= order; ++t) {
            FC v = cscale(cmul(Z, k[static_cast<std::size_t>(t)]), two);
            for (int l = 1; l < t; ++l) v = cadd(v, cmul(k[static_cast<std::size_t>(l)], k[static_cast<std::size_t>(t - l)]));
            if (t == 1) v = cadd(v, FC{fe(1.0, 0), {}});
            nk[static_cast<std::size_t>(t)] = v;
        }
        std::swap(k, nk);
        bool safe = true;
        for (int p = 0; p < 12 && safe; ++p) {
            exact[p] = cadd(cscale(cmul(Z, exact[p]), two), cadd(cmul(exact[p], exact[p]), probes[p]));
            if (it + 1 < order) continue;
            FC approx = poly(k, probes[p]);
            FE scale = cnorm(exact[p]);
            if (cmp(scale, floor2) < 0) scale = floor2;
            if (cmp(cnorm(csub(approx, exact[p])), mul(scale, tol)) > 0) safe = false;
            const FC& Zn = orb[static_cast<std::size_t>(it + 1)];
            if (safe && !(cmp(margin_fc(Zn, exact[p], R.escape_mode), FE{}) <= 0
                          && cmp(margin_fc(Zn, approx, R.escape_mode), FE{}) <= 0)) safe = false;
        }
        if (!safe) break;
        if (it + 1 >= order) {
            best = it + 1;
            keep = k;
        }
    }
    if (best <= 1 || keep.empty()) return;
    R.series_on = true;
    R.series_order = order;
    R.series_it = best;
    R.series_r2 = sq(pr);
    for (const FC& c : keep) R.series.push_back(from_fc(c.r, c.i));
}

struct BCubic {
    FC k[9];
    FE r2;
    int len;
};
struct BLinear {
    FC a, b;
    FE r2;
    int len;
};

FE composed_radius(const FE& xr2, const FE& yr2, const FE& xa, const FE& xb, const FE& in) {
    FE r = root(xr2);
    FE left = sub(root(yr2), mul(xb, in));
    if (cmp(left, FE{}) > 0 && cmp(xa, FE{}) > 0) return lesser(r, divide(left, xa));
    return {};
}

BCubic compose(const BCubic& y, const BCubic& x, const FE& in) {
    const FE two = fe(2.0, 0), three = fe(3.0, 0);
    const FC *X = x.k, *Y = y.k;
    FC a2 = cmul(X[0], X[0]), ab = cmul(X[0], X[1]), b2 = cmul(X[1], X[1]);
    FC a3 = cmul(a2, X[0]), a2b = cmul(a2, X[1]), ab2 = cmul(X[0], b2), b3 = cmul(b2, X[1]);
    BCubic r;
    r.k[0] = cmul(Y[0], X[0]);
    r.k[1] = cadd(cmul(Y[0], X[1]), Y[1]);
    r.k[2] = cadd(cmul(Y[0], X[2]), cmul(Y[2], a2));
    r.k[3] = cadd(cadd(cmul(Y[0], X[3]), cmul(Y[2], cscale(ab, two))), cmul(Y[3], X[0]));
    r.k[4] = cadd(cadd(cmul(Y[0], X[4]), cmul(Y[2], b2)), cadd(cmul(Y[3], X[1]), Y[4]));
    r.k[5] = cadd(cadd(cmul(Y[0], X[5]), cmul(Y[2], cscale(cmul(X[0], X[2]), two))), cmul(Y[5], a3));
    r.k[6] = cadd(cadd(cadd(cmul(Y[0], X[6]), cmul(Y[2], cscale(cadd(cmul(X[0], X[3]), cmul(X[1], X[2])), two))),
                       cadd(cmul(Y[3], X[2]), cmul(Y[5], cscale(a2b, three)))),
                  cmul(Y[6], a2));
    r.k[7] = cadd(cadd(cadd(cmul(Y[0], X[7]), cmul(Y[2], cscale(cadd(cmul(X[0], X[4]), cmul(X[1], X[3])), two))),
                       cadd(cmul(Y[3], X[3]), cmul(Y[5], cscale(ab2, three)))),
                  cadd(cmul(Y[6], cscale(ab, two)), cmul(Y[7], X[0])));
    r.k[8] = cadd(cadd(cadd(cmul(Y[0], X[8]), cmul(Y[2], cscale(cmul(X[1], X[4]), two))),
                       cadd(cmul(Y[3], X[4]), cmul(Y[5], b3))),
                  cadd(cmul(Y[6], b2), cadd(cmul(Y[7], X[1]), Y[8])));
    r.r2 = sq(composed_radius(x.r2, y.r2, root(cnorm(X[0])), root(cnorm(X[1])), in));
    r.len = x.len + y.len;
    return r;
}

std::vector<std::vector<Linear>> linear_levels(const Reference& R, int count, const FE& in) {
    const FE tol = fe(ldexp2(1.0, -38), 0), two = fe(2.0, 0);
    std::vector<std::vector<BLinear>> lv(1, std::vector<BLinear>(static_cast<std::size_t>(count)));
    for (int s = 1; s <= count; ++s) {
        const FC& Z = R.builder[static_cast<std::size_t>(s)];
        lv[0][static_cast<std::size_t>(s - 1)] = {cscale(Z, two), {fe(1.0, 0), {}}, sq(mul(tol, root(cnorm(Z)))), 1};
    }
    for (std::size_t L = 1; (1u << L) <= 4096u; ++L) {
        const auto& p = lv[L - 1];
        std::size_t n = (p.size() + 1) / 2;
        if (n == 0) break;
        std::vector<BLinear> cur(n);
        for (std::size_t i = 0; i < n; ++i) {
            if (2 * i + 1 < p.size()) {
                const BLinear &x = p[2 * i], &y = p[2 * i + 1];
                cur[i] = {cmul(y.a, x.a), cadd(cmul(y.a, x.b), y.b),
                          sq(composed_radius(x.r2, y.r2, root(cnorm(x.a)), root(cnorm(x.b)), in)), x.len + y.len};
            } else {
                cur[i] = p[2 * i];
            }
        }
        lv.push_back(std::move(cur));
    }
    std::vector<std::vector<Linear>> out;
    for (const auto& level : lv) {
        std::vector<Linear> dst;
        for (const BLinear& s : level) {
            bool fin = ok(s.r2) && cok(s.a) && cok(s.b);
            dst.push_back({from_fc(s.a.r, s.a.i), from_fc(s.b.r, s.b.i), fin ? s.r2 : FE{}, s.len});
        }
        out.push_back(std::move(dst));
    }
    return out;
}

void tables(Reference& R) {
    const int mi = static_cast<int>(R.builder.size()) - 1;
    const int count = std::max(0, std::min(mi, std::clamp(R.map_end, 0, mi)) - 1);
    image_series(R, R.builder);
    R.cubic.clear();
    R.linear.clear();
    R.deep.clear();
    if (count == 0) return;
    const FE tol = fe(ldexp2(1.0, -38), 0), two = fe(2.0, 0);
    std::vector<std::vector<BCubic>> lv(1, std::vector<BCubic>(static_cast<std::size_t>(count)));
    for (int s = 1; s <= count; ++s) {
        const FC& Z = R.builder[static_cast<std::size_t>(s)];
        BCubic b{};
        b.k[0] = cscale(Z, two);
        b.k[1] = {fe(1.0, 0), {}};
        b.k[2] = {fe(1.0, 0), {}};
        b.r2 = sq(mul(tol, root(cnorm(Z))));
        b.len = 1;
        lv[0][static_cast<std::size_t>(s - 1)] = b;
    }
    for (std::size_t L = 1; (1u << L) <= 64u; ++L) {
        const auto& p = lv[L - 1];
        std::size_t n = p.size() / 2;
        if (n == 0) break;
        std::vector<BCubic> cur(n);
        for (std::size_t i = 0; i < n; ++i) cur[i] = compose(p[2 * i + 1], p[2 * i], R.radius);
        lv.push_back(std::move(cur));
    }
    for (const auto& level : lv) {
        std::vector<Cubic> dst;
        for (const BCubic& s : level) {
            bool fin = ok(s.r2);
            Cubic c;
            for (int j = 0; j < 9; ++j) {
                fin = fin && cok(s.k[j]);
                c.k[static_cast<std::size_t>(j)] = from_fc(s.k[j].r, s.k[j].i);
            }
            c.r2 = fin ? s.r2 : FE{};
            c.len = s.len;
            dst.push_back(c);
        }
        R.cubic.push_back(std::move(dst));
    }
    R.deep_radius = mul(R.radius, 1.0e-20);
    R.linear = linear_levels(R, count, R.radius);
    R.deep = linear_levels(R, count, R.deep_radius);
}

FE retarget(const FE& xr2, const FE& yr2, const SC& xa, const SC& xb, const FE& in) {
    NM na = norm(xa), nb = norm(xb);
    FE r = composed_radius(xr2, yr2, root(FE{na.m, na.e}), root(FE{nb.m, nb.e}), in);
    return sq(mul(r, 1.0 - ldexp2(1.0, -40)));
}

// ------------------------------------------------------------ deep render
struct Options {
    FractalRenderOptions o;
};

template <typename Step>
const Step* find(const std::vector<std::vector<Step>>& lv, int start, const FE& dn, int max_len) {
    if (start <= 0 || max_len <= 0 || !ok(dn)) return nullptr;
    int base = lv.empty() ? 0 : static_cast<int>(lv[0].size());
    if (start > base) return nullptr;
    int top = std::min(31 - __builtin_clz(static_cast<unsigned>(max_len)), static_cast<int>(lv.size()) - 1);
    int off = start - 1;
    for (int L = top; L >= 0; --L) {
        if (off & ((1 << L) - 1)) continue;
        int idx = off >> L;
        if (idx >= static_cast<int>(lv[static_cast<std::size_t>(L)].size())) continue;
        const Step& s = lv[static_cast<std::size_t>(L)][static_cast<std::size_t>(idx)];
        if (s.len > 1 && ok(s.r2) && cmp(dn, s.r2) < 0) return &s;
    }
    return nullptr;
}

SC cubic_value(const Cubic& s, const SC& d, const SC& c, int order) {
    const auto& k = s.k;
    if (order <= 1) return sadd(smul(k[0], d), smul(k[1], c));
    if (order == 2) {
        return sadd(smul(d, sadd(k[0], sadd(smul(k[2], d), smul(k[3], c)))), smul(c, sadd(k[1], smul(k[4], c))));
    }
    SC dcub = sadd(sadd(smul(k[5], d), smul(k[6], c)), k[2]);
    SC ccub = sadd(k[3], smul(k[7], c));
    SC din = sadd(k[0], sadd(smul(d, dcub), smul(c, ccub)));
    SC cin = sadd(k[1], smul(c, sadd(k[4], smul(k[8], c))));
    return sadd(smul(d, din), smul(c, cin));
}

SC cubic_slope(const Cubic& s, const SC& d, const SC& c, const SC& dd, int order) {
    const auto& k = s.k;
    if (order <= 1) return sadd(smul(k[0], dd), k[1]);
    SC pd = sadd(k[0], sadd(stwice(smul(k[2], d)), smul(k[3], c)));
    SC pc = sadd(k[1], sadd(smul(k[3], d), stwice(smul(k[4], c))));
    if (order >= 3) {
        SC d2 = smul(d, d), c2 = smul(c, c);
        pd = sadd(pd, sadd(smul(sadd(stwice(smul(k[5], d)), smul(k[5], d)), d),
                           sadd(stwice(smul(k[6], smul(d, c))), smul(k[7], c2))));
        pc = sadd(pc, sadd(smul(k[6], d2),
                           sadd(stwice(smul(k[7], smul(d, c))), smul(sadd(stwice(smul(k[8], c)), smul(k[8], c)), c))));
    }
    return sadd(smul(pd, dd), pc);
}

// Kalles analytic DE |z| log|z| / (zhat conj(dz) spacing) (renderer.cpp:7844-7890).
bool de_value(const SC& total, const SC& der, const FE& spacing, double& ox, double& oy) {
    double mag = std::hypot(total.x, total.y);
    if (!(mag > 0.0) || !std::isfinite(mag)) return false;
    double lm = static_cast<double>(std::log(mag) + static_cast<double>(total.e) * LN2);
    if (!(lm > 0.0) || !std::isfinite(lm)) return false;
    SC unit = from_fc(fe(total.x / mag, 0), fe(total.y / mag, 0));
    SC den = smul(unit, smul(sconj(der), from_fc(spacing, FE{})));
    double d2 = den.x * den.x + den.y * den.y;
    if (!(d2 > 0.0) || !std::isfinite(d2)) return false;
    SC r{mag * lm * den.x / d2, -mag * lm * den.y / d2, clamp_exp(static_cast<long long>(total.e) - den.e)};
    fix(r);
    ox = sx(r);
    oy = sy(r);
    return std::isfinite(ox) && std::isfinite(oy);
}

struct PlaneSink {
    FractalRenderPlanes* p;
    void clear(std::size_t i, int max_iter) const {
        if (!p) return;
        p->orbit_iteration[i] = max_iter;
        p->phase[i] = p->de_x[i] = p->de_y[i] = p->test1[i] = p->test2[i] = 0.0;
    }
    void escape(std::size_t i, int raw, const SC& total, const NM& t1, const NM& t2, const SC& der,
                const FE& spacing) const {
        if (!p) return;
        p->orbit_iteration[i] = raw;
        double re = sx(total), im = sy(total), ph = 0.0;
        if (std::isfinite(re) && std::isfinite(im)) {
            ph = std::atan2(im, re) / TAU;
            ph -= std::floor(ph);
            if (!std::isfinite(ph)) ph = 0.0;
        }
        p->phase[i] = ph;
        p->de_x[i] = p->de_y[i] = 0.0;
        double ox = 0.0, oy = 0.0;
        if (de_value(total, der, spacing, ox, oy)) {
            p->de_x[i] = ox;
            p->de_y[i] = oy;
        }
        p->test1[i] = norm_double(t1);
        p->test2[i] = norm_double(t2);
    }
};

float encode(long double v, double bias) { return static_cast<float>(v - static_cast<long double>(bias)); }

float smooth(int it, const NM& n, double bias) {
    if (n.m == 0.0) return encode(it, bias);
    long double lm = 0.5L * (std::log(static_cast<long double>(n.m)) + static_cast<long double>(n.e) * LN2);
    if (!(lm > 0.0L) || !std::isfinite(lm)) return encode(it, bias);
    return encode(static_cast<long double>(it) - std::log(lm) / LN2, bias);
}

struct Pixel {
    const Reference& R;
    const FractalRenderOptions& o;
    const PlaneSink& planes;
    std::size_t index;
    SC dc;
    int max_iter;
    FE spacing;
    bool cycle;
    float out = 0.0f;
    SC der = ONE;

    // Direct scaled recurrence from the total once the pixel leaves the
    // reference (renderer.cpp:13053-13146, 13155-13250).
    void continue_exact(SC total, NM tn, int& it) {
        SC c = sadd(R.z[1], dc);
        SC tort{};
        int power = 1, length = 0;
        bool ready = false;
        int cmin = o.strict_cycle ? 2048 : 512, cmargin = o.strict_cycle ? 78 : 60;
        while (it < max_iter) {
            NM prior = tn;
            der = sadd(stwice(smul(total, der)), ONE);
            total = sadd(smul(total, total), c);
            ++it;
            tn = norm(total);
            if (escaped_norm(tn, o.escape_radius_mode)) {
                out = smooth(it, tn, o.output_bias);
                planes.escape(index, std::max(0, it - 1), total, tn, prior, der, spacing);
                return;
            }
            if (cycle && it >= cmin && (it & 31) == 0 && ncmp(tn, NM{0.75, 2}) < 0) {
                if (!ready) {
                    tort = total;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    NM dist = norm(ssub(total, tort));
                    if (dist.m == 0.0 || dist.e <= std::max(tn.e, 0) - cmargin) {
                        out = encode(max_iter, o.output_bias);
                        return;
                    }
                    if (++length >= power) {
                        tort = total;
                        power = std::min(power * 2, 1 << 20);
                        length = 0;
                    }
                }
            }
        }
        out = encode(max_iter, o.output_bias);
    }

    // Plain-double tail (renderer.cpp:12451-12669); true = pathological.
    bool tail(int& it, int& ref, SC delta, const NM& start_norm, bool& unresolved) {
        double cr = sx(dc), ci = ldexp2(dc.y, dc.e);
        double esc = static_cast<double>(o.escape_radius_mode == 1 ? 1.0e8L : 4.0L), safe = esc + 1.0e-7;
        double dr = sx(delta), di = ldexp2(delta.y, delta.e);
        out = encode(max_iter, o.output_bias);
        double tr0 = 0, ti0 = 0;
        int power = 1, length = 0, steps = 0, iters = 0, rebases = 0;
        NM prev = start_norm;
        bool ready = false;
        bool strict = o.strict != 0;
        const int n = static_cast<int>(R.zr.size());
        while (it < max_iter && ref >= 0 && ref + 1 < n) {
            double Zr = R.zr[static_cast<std::size_t>(ref)], Zi = R.zi[static_cast<std::size_t>(ref)];
            SC pt{Zr + dr, Zi + di, 0};
            fix(pt);
            der = sadd(stwice(smul(pt, der)), ONE);
            double lr = 2.0 * (Zr * dr - Zi * di), li = 2.0 * (Zr * di + Zi * dr);
            double qr = dr * dr - di * di, qi = 2.0 * dr * di;
            dr = lr + qr + cr;
            di = li + qi + ci;
            ++ref;
            ++it;
            if (++iters > 65536) {
                unresolved = true;
                out = strict ? NAN : encode(it, o.output_bias);
                return true;
            }
            double tr = R.zr[static_cast<std::size_t>(ref)] + dr, ti = R.zi[static_cast<std::size_t>(ref)] + di;
            double m2 = tr * tr + ti * ti;
            if (!std::isfinite(m2)) {
                unresolved = true;
                out = strict ? NAN : encode(it, o.output_bias);
                return false;
            }
            if (m2 > esc) {
                double mag = std::sqrt(std::max(m2, safe));
                out = encode(static_cast<long double>(it) - std::log(std::log(mag)) / static_cast<double>(LN2), o.output_bias);
                SC et{tr, ti, 0};
                fix(et);
                planes.escape(index, std::max(0, it - 1), et, norm_of_double(m2), prev, der, spacing);
                return false;
            }
            prev = norm_of_double(m2);
            double dm2 = dr * dr + di * di;
            ++steps;
            if (cycle && steps >= 64 && (steps & 31) == 0) {
                if (!ready) {
                    tr0 = tr;
                    ti0 = ti;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    double a = tr - tr0, b = ti - ti0, d2 = a * a + b * b;
                    int cmin = o.strict_cycle ? 2048 : 512;
                    double tol = o.strict_cycle ? 1.0e-24 : 1.0e-18;
                    if (it >= cmin && m2 < 3.0 && d2 <= tol * std::max(1.0, m2)) {
                        planes.clear(index, max_iter);
                        return false;
                    }
                    if (++length >= power) {
                        tr0 = tr;
                        ti0 = ti;
                        power = std::min(power * 2, 1 << 20);
                        length = 0;
                    }
                }
            }
            if (m2 < dm2) {
                dr = tr;
                di = ti;
                ref = 0;
                steps = 0;
                ready = false;
                if (++rebases > 64) {
                    unresolved = true;
                    out = strict ? NAN : encode(it, o.output_bias);
                    planes.clear(index, max_iter);
                    return true;
                }
            }
        }
        if (it < max_iter) {
            unresolved = true;
            out = strict ? NAN : encode(it, o.output_bias);
            planes.clear(index, max_iter);
        }
        return false;
    }

    void run(const std::vector<std::vector<Linear>>& lin_levels, bool no_bla, bool series_ok, int order_cap,
             int bla_len, int lin_len) {
        planes.clear(index, max_iter);
        SC delta = dc;
        der = ONE;
        int ref = 1, it = 1;
        if (series_ok && ncmp(norm(dc), NM{R.series_r2.m, R.series_r2.e}) <= 0) {
            SC v = R.series.back(), pd{};
            for (std::size_t k = R.series.size() - 1; k > 1; --k) {
                pd = sadd(smul(pd, dc), v);
                v = sadd(smul(v, dc), R.series[k - 1]);
            }
            der = sadd(smul(pd, dc), v);
            delta = smul(v, dc);
            ref = it = R.series_it;
        }
        bool done = false, have = false, unresolved = false, no_pixel_bla = false;
        SC total{};
        NM tn{}, prev_tn{};
        FE margin{};
        SC tort{};
        int power = 1, length = 0, rebases = 0;
        bool ready = false;
        const int mode = o.escape_radius_mode;
        const int cmin = o.strict_cycle ? 2048 : 512, cmargin = o.strict_cycle ? 78 : 60;
        const int n = static_cast<int>(R.z.size());
        while (it < max_iter) {
            if (ref < 0 || ref >= n) {
                out = encode(it, o.output_bias);
                planes.escape(index, std::max(0, it - 1), total, tn, prev_tn, der, spacing);
                done = true;
                break;
            }
            const SC& Z = R.z[static_cast<std::size_t>(ref)];
            if (!have) {
                total = sadd(Z, delta);
                margin = margin_sc(Z, delta, mode);
                tn = norm_with_margin(margin, mode);
            }
            have = false;
            NM zn = norm(Z);
            FE zf{zn.m, zn.e};
            if (zf.m != 0.0 && ok(zf) && cmp(FE{tn.m, tn.e}, mul(zf, 1.0e-7)) < 0) {
                if (o.allow_recovery && sok(total) && ++rebases <= 64) {
                    delta = total;
                    ref = 0;
                    continue;
                }
                out = NAN;
                unresolved = true;
                break;
            }
            if (escaped_norm(tn, mode) || cmp(margin, FE{}) > 0) {
                out = smooth(it, tn, o.output_bias);
                planes.escape(index, std::max(0, it - 1), total, tn, prev_tn, der, spacing);
                done = true;
                break;
            }
            if (cycle && it >= cmin && (it & 31) == 0 && ncmp(tn, NM{0.75, 2}) < 0) {
                if (!ready) {
                    tort = total;
                    power = 1;
                    length = 0;
                    ready = true;
                } else {
                    NM dist = norm(ssub(total, tort));
                    if (dist.m == 0.0 || dist.e <= std::max(tn.e, 0) - cmargin) {
                        out = encode(max_iter, o.output_bias);
                        done = true;
                        break;
                    }
                    if (++length >= power) {
                        tort = total;
                        power = std::min(power * 2, 1 << 20);
                        length = 0;
                    }
                }
            }
            NM dn = norm(delta);
            if (ncmp(tn, dn) < 0) {
                if (++rebases > 64) {
                    continue_exact(total, tn, it);
                    done = true;
                    break;
                }
                delta = total;
                ref = 0;
                continue;
            }
            if (R.map_end > 1 && ref >= R.map_end) {
                continue_exact(total, tn, it);
                done = true;
                break;
            }
            const FE dnf{dn.m, dn.e};
            const int remaining = max_iter - it;
            const int order = order_cap >= 3 && dn.e < -115 ? (dn.e < -160 ? 1 : 2) : order_cap;
            const Linear* ls = nullptr;
            const Cubic* cs = nullptr;
            const bool bla = !no_bla && !no_pixel_bla;
            if (bla) {
                if (order <= 1) ls = find(lin_levels, ref, dnf, std::min(lin_len, remaining));
                else cs = find(R.cubic, ref, dnf, std::min(bla_len, remaining));
            }
            const int len = ls ? ls->len : (cs ? cs->len : 0);
            if (bla && (len <= 0 || ref + len > max_iter) && dn.e > -90) {
                bool tail_unresolved = false;
                const bool pathological = tail(it, ref, delta, tn, tail_unresolved);
                if (tail_unresolved) {
                    unresolved = true;
                    break;
                }
                if (pathological) {
                    delta = dc;
                    der = ONE;
                    ref = 1;
                    it = 1;
                    have = false;
                    no_pixel_bla = true;
                    continue;
                }
                done = true;
                break;
            }
            if (len > 0 && ref + len <= max_iter) {
                const SC d0 = delta, g0 = der;
                const int r0 = ref, i0 = it;
                delta = ls ? sadd(smul(ls->a, d0), smul(ls->b, dc)) : cubic_value(*cs, d0, dc, order);
                der = ls ? sadd(smul(ls->a, g0), ls->b) : cubic_slope(*cs, d0, dc, g0, order);
                ref += len;
                it += len;
                const SC& Zn = R.z[static_cast<std::size_t>(ref)];
                SC end = sadd(Zn, delta);
                FE em = margin_sc(Zn, delta, mode);
                NM en = norm_with_margin(em, mode);
                if (!sok(delta) || !sok(end)) {
                    delta = d0;
                    der = g0;
                    ref = r0;
                    it = i0;
                    no_pixel_bla = true;
                    continue;
                }
                if (ncmp(en, NM{0.75, 2}) >= 0) {
                    delta = d0;
                    der = g0;
                    ref = r0;
                    it = i0;
                    SC rt{};
                    NM rn{};
                    FE rm{};
                    bool retry = false, esc = false;
                    for (int k = 0; k < len && it < max_iter; ++k) {
                        const SC& Zk = R.z[static_cast<std::size_t>(ref)];
                        der = sadd(stwice(smul(sadd(Zk, delta), der)), ONE);
                        delta = sadd(stwice(smul(Zk, delta)), sadd(smul(delta, delta), dc));
                        ++ref;
                        ++it;
                        const SC& Zk1 = R.z[static_cast<std::size_t>(ref)];
                        rt = sadd(Zk1, delta);
                        rm = margin_sc(Zk1, delta, mode);
                        rn = norm_with_margin(rm, mode);
                        if (!sok(delta) || !sok(rt)) {
                            retry = true;
                            break;
                        }
                        if (escaped_norm(rn, mode) || cmp(rm, FE{}) > 0) {
                            out = smooth(it, rn, o.output_bias);
                            planes.escape(index, std::max(0, it - 1), rt, rn, tn, der, spacing);
                            esc = true;
                            break;
                        }
                    }
                    if (esc) {
                        done = true;
                        break;
                    }
                    if (retry) {
                        delta = d0;
                        der = g0;
                        ref = r0;
                        it = i0;
                        no_pixel_bla = true;
                        continue;
                    }
                    total = rt;
                    tn = rn;
                    margin = rm;
                } else {
                    total = end;
                    tn = en;
                    margin = em;
                }
                prev_tn = tn;
                have = true;
                continue;
            }
            prev_tn = tn;
            der = sadd(stwice(smul(sadd(Z, delta), der)), ONE);
            delta = sadd(stwice(smul(Z, delta)), sadd(smul(delta, delta), dc));
            ++ref;
            ++it;
        }
        if (!done && !unresolved) out = encode(max_iter, o.output_bias);
    }
};

}  // namespace oracle

// ------------------------------------------------------------ ABI layer
namespace oracle {

FractalRenderOptions defaults() {
    FractalRenderOptions o{};
    o.struct_size = sizeof o;
    o.version = 2;
    o.strict = 1;
    o.series_min_terms = 8;
    o.series_max_terms = 32;
    o.max_bla_length = 64;
    o.max_linear_bla_length = 4096;
    return o;
}

FractalRenderOptions checked(const FractalRenderOptions* in) {
    FractalRenderOptions o = defaults();
    if (!in) return o;
    if (in->struct_size < sizeof(FractalRenderOptions) || in->version != 2)
        throw Oops("unsupported FractalRenderOptions version or size");
    o = *in;
    for (int v : {o.strict, o.allow_recovery, o.disable_bla, o.disable_cycle, o.strict_cycle})
        if (v != 0 && v != 1) throw Oops("render flag must be 0 or 1");
    if ((o.escape_radius_mode != 0 && o.escape_radius_mode != 1) || (o.coordinate_mode != 0 && o.coordinate_mode != 1))
        throw Oops("unknown escape-radius or coordinate mode");
    o.series_min_terms = std::clamp(o.series_min_terms, 1, 32);
    o.series_max_terms = std::clamp(o.series_max_terms, o.series_min_terms, 32);
    o.max_bla_length = std::clamp(o.max_bla_length, 1, 64);
    o.max_linear_bla_length = std::clamp(o.max_linear_bla_length, 1, 4096);
    if (o.time_budget_ms < 0 || !std::isfinite(o.output_bias) || o.output_bias < 0.0)
        throw Oops("invalid render options");
    return o;
}

bool dims_ok(int w, int h) {
    return w > 0 && h > 0 && static_cast<unsigned long long>(w) <= 100000000ULL / static_cast<unsigned long long>(h);
}

std::shared_ptr<Reference> lookup(void* h) {
    std::lock_guard<std::mutex> lock(table_mutex);
    auto it = table.find(reinterpret_cast<std::uintptr_t>(h));
    return it == table.end() ? nullptr : it->second;
}

void* add_reference(std::shared_ptr<Reference> r) {
    std::lock_guard<std::mutex> lock(table_mutex);
    std::uintptr_t id = next_id++;
    table.emplace(id, std::move(r));
    return reinterpret_cast<void*>(id);
}

void* create(const char* x, const char* y, const char* z, int max_iter, int bits, int order, int formula,
             const FractalRenderOptions* in, bool retain) {
    if (!x || !y || !z || max_iter <= 0 || max_iter > 10000000 || bits < 128 || bits > 131072 || order < 1 ||
        order > 32)
        throw Oops("invalid reference configuration");
    if (formula != 0) throw Oops("the oracle port restates the Mandelbrot deep path only");
    FractalRenderOptions o = checked(in);
    (void)zoom_of(z, bits);
    auto R = std::make_shared<Reference>();
    R->xc = parse_ld(x, "real");
    R->yc = parse_ld(y, "imaginary");
    R->escape_mode = o.escape_radius_mode;
    R->coordinate_mode = o.coordinate_mode;
    R->series_request = std::clamp(order, 8, 32);
    orbit(*R, x, y, z, max_iter, bits);
    tables(*R);
    if (!retain) R->builder.clear();
    return add_reference(std::move(R));
}

void* clone(void* source, const char* z) {
    auto S = lookup(source);
    if (!S) throw Oops("invalid or already-destroyed reference handle");
    if (S->builder.empty()) throw Oops("reference was not created as a reusable tier root");
    auto R = std::make_shared<Reference>(*S);
    R->builder.clear();
    FE zoom = zoom_of(z, R->bits);
    R->radius = divide(fe(height_factor(R->coordinate_mode), 0), zoom);
    image_series(*R, S->builder);
    for (auto* lv : {&R->cubic}) {
        for (std::size_t L = 1; L < lv->size(); ++L)
            for (std::size_t i = 0; i < (*lv)[L].size(); ++i) {
                const Cubic &x = (*lv)[L - 1][2 * i], &y = (*lv)[L - 1][2 * i + 1];
                (*lv)[L][i].r2 = retarget(x.r2, y.r2, x.k[0], x.k[1], R->radius);
            }
    }
    auto relink = [](std::vector<std::vector<Linear>>& lv, const FE& in) {
        for (std::size_t L = 1; L < lv.size(); ++L)
            for (std::size_t i = 0; i < lv[L].size(); ++i) {
                if (2 * i + 1 >= lv[L - 1].size()) {
                    lv[L][i].r2 = lv[L - 1][2 * i].r2;
                    continue;
                }
                const Linear &x = lv[L - 1][2 * i], &y = lv[L - 1][2 * i + 1];
                lv[L][i].r2 = retarget(x.r2, y.r2, x.a, x.b, in);
            }
    };
    relink(R->linear, R->radius);
    R->deep_radius = mul(R->radius, 1.0e-20);
    R->deep = S->linear;
    relink(R->deep, R->deep_radius);
    return add_reference(std::move(R));
}

void deep(const Reference& R, float* out, int W, int H, const char* zs, int max_iter, int threads, int order,
          int block, const FractalRenderOptions& o, FractalRenderPlanes* planes,
          const std::vector<SC>* points = nullptr, const FE* point_radius = nullptr) {
    FE zoom = zoom_of(zs, R.bits);
    FE inv = divide(fe(1.0, 0), zoom);
    double hf = height_factor(o.coordinate_mode);
    FE vh = mul(inv, hf), vw = mul(vh, static_cast<double>(W) / static_cast<double>(H));
    FE spacing = divide(vh, fe(static_cast<double>(H), 0));
    FE cur = point_radius ? *point_radius : mul(inv, hf);
    bool no_bla = cmp(cur, R.radius) > 0 || o.disable_bla != 0;
    bool cyc = o.disable_cycle == 0 && (o.strict == 0 || o.strict_cycle != 0);
    bool use_deep = cmp(cur, R.deep_radius) <= 0;
    bool ultra = cmp(cur, mul(R.radius, 1.0e-40)) <= 0;
    int bla_len = std::clamp(std::min(block, o.max_bla_length), 2, 64);
    int lin_len = std::clamp(std::min(block, o.max_linear_bla_length), 2, ultra ? 4096 : (use_deep ? 1024 : 64));
    int oc = std::clamp(order, 1, 3);
    bool series_ok = R.series_on && R.series_order >= o.series_min_terms && R.series_order <= o.series_max_terms &&
                     cmp(cur, root(R.series_r2)) <= 0 && R.series_it < max_iter;
    std::vector<FE> xo(static_cast<std::size_t>(W)), yo(static_cast<std::size_t>(H));
    for (int py = 0; py < H; ++py) yo[static_cast<std::size_t>(py)] = mul(vh, -axis(py, H, o.coordinate_mode) / static_cast<double>(H));
    for (int px = 0; px < W; ++px) xo[static_cast<std::size_t>(px)] = mul(vw, axis(px, W, o.coordinate_mode) / static_cast<double>(W));
    const auto& lin = use_deep ? R.deep : R.linear;
    PlaneSink sink{planes};
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < static_cast<long long>(W) * H; ++i) {
        int py = static_cast<int>(i / W), px = static_cast<int>(i % W);
        const SC dc = points ? (*points)[static_cast<std::size_t>(i)]
                             : from_fc(xo[static_cast<std::size_t>(px)], yo[static_cast<std::size_t>(py)]);
        Pixel p{R, o, sink, static_cast<std::size_t>(i), dc, max_iter, spacing, cyc};
        p.run(lin, no_bla, series_ok, oc, bla_len, lin_len);
        out[i] = p.out;
    }
}

void direct(float* out, int W, int H, long double zoom, long double xc, long double yc, int max_iter, int threads,
            int formula, double jr, double ji, const FractalRenderOptions& o, FractalRenderPlanes* planes) {
    const double zv = static_cast<double>(zoom), cr0 = static_cast<double>(xc), ci0 = static_cast<double>(yc);
    const double hs = height_factor(o.coordinate_mode) / zv, ws = hs * static_cast<double>(W) / static_cast<double>(H);
    const double esc = o.escape_radius_mode == 1 ? 1.0e8 : 4.0, safe = esc + 1.0e-7;
    const double lp = std::log(2.0);
    const bool need_phase = (static_cast<unsigned>(o.reserved[0]) & 1u) == 0;
    const bool need_de = (static_cast<unsigned>(o.reserved[0]) & 2u) == 0 && (formula == 0 || formula == 1);
    const FE spacing = fe(hs / static_cast<double>(H), 0);
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int py = 0; py < H; ++py) {
        const double cy = ci0 + (-axis(py, H, o.coordinate_mode) * hs / static_cast<double>(H));
        for (int px = 0; px < W; ++px) {
            const double cx = cr0 + axis(px, W, o.coordinate_mode) * ws / static_cast<double>(W);
            const std::size_t i = static_cast<std::size_t>(py) * W + px;
            auto inside = [&] {
                out[i] = encode(max_iter, o.output_bias);
                if (planes) {
                    planes->orbit_iteration[i] = max_iter;
                    planes->phase[i] = planes->de_x[i] = planes->de_y[i] = planes->test1[i] = planes->test2[i] = 0.0;
                }
            };
            if (formula == 0) {
                double q = (cx - 0.25) * (cx - 0.25) + cy * cy;
                if (q * (q + cx - 0.25) <= 0.25 * cy * cy || (cx + 1.0) * (cx + 1.0) + cy * cy <= 0.0625) {
                    inside();
                    continue;
                }
            }
            double zr = formula == 1 ? cx : 0.0, zi = formula == 1 ? cy : 0.0;
            const double pr = formula == 1 ? jr : cx, pi = formula == 1 ? ji : cy;
            double dr = formula == 1 ? 1.0 : 0.0, di = 0.0, t1 = 0.0, t2 = 0.0;
            const double add_re = formula == 1 ? 0.0 : 1.0;
            int it = 0;
            for (; it < max_iter; ++it) {
                if (planes && need_de) {
                    double ndr = 2.0 * zr * dr - 2.0 * zi * di + add_re;
                    double ndi = 2.0 * zr * di + 2.0 * zi * dr + 0.0;
                    dr = ndr;
                    di = ndi;
                }
                double nr, ni;
                if (formula == 2) {
                    double ar = std::fabs(zr), ai = std::fabs(zi);
                    double a2 = ar * ar, b2 = ai * ai, cr = 2.0 * ar * ai;
                    nr = (a2 - b2) + pr;
                    ni = cr + pi;
                } else if (formula == 3) {
                    double a2 = zr * zr, b2 = zi * zi, cr = -2.0 * zr * zi;
                    nr = (a2 - b2) + pr;
                    ni = cr + pi;
                } else {
                    nr = zr * zr - zi * zi + pr;
                    ni = 2.0 * zr * zi + pi;
                }
                zr = nr;
                zi = ni;
                double m2 = zr * zr + zi * zi;
                t2 = t1;
                t1 = m2;
                if (m2 > esc || !std::isfinite(m2)) {
                    double mag = std::sqrt(std::isfinite(m2) ? std::max(m2, safe) : std::numeric_limits<double>::max());
                    out[i] = encode(static_cast<long double>(it + 1) - std::log(std::log(mag)) / lp, o.output_bias);
                    if (planes) {
                        planes->orbit_iteration[i] = it;
                        double ph = 0.0;
                        if (need_phase && std::isfinite(zr) && std::isfinite(zi)) {
                            ph = std::atan2(zi, zr) / TAU;
                            ph -= std::floor(ph);
                        }
                        planes->phase[i] = ph;
                        planes->de_x[i] = planes->de_y[i] = 0.0;
                        if (need_de && std::isfinite(zr) && std::isfinite(zi) && std::isfinite(dr) && std::isfinite(di)) {
                            double ox = 0.0, oy = 0.0;
                            if (de_value(from_fc(fe(zr, 0), fe(zi, 0)), from_fc(fe(dr, 0), fe(di, 0)), spacing, ox, oy)) {
                                planes->de_x[i] = ox;
                                planes->de_y[i] = oy;
                            }
                        }
                        planes->test1[i] = t1;
                        planes->test2[i] = t2;
                    }
                    break;
                }
            }
            if (it == max_iter) inside();
        }
    }
}

long double zoom_direct(const char* s) {
    if (!text_ok(s)) throw Oops("native zoom text is too long or null");
    std::istringstream in(s);
    in.imbue(std::locale::classic());
    long double v = 0;
    in >> v;
    bool good = !in.fail();
    in >> std::ws;
    if (!good || !in.eof() || !std::isfinite(v) || v <= 0) throw Oops("invalid Mandelbrot zoom");
    return v;
}

template <typename F>
int status_of(F&& f) {
    try {
        f();
        error_text.clear();
        return 0;
    } catch (const std::exception& e) {
        error_text = e.what();
        return 1;
    }
}

template <typename F>
void* handle_of(F&& f) {
    try {
        void* h = f();
        error_text.clear();
        return h;
    } catch (const std::exception& e) {
        error_text = e.what();
        return nullptr;
    }
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int fractal_abi_version(void) { return 10; }
int fractal_render_options_version(void) { return 2; }
void fractal_render_options_default(FractalRenderOptions* o) {
    if (o) *o = defaults();
}
int fractal_backend_capabilities(void) { return 1; }
const char* fractal_last_error(void) { return error_text.c_str(); }
void fractal_set_stats_enabled(int) {}
int fractal_get_last_stats(uint64_t* v, int n) {
    if (!v || n < 16) return -1;
    std::fill(v, v + 16, 0);
    return 16;
}
int fractal_get_last_stats_ex(uint64_t* v, int n) {
    if (!v || n < 39) return -1;
    std::fill(v, v + 39, 0);
    return 39;
}

void* fractal_create_reference(const char* x, const char* y, const char* z, int m, int b, int s) {
    return handle_of([&] { return create(x, y, z, m, b, s, 0, nullptr, false); });
}
void* fractal_create_reference_reusable(const char* x, const char* y, const char* z, int m, int b, int s) {
    return handle_of([&] { return create(x, y, z, m, b, s, 0, nullptr, true); });
}
void* fractal_create_reference_reusable_options(const char* x, const char* y, const char* z, int m, int b, int s,
                                                const FractalRenderOptions* o) {
    return handle_of([&] { return create(x, y, z, m, b, s, 0, o, true); });
}
void* fractal_create_reference_ex(const char* x, const char* y, const char* z, int m, int b, int s, int f,
                                  const char*, const char*) {
    return handle_of([&] { return create(x, y, z, m, b, s, f, nullptr, f != 0); });
}
void* fractal_create_reference_ex_options(const char* x, const char* y, const char* z, int m, int b, int s, int f,
                                          const char*, const char*, const FractalRenderOptions* o) {
    return handle_of([&] { return create(x, y, z, m, b, s, f, o, f != 0); });
}
void* fractal_clone_reference(void* h, const char* z) {
    return handle_of([&] { return clone(h, z); });
}
void fractal_destroy_reference(void* h) {
    std::lock_guard<std::mutex> lock(table_mutex);
    if (h && table.erase(reinterpret_cast<std::uintptr_t>(h)) == 0) {
        error_text = "invalid or already-destroyed reference handle";
    } else {
        error_text.clear();
    }
}
int fractal_get_reference_stats(void* h, uint64_t* v, int n) {
    auto R = lookup(h);
    if (!R || !v || n < 5) return -1;
    v[0] = v[1] = v[2] = 0;
    v[3] = R->series_on ? static_cast<uint64_t>(R->series_it) : 0;
    v[4] = R->series_on ? static_cast<uint64_t>(R->series_order) : 0;
    return 5;
}

int fractal_render_reference_ex_planes(float* out, int W, int H, const char* z, void* h, int max_iter, int threads,
                                       int order, int block, const FractalRenderOptions* in, FractalRenderPlanes* planes) {
    return status_of([&] {
        if (!out || !z || !h || !dims_ok(W, H) || max_iter <= 0) throw Oops("invalid native render dimensions or handle");
        FractalRenderOptions o = checked(in);
        auto R = lookup(h);
        if (!R) throw Oops("invalid or already-destroyed reference handle");
        if (max_iter > R->max_iter) throw Oops("render iteration count exceeds prepared reference");
        FE zoom = zoom_of(z, R->bits);
        long double lz = (std::log(std::fabs(static_cast<long double>(zoom.m))) + zoom.e * LN2) / std::log(10.0L);
        if (lz >= 6.0L) {
            deep(*R, out, W, H, z, max_iter, threads, order, block, o, planes);
        } else {
            direct(out, W, H, zoom_direct(z), R->xc, R->yc, max_iter, threads, 0, 0.0, 0.0, o, planes);
        }
    });
}
int fractal_render_reference_ex(float* out, int W, int H, const char* z, void* h, int m, int t, int s, int b,
                                const FractalRenderOptions* o) {
    return fractal_render_reference_ex_planes(out, W, H, z, h, m, t, s, b, o, nullptr);
}

int render_fractal_ex_planes(float* out, int W, int H, const char* z, const char* x, const char* y, int max_iter,
                             int bits, int use_perturbation, int threads, int formula, double jr, double ji,
                             const FractalRenderOptions* in, FractalRenderPlanes* planes) {
    return status_of([&] {
        if (!out || !z || !x || !y || !dims_ok(W, H) || max_iter <= 0 || formula < 0 || formula > 3)
            throw Oops("invalid native render dimensions, formula, or argument");
        FractalRenderOptions o = checked(in);
        if (!use_perturbation) {
            direct(out, W, H, zoom_direct(z), parse_ld(x, "real"), parse_ld(y, "imaginary"), max_iter, threads, formula, jr,
                   ji, o, planes);
            return;
        }
        void* h = create(x, y, z, max_iter, bits, 8, formula, &o, false);
        int st = fractal_render_reference_ex_planes(out, W, H, z, h, max_iter, threads, 8, 32, &o, planes);
        std::string e = error_text;
        fractal_destroy_reference(h);
        if (st != 0) throw Oops(e);
    });
}
int render_fractal_ex(float* out, int W, int H, const char* z, const char* x, const char* y, int m, int b, int u,
                      int t, int f, double jr, double ji, const FractalRenderOptions* o) {
    return render_fractal_ex_planes(out, W, H, z, x, y, m, b, u, t, f, jr, ji, o, nullptr);
}

}  // extern "C"

namespace oracle {

// aurora_palette_for (renderer.cpp:4841-4923), with the optional three-accent
// projection (:4883-4911).
std::vector<uint8_t> aurora_table(int max_iter, double phase, double vocal, double pitch, const uint8_t* accents) {
    const int n = std::min(65536, std::max(4096, max_iter * 4));
    std::vector<uint8_t> lut(static_cast<std::size_t>(n) * 3);
    const double v = std::clamp(vocal, 0.0, 1.0), split = 5.0 * v * v;
    const double p[3] = {phase, phase + split * 0.4, phase + split};
    const double sp = std::clamp(2.0 * (pitch - 0.5), -1.0, 1.0), hue = sp * 0.16 * TAU;
    const bool rot = std::fabs(hue) > 1.0e-15;
    const double hc = rot ? std::cos(hue) : 1.0, hs = rot ? std::sin(hue) : 0.0;
    auto byte = [](double x) { return static_cast<uint8_t>(std::clamp(x, 0.0, 255.0)); };
    for (int k = 0; k < n; ++k) {
        double angle = 0.15 * static_cast<double>(max_iter) * static_cast<double>(k) / std::max(1, n - 1);
        double c = static_cast<float>(std::cos(angle)), s = static_cast<float>(std::sin(angle));
        double col[3];
        for (int j = 0; j < 3; ++j) col[j] = (0.5 - 0.5 * (c * std::cos(p[j]) + s * std::sin(p[j]))) * 140.0;
        if (accents) {
            double w[3];
            for (int j = 0; j < 3; ++j) w[j] = std::clamp(static_cast<double>(byte(col[j])) / 140.0, 0.0, 1.0);
            for (int j = 0; j < 3; ++j)
                col[j] = (w[0] * accents[j] + w[1] * accents[3 + j] + w[2] * accents[6 + j]) / 1.8;
        }
        if (rot) {
            double Y = 0.299 * col[0] + 0.587 * col[1] + 0.114 * col[2];
            double I = 0.596 * col[0] - 0.275 * col[1] - 0.321 * col[2];
            double Q = 0.212 * col[0] - 0.523 * col[1] + 0.311 * col[2];
            double ri = I * hc - Q * hs, rq = I * hs + Q * hc;
            col[0] = Y + 0.956 * ri + 0.621 * rq;
            col[1] = Y - 0.272 * ri - 0.647 * rq;
            col[2] = Y - 1.106 * ri + 1.703 * rq;
        }
        for (int j = 0; j < 3; ++j) lut[3 * static_cast<std::size_t>(k) + j] = byte(col[j]);
    }
    return lut;
}

// write_colour_pixel (renderer.cpp:5210-5237).
void aurora_pixel(float f, int cap, const std::vector<uint8_t>& lut, float scale, const int* interior, uint8_t* d) {
    const int n = static_cast<int>(lut.size() / 3);
    if (!std::isfinite(f) || f >= static_cast<float>(cap)) {
        for (int j = 0; j < 3; ++j) d[j] = interior ? static_cast<uint8_t>(interior[j]) : 0;
        return;
    }
    double x = static_cast<double>(f) * static_cast<double>(scale);
    int k = x >= static_cast<double>(n - 1) ? n - 1 : (!std::isfinite(x) || x <= 0.0 ? 0 : static_cast<int>(x));
    std::memcpy(d, &lut[3 * static_cast<std::size_t>(k)], 3);
}

bool colour_controls_ok(double a, double b, double c, double d) {
    return std::isfinite(a) && std::isfinite(b) && std::isfinite(c) && std::isfinite(d);
}

bool rgb_ok(const int* c) {
    return !c || (c[0] >= 0 && c[0] <= 255 && c[1] >= 0 && c[1] <= 255 && c[2] >= 0 && c[2] <= 255);
}

void colourise(const float* field, uint8_t* rgb, int W, int H, int max_iter, double phase, double vocal,
               double instrumental, double pitch, int threads, const int* interior, const uint8_t* accents) {
    if (!field || !rgb || !dims_ok(W, H) || max_iter <= 0 || !colour_controls_ok(phase, vocal, instrumental, pitch)
        || !rgb_ok(interior))
        throw Oops("invalid native colour dimensions or palette");
    const std::vector<uint8_t> lut = aurora_table(max_iter, phase, vocal, pitch, accents);
    const int n = static_cast<int>(lut.size() / 3);
    const float scale = static_cast<float>(n - 1) / static_cast<float>(max_iter);
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(W) * H; ++i) aurora_pixel(field[i], max_iter, lut, scale, interior, rgb + 3 * i);
}

// ------------------------------------------------------------------ atlas
// fill_bilinear_axis (renderer.cpp:4931-4961).
struct Axis {
    std::vector<int> i0, i1;
    std::vector<float> w;
};

Axis axis_of(int src, int dst, double zoom) {
    zoom = std::max(zoom, 1.0);
    const double crop = static_cast<double>(src) * (1.0 / zoom);
    const double left = (static_cast<double>(src) - crop) * 0.5, step = crop / static_cast<double>(dst);
    Axis a;
    for (int d = 0; d < dst; ++d) {
        double x = std::clamp(left + (static_cast<double>(d) + 0.5) * step - 0.5, 0.0, static_cast<double>(src - 1));
        int k = static_cast<int>(std::floor(x));
        a.i0.push_back(k);
        a.i1.push_back(std::min(k + 1, src - 1));
        a.w.push_back(static_cast<float>(x - static_cast<double>(k)));
    }
    return a;
}

// sample_bilinear_mapped_preserving_interior (renderer.cpp:5141-5208).
float sample(const float* f, int width, const Axis& ax, const Axis& ay, int x, int y, int cap, bool& inside,
             double bias) {
    const double xw = ax.w[x], yw = ay.w[y];
    const float v[4] = {f[static_cast<std::size_t>(ay.i0[y]) * width + ax.i0[x]],
                        f[static_cast<std::size_t>(ay.i0[y]) * width + ax.i1[x]],
                        f[static_cast<std::size_t>(ay.i1[y]) * width + ax.i0[x]],
                        f[static_cast<std::size_t>(ay.i1[y]) * width + ax.i1[x]]};
    const double w[4] = {(1.0 - yw) * (1.0 - xw), (1.0 - yw) * xw, yw * (1.0 - xw), yw * xw};
    double in = 0.0, out = 0.0, sum = 0.0;
    for (int k = 0; k < 4; ++k) {
        if (!std::isfinite(v[k])) continue;
        if (static_cast<double>(v[k]) >= static_cast<double>(cap) - bias) {
            in += w[k];
        } else {
            out += w[k];
            sum += (static_cast<double>(v[k]) + bias) * w[k];
        }
    }
    inside = in >= 0.5;
    if (inside) return static_cast<float>(cap);
    return out <= 1.0e-12 ? 0.0F : static_cast<float>(sum / out);
}

std::vector<float> ramp(int size, int feather) {
    std::vector<float> r(size);
    for (int i = 0; i < size; ++i) {
        float l = std::min(1.0F, static_cast<float>(std::min(i, size - 1 - i)) / static_cast<float>(feather));
        r[i] = l * l * (3.0F - 2.0F * l);
    }
    return r;
}

struct Frame {
    bool child = false, full = false;
    int vw = 0, vh = 0, left = 0, top = 0;
};

Frame frame_of(bool child, double fraction, int W, int H) {
    Frame f;
    f.child = child;
    f.full = child && fraction >= 0.999999;
    if (child) {
        f.vw = std::max(1, static_cast<int>(std::lround(static_cast<double>(W) * fraction)));
        f.vh = std::max(1, static_cast<int>(std::lround(static_cast<double>(H) * fraction)));
    }
    f.left = (W - f.vw) / 2;
    f.top = (H - f.vh) / 2;
    return f;
}

// fractal_atlas_field_ex (renderer.cpp:18697-18888).
void atlas_field(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap, float* out,
                 int W, int H, double pzoom, double fraction, double czoom, double pbias, double cbias, double obias,
                 int palette, int feather, int threads) {
    if (!P || !out || !dims_ok(pw, ph) || !dims_ok(W, H) || pcap <= 0 || !std::isfinite(pzoom) || pzoom <= 0.0
        || !std::isfinite(fraction) || fraction < 0.0 || fraction > 1.0 || !std::isfinite(czoom) || czoom <= 0.0
        || !std::isfinite(pbias) || pbias < 0.0 || pbias > pcap || !std::isfinite(cbias) || cbias < 0.0
        || !std::isfinite(obias) || obias < 0.0 || feather < 0 || palette <= 0)
        throw Oops("invalid native scalar atlas dimensions");
    const Frame f = frame_of(C != nullptr && fraction > 0.0, fraction, W, H);
    if (f.child && (!dims_ok(cw, chh) || ccap <= 0 || cbias > ccap)) throw Oops("invalid native scalar atlas child tile");
    const int cap = std::max(palette, std::max(pcap, f.child ? ccap : 0));
    if (obias > cap) throw Oops("invalid native scalar atlas iteration cap");
    const int seam = f.child && !f.full ? std::min(feather, std::min(f.vw / 2, f.vh / 2)) : 0;
    Axis px, py, cx, cy;
    if (!f.full) {
        px = axis_of(pw, W, pzoom);
        py = axis_of(ph, H, pzoom);
    }
    if (f.child) {
        cx = axis_of(cw, f.full ? W : f.vw, std::max(czoom, 1.0));
        cy = axis_of(chh, f.full ? H : f.vh, std::max(czoom, 1.0));
    }
    std::vector<float> ex, ey;
    if (seam >= 2) {
        ex = ramp(f.vw, seam);
        ey = ramp(f.vh, seam);
    }
    const float interior = static_cast<float>(cap - obias);
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            bool in = false;
            float v;
            if (f.full) {
                float s = sample(C, cw, cx, cy, x, y, ccap, in, cbias);
                v = in ? interior : s - static_cast<float>(obias);
            } else {
                float s = sample(P, pw, px, py, x, y, pcap, in, pbias);
                v = in ? interior : s - static_cast<float>(obias);
                if (f.child && x >= f.left && x < f.left + f.vw && y >= f.top && y < f.top + f.vh) {
                    bool cin = false;
                    float cs = sample(C, cw, cx, cy, x - f.left, y - f.top, ccap, cin, cbias);
                    float cv = cin ? interior : cs - static_cast<float>(obias);
                    float alpha = seam >= 2 ? std::min(ex[x - f.left], ey[y - f.top]) : 1.0F;
                    v = v * (1.0F - alpha) + cv * alpha;
                }
            }
            out[static_cast<std::size_t>(y) * W + x] = v;
        }
    }
}

// atlas_colourise_impl (renderer.cpp:19138-19430).
void atlas_colour(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap, uint8_t* out,
                  int W, int H, double pzoom, double fraction, int palette, double phase, double vocal,
                  double instrumental, double pitch, int threads, const int* interior, const uint8_t* accents) {
    if (!P || !out || !dims_ok(pw, ph) || !dims_ok(W, H) || pcap <= 0 || !std::isfinite(pzoom) || pzoom <= 0.0
        || !std::isfinite(fraction) || fraction < 0.0 || fraction > 1.0 || palette < 0
        || !colour_controls_ok(phase, vocal, instrumental, pitch) || !rgb_ok(interior))
        throw Oops("invalid native atlas dimensions or controls");
    const Frame f = frame_of(C != nullptr && fraction > 0.0, fraction, W, H);
    if (f.child && (!dims_ok(cw, chh) || ccap <= 0)) throw Oops("invalid native atlas child tile");
    const int cap = std::max(1, std::max(palette, std::max(pcap, f.child ? ccap : 0)));
    const std::vector<uint8_t> lut = aurora_table(cap, phase, vocal, pitch, accents);
    const float scale = static_cast<float>(static_cast<int>(lut.size() / 3) - 1) / static_cast<float>(cap);
    const int feather = f.child ? std::min(48, std::min(f.vw / 8, f.vh / 8)) : 0;
    Axis px, py, cx, cy;
    if (!f.full) {
        px = axis_of(pw, W, pzoom);
        py = axis_of(ph, H, pzoom);
    }
    if (f.child) {
        cx = axis_of(cw, f.full ? W : f.vw, 1.0);
        cy = axis_of(chh, f.full ? H : f.vh, 1.0);
    }
    std::vector<float> ex, ey;
    if (f.child && !f.full && feather >= 2) {
        ex = ramp(f.vw, feather);
        ey = ramp(f.vh, feather);
    }
    const float icap = static_cast<float>(cap);
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            uint8_t* d = out + (static_cast<std::size_t>(y) * W + x) * 3;
            bool in = false;
            if (f.full) {
                float s = sample(C, cw, cx, cy, x, y, ccap, in, 0.0);
                aurora_pixel(in ? icap : s, cap, lut, scale, interior, d);
                continue;
            }
            const bool inside_child = f.child && x >= f.left && x < f.left + f.vw && y >= f.top && y < f.top + f.vh;
            if (!inside_child) {
                float s = sample(P, pw, px, py, x, y, pcap, in, 0.0);
                aurora_pixel(in ? icap : s, cap, lut, scale, interior, d);
                continue;
            }
            bool cin = false;
            float cs = sample(C, cw, cx, cy, x - f.left, y - f.top, ccap, cin, 0.0);
            float alpha = feather >= 2 ? std::min(ex[x - f.left], ey[y - f.top]) : 1.0F;
            if (alpha >= 0.999999F) {
                aurora_pixel(cin ? icap : cs, cap, lut, scale, interior, d);
                continue;
            }
            float ps = sample(P, pw, px, py, x, y, pcap, in, 0.0);
            uint8_t a[3], b[3];
            aurora_pixel(in ? icap : ps, cap, lut, scale, interior, a);
            aurora_pixel(cin ? icap : cs, cap, lut, scale, interior, b);
            for (int j = 0; j < 3; ++j) {
                double v = static_cast<double>(a[j]) * (1.0 - alpha) + static_cast<double>(b[j]) * alpha;
                d[j] = static_cast<uint8_t>(std::clamp(static_cast<int>(std::nearbyint(std::clamp(v, 0.0, 255.0))), 0, 255));
            }
        }
    }
}

// fill_bilinear_axis_window (renderer.cpp:4969-5003).
Axis window_of(int src, int dst, double origin, double span, double zoom) {
    zoom = std::max(zoom, 1.0);
    const double crop = static_cast<double>(src) / zoom, left = (static_cast<double>(src) - crop) * 0.5;
    Axis a;
    for (int d = 0; d < dst; ++d) {
        const double logical = origin + static_cast<double>(d) + 0.5;
        double x = std::clamp(left + logical * crop / span - 0.5, 0.0, static_cast<double>(src - 1));
        int k = static_cast<int>(std::floor(x));
        a.i0.push_back(k);
        a.i1.push_back(std::min(k + 1, src - 1));
        a.w.push_back(static_cast<float>(x - static_cast<double>(k)));
    }
    return a;
}

// The scalar surface of fractal_atlas_colourise_kfp_raw (renderer.cpp:
// 18010-18288): parent view, child view with its halo, ownership blend.
void kfp_surface(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap, float* out,
                 int W, int H, double pzoom, double fraction, double czoom, int max_iter, double field_bias) {
    if (!P || !out || !dims_ok(pw, ph) || !dims_ok(W, H) || pcap <= 0 || max_iter <= 0 || !std::isfinite(pzoom)
        || pzoom <= 0.0 || !std::isfinite(fraction) || fraction < 0.0 || fraction > 1.0 || !std::isfinite(czoom)
        || czoom <= 0.0)
        throw Oops("invalid native raw KFP atlas dimensions or controls");
    pzoom = std::max(pzoom, 1.0);
    czoom = std::max(czoom, 1.0);
    const bool child = C != nullptr && fraction > 0.0;
    if (child && (!dims_ok(cw, chh) || ccap <= 0)) throw Oops("invalid native raw KFP atlas child tile");
    if (!child && C) throw Oops("raw KFP atlas child needs a positive visible fraction");
    if (!child && (cw || chh || ccap)) throw Oops("invalid native raw KFP atlas child absence");
    if (field_bias > max_iter) throw Oops("native KFP field bias exceeds iteration cap");
    const bool centred = field_bias > 0.0;
    const double pbias = centred ? pcap : 0.0, cbias = centred ? ccap : 0.0;
    auto enc = [&](long double v) { return static_cast<float>(v - static_cast<long double>(field_bias)); };
    const Frame f = frame_of(child, fraction, W, H);
    const int halo = child ? std::min(2, std::min(std::min(f.left, W - f.left - f.vw), std::min(f.top, H - f.top - f.vh))) : 0;
    int seam = 0;
    if (child) {
        const int m = std::min(f.vw, f.vh);
        seam = m <= 0 ? 0 : std::min(std::max(2, std::min(64, m / 2)), std::max(0, (m - 1) / 2));
    }
    const Axis px = axis_of(pw, W, pzoom), py = axis_of(ph, H, pzoom);
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            bool in = false;
            float s = sample(P, pw, px, py, x, y, pcap, in, pbias);
            out[static_cast<std::size_t>(y) * W + x] = in ? enc(max_iter) : enc(s);
        }
    }
    if (!child) return;
    const int sw = f.vw + 2 * halo, sh = f.vh + 2 * halo;
    const Axis cx = window_of(cw, sw, -halo, f.vw, czoom), cy = window_of(chh, sh, -halo, f.vh, czoom);
    std::vector<float> view(static_cast<std::size_t>(sw) * sh);
    for (int y = 0; y < sh; ++y) {
        for (int x = 0; x < sw; ++x) {
            bool in = false;
            float s = sample(C, cw, cx, cy, x, y, ccap, in, cbias);
            view[static_cast<std::size_t>(y) * sw + x] = in ? enc(max_iter) : enc(s);
        }
    }
    for (int y = f.top; y < f.top + f.vh; ++y) {
        for (int x = f.left; x < f.left + f.vw; ++x) {
            const float cv = view[static_cast<std::size_t>(y - f.top + halo) * sw + (x - f.left + halo)];
            float alpha = 1.0F;
            if (seam >= 2) {
                const int vx = x - f.left, vy = y - f.top;
                const int edge = std::min(std::min(vx, f.vw - 1 - vx), std::min(vy, f.vh - 1 - vy));
                const float l = std::clamp(static_cast<float>(edge) / static_cast<float>(seam), 0.0F, 1.0F);
                alpha = l * l * (3.0F - 2.0F * l);
            }
            float& o = out[static_cast<std::size_t>(y) * W + x];
            o = alpha >= 0.999999F ? cv : o * (1.0F - alpha) + cv * alpha;
        }
    }
}

// fractal_crop_colourise_kfp's scalar crop (renderer.cpp:17836-17868).
void crop_kfp_surface(const float* S, int sw, int sh, float* out, int W, int H, double zoom, int max_iter,
                      double field_bias) {
    if (!S || !out || !dims_ok(sw, sh) || !dims_ok(W, H) || max_iter <= 0 || !std::isfinite(zoom) || zoom <= 0.0)
        throw Oops("invalid native KFP crop dimensions or controls");
    if (field_bias > max_iter) throw Oops("native KFP field bias exceeds iteration cap");
    zoom = std::max(zoom, 1.0);
    const Axis ax = axis_of(sw, W, zoom), ay = axis_of(sh, H, zoom);
    auto enc = [&](long double v) { return static_cast<float>(v - static_cast<long double>(field_bias)); };
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            bool in = false;
            float s = sample(S, sw, ax, ay, x, y, max_iter, in, field_bias);
            out[static_cast<std::size_t>(y) * W + x] = in ? enc(max_iter) : enc(s);
        }
    }
}

// sample_bilinear_mapped (renderer.cpp:5053-5073) over a crop
// (fractal_crop_field, renderer.cpp:18631-18696).
void crop_field(const float* S, int sw, int sh, float* out, int W, int H, double zoom) {
    if (!S || !out || !dims_ok(sw, sh) || !dims_ok(W, H) || !std::isfinite(zoom) || zoom <= 0.0)
        throw Oops("invalid native raw-field crop dimensions");
    zoom = std::max(zoom, 1.0);
    const Axis ax = axis_of(sw, W, zoom), ay = axis_of(sh, H, zoom);
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const float* t = S + static_cast<std::size_t>(ay.i0[y]) * sw;
            const float* b = S + static_cast<std::size_t>(ay.i1[y]) * sw;
            const float xw = ax.w[x], yw = ay.w[y];
            const float tv = t[ax.i0[x]] * (1.0F - xw) + t[ax.i1[x]] * xw;
            const float bv = b[ax.i0[x]] * (1.0F - xw) + b[ax.i1[x]] * xw;
            out[static_cast<std::size_t>(y) * W + x] = tv * (1.0F - yw) + bv * yw;
        }
    }
}

uint8_t rounded_byte(double v) {
    return static_cast<uint8_t>(std::clamp(static_cast<int>(std::nearbyint(std::clamp(v, 0.0, 255.0))), 0, 255));
}

// sample_rgb_bilinear_mapped (renderer.cpp:5262-5298).
void rgb_sample(const uint8_t* S, int sw, const Axis& ax, const Axis& ay, int x, int y, uint8_t* d) {
    const uint8_t* t0 = S + (static_cast<std::size_t>(ay.i0[y]) * sw + ax.i0[x]) * 3;
    const uint8_t* t1 = S + (static_cast<std::size_t>(ay.i0[y]) * sw + ax.i1[x]) * 3;
    const uint8_t* b0 = S + (static_cast<std::size_t>(ay.i1[y]) * sw + ax.i0[x]) * 3;
    const uint8_t* b1 = S + (static_cast<std::size_t>(ay.i1[y]) * sw + ax.i1[x]) * 3;
    const float xw = ax.w[x], yw = ay.w[y], ix = 1.0F - xw, iy = 1.0F - yw;
    for (int c = 0; c < 3; ++c) {
        const float tv = static_cast<float>(t0[c]) * ix + static_cast<float>(t1[c]) * xw;
        const float bv = static_cast<float>(b0[c]) * ix + static_cast<float>(b1[c]) * xw;
        d[c] = rounded_byte(static_cast<double>(tv * iy + bv * yw));
    }
}

// fractal_atlas_composite_rgb (renderer.cpp:18467-18629); a null child with
// zero fraction is fractal_crop_rgb (renderer.cpp:18399-18465).
void composite_rgb(const uint8_t* P, int pw, int ph, const uint8_t* C, int cw, int chh, uint8_t* out, int W, int H,
                   double pzoom, double fraction, double czoom, int feather) {
    pzoom = std::max(pzoom, 1.0);
    czoom = std::max(czoom, 1.0);
    const bool child = C != nullptr && fraction > 0.0;
    const Frame f = frame_of(child, fraction, W, H);
    const int fe = child ? std::min(feather, std::min(f.vw, f.vh)) : 0;
    const Axis px = axis_of(pw, W, pzoom), py = axis_of(ph, H, pzoom);
    Axis cx, cy;
    if (child) {
        cx = axis_of(cw, f.vw, czoom);
        cy = axis_of(chh, f.vh, czoom);
    }
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            uint8_t* d = out + (static_cast<std::size_t>(y) * W + x) * 3;
            rgb_sample(P, pw, px, py, x, y, d);
            if (!child || x < f.left || x >= f.left + f.vw || y < f.top || y >= f.top + f.vh) continue;
            uint8_t c[3];
            rgb_sample(C, cw, cx, cy, x - f.left, y - f.top, c);
            double alpha = 1.0;
            if (fe >= 2) {
                const int e = std::min(std::min(x - f.left, f.vw - 1 - (x - f.left)),
                                       std::min(y - f.top, f.vh - 1 - (y - f.top)));
                const double l = std::clamp(static_cast<double>(e) / static_cast<double>(fe), 0.0, 1.0);
                alpha = l * l * (3.0 - 2.0 * l);
            }
            for (int k = 0; k < 3; ++k) d[k] = rounded_byte(static_cast<double>(d[k]) * (1.0 - alpha) + static_cast<double>(c[k]) * alpha);
        }
    }
}

// crop_colourise_impl (renderer.cpp:18977-19020).
void crop_colour(const float* S, int sw, int sh, uint8_t* out, int W, int H, double zoom, int max_iter, double phase,
                 double vocal, double instrumental, double pitch, const int* interior, const uint8_t* accents) {
    if (!S || !out || !dims_ok(sw, sh) || !dims_ok(W, H) || max_iter <= 0 || !std::isfinite(zoom) || zoom <= 0.0
        || !colour_controls_ok(phase, vocal, instrumental, pitch) || !rgb_ok(interior))
        throw Oops("invalid native crop/colour dimensions or palette");
    zoom = std::max(zoom, 1.0);
    const std::vector<uint8_t> lut = aurora_table(max_iter, phase, vocal, pitch, accents);
    const int n = static_cast<int>(lut.size() / 3);
    const float scale = static_cast<float>(n - 1) / static_cast<float>(max_iter);
    const Axis ax = axis_of(sw, W, zoom), ay = axis_of(sh, H, zoom);
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            uint8_t* d = out + (static_cast<std::size_t>(y) * W + x) * 3;
            bool in = false;
            const float s = sample(S, sw, ax, ay, x, y, max_iter, in, 0.0);
            if (in) {
                for (int j = 0; j < 3; ++j) d[j] = interior ? static_cast<uint8_t>(interior[j]) : 0;
                continue;
            }
            const double v = static_cast<double>(s) * static_cast<double>(scale);
            const int k = v >= static_cast<double>(n - 1) ? n - 1 : (!std::isfinite(v) || v <= 0.0 ? 0 : static_cast<int>(v));
            std::memcpy(d, &lut[3 * static_cast<std::size_t>(k)], 3);
        }
    }
}

}  // namespace oracle

extern "C" {
int oracle_crop_kfp_surface(const float* S, int sw, int sh, float* out, int W, int H, double zoom, int max_iter,
                            double field_bias) {
    return status_of([&] { crop_kfp_surface(S, sw, sh, out, W, H, zoom, max_iter, field_bias); });
}

int fractal_crop_field(const float* S, int sw, int sh, float* out, int W, int H, double zoom, int) {
    return status_of([&] { crop_field(S, sw, sh, out, W, H, zoom); });
}

int fractal_crop_rgb(const uint8_t* S, int sw, int sh, uint8_t* out, int W, int H, double zoom, int) {
    return status_of([&] {
        if (!S || !out || !dims_ok(sw, sh) || !dims_ok(W, H) || !std::isfinite(zoom) || zoom <= 0.0)
            throw Oops("invalid native RGB crop dimensions");
        composite_rgb(S, sw, sh, nullptr, 0, 0, out, W, H, zoom, 0.0, 1.0, 0);
    });
}

int fractal_atlas_composite_rgb(const uint8_t* P, int pw, int ph, const uint8_t* C, int cw, int chh, uint8_t* out,
                                int W, int H, double pzoom, double fraction, double czoom, int feather, int) {
    return status_of([&] {
        if (!P || !out || !dims_ok(pw, ph) || !dims_ok(W, H) || !std::isfinite(pzoom) || pzoom <= 0.0
            || !std::isfinite(fraction) || fraction < 0.0 || fraction > 1.0 || !std::isfinite(czoom) || czoom <= 0.0
            || feather < 0)
            throw Oops("invalid native RGB atlas dimensions or controls");
        const bool child = C != nullptr && fraction > 0.0;
        if (!child && fraction > 0.0) throw Oops("RGB atlas child data is missing for a positive fraction");
        if (!child && C) throw Oops("RGB atlas child needs a positive visible fraction");
        if (!child && (cw || chh)) throw Oops("invalid native RGB atlas child absence");
        if (child && (!dims_ok(cw, chh) || feather > std::min(W, H))) throw Oops("invalid native RGB atlas child tile");
        composite_rgb(P, pw, ph, C, cw, chh, out, W, H, pzoom, fraction, czoom, feather);
    });
}

int fractal_crop_colourise(const float* S, int sw, int sh, uint8_t* out, int W, int H, double zoom, int max_iter,
                           double phase, double vocal, double instrumental, double pitch, int) {
    return status_of([&] { crop_colour(S, sw, sh, out, W, H, zoom, max_iter, phase, vocal, instrumental, pitch, nullptr, nullptr); });
}

int fractal_crop_colourise_interior(const float* S, int sw, int sh, uint8_t* out, int W, int H, double zoom,
                                    int max_iter, double phase, double vocal, double instrumental, double pitch, int r,
                                    int g, int b, int) {
    const int interior[3] = {r, g, b};
    return status_of([&] { crop_colour(S, sw, sh, out, W, H, zoom, max_iter, phase, vocal, instrumental, pitch, interior, nullptr); });
}

int fractal_crop_colourise_accents(const float* S, int sw, int sh, uint8_t* out, int W, int H, double zoom,
                                   int max_iter, double phase, double vocal, double instrumental, double pitch,
                                   const uint8_t* accents, int r, int g, int b, int) {
    const int interior[3] = {r, g, b};
    return status_of([&] { crop_colour(S, sw, sh, out, W, H, zoom, max_iter, phase, vocal, instrumental, pitch, interior, accents); });
}

// fractal_render_points (renderer.cpp:20019-20186) for Mandelbrot references:
// the point list and its largest radius drive the same pixel loop.  The
// exact MPFR repair of strict glitch points is not restated here.
int fractal_render_points_ex_planes(float* out, int n, const char* z, const double* re, const double* im,
                                    const int32_t* ex, void* h, int max_iter, int threads, int order, int block,
                                    const FractalRenderOptions* opt, FractalRenderPlanes* planes) {
    return status_of([&] {
        if (!out || n <= 0 || !z || !re || !im || !ex || !h) throw Oops("invalid native point-render arguments");
        const FractalRenderOptions o = checked(opt);
        auto R = lookup(h);
        if (!R) throw Oops("invalid or already-destroyed reference handle");
        if (max_iter > R->max_iter) throw Oops("point render iteration count exceeds prepared reference");
        std::vector<SC> points(static_cast<std::size_t>(n));
        NM largest{};
        for (int i = 0; i < n; ++i) {
            SC p{re[i], im[i], ex[i]};
            if (!std::isfinite(p.x) || !std::isfinite(p.y)) throw Oops("non-finite point offset");
            fix(p);
            points[static_cast<std::size_t>(i)] = p;
            const NM r = norm(p);
            if (ncmp(r, largest) > 0) largest = r;
        }
        const FE radius = root(FE{largest.m, largest.e});
        deep(*R, out, n, 1, z, max_iter, threads, order, block, o, planes, &points, &radius);
    });
}

int fractal_render_points(float* out, int n, const char* z, const double* re, const double* im, const int32_t* ex,
                          void* h, int max_iter, int threads, int order, int block, const FractalRenderOptions* opt) {
    return fractal_render_points_ex_planes(out, n, z, re, im, ex, h, max_iter, threads, order, block, opt, nullptr);
}

// Test-only export: the raw KFP atlas surface (no reference symbol).
int oracle_atlas_kfp_surface(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap,
                             float* out, int W, int H, double pzoom, double fraction, double czoom, int max_iter,
                             double field_bias) {
    return status_of([&] { kfp_surface(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, czoom, max_iter, field_bias); });
}

int fractal_colourise(const float* field, uint8_t* rgb, int W, int H, int max_iter, double phase, double vocal,
                      double instrumental, double pitch, int threads) {
    return status_of([&] { colourise(field, rgb, W, H, max_iter, phase, vocal, instrumental, pitch, threads, nullptr, nullptr); });
}

int fractal_colourise_accents(const float* field, uint8_t* rgb, int W, int H, int max_iter, double phase,
                              double vocal, double instrumental, double pitch, const uint8_t* accents, int r, int g,
                              int b, int threads) {
    if (!accents) {
        error_text = "ordinary palette accents are required";
        return 1;
    }
    const int interior[3] = {r, g, b};
    return status_of([&] { colourise(field, rgb, W, H, max_iter, phase, vocal, instrumental, pitch, threads, interior, accents); });
}

int fractal_atlas_field_ex(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap,
                           float* out, int W, int H, double pzoom, double fraction, double czoom, double pbias,
                           double cbias, double obias, int palette, int feather, int threads) {
    return status_of([&] { atlas_field(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, czoom, pbias, cbias, obias, palette, feather, threads); });
}

int fractal_atlas_field(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap,
                        float* out, int W, int H, double pzoom, double fraction, int palette, int threads) {
    return fractal_atlas_field_ex(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, 1.0, 0.0, 0.0, 0.0,
                                  palette, 48, threads);
}

int fractal_atlas_colourise(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh, int ccap,
                            uint8_t* out, int W, int H, double pzoom, double fraction, int palette, double phase,
                            double vocal, double instrumental, double pitch, int threads) {
    return status_of([&] { atlas_colour(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, palette, phase, vocal, instrumental, pitch, threads, nullptr, nullptr); });
}

int fractal_atlas_colourise_interior(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh,
                                     int ccap, uint8_t* out, int W, int H, double pzoom, double fraction, int palette,
                                     double phase, double vocal, double instrumental, double pitch, int r, int g,
                                     int b, int threads) {
    const int interior[3] = {r, g, b};
    return status_of([&] { atlas_colour(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, palette, phase, vocal, instrumental, pitch, threads, interior, nullptr); });
}

int fractal_atlas_colourise_accents(const float* P, int pw, int ph, int pcap, const float* C, int cw, int chh,
                                    int ccap, uint8_t* out, int W, int H, double pzoom, double fraction, int palette,
                                    double phase, double vocal, double instrumental, double pitch,
                                    const uint8_t* accents, int r, int g, int b, int threads) {
    if (!accents) {
        error_text = "ordinary palette accents are required";
        return 1;
    }
    const int interior[3] = {r, g, b};
    return status_of([&] { atlas_colour(P, pw, ph, pcap, C, cw, chh, ccap, out, W, H, pzoom, fraction, palette, phase, vocal, instrumental, pitch, threads, interior, accents); });
}

}  // extern "C"
