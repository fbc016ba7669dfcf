// Direct (shallow) field render in plain double: a persistent lane-refill
// queue over a batch of fields.
//
// Restates render_direct_scalar_formula and render_direct_with_planes_formula
// (renderer.cpp:10054-10135, 10281-10438): cardioid/bulb culling for the
// Mandelbrot set, z^2 + c for the four formulas with the same operation
// order as the reference (the alternate maps keep separate products, which
// this --fmad=false translation unit guarantees for every formula), escape at
// |z|^2 > R^2 and smooth value n + 1 - log(log|z|)/log 2.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.h"

namespace fgb {
namespace {

using namespace fx;

constexpr double kLogTwoD = 0.6931471805599453094;  // log(2.0) as a double
constexpr double kTwoPi = 6.283185307179586476925286766559005768;

template <int Formula>
__device__ __forceinline__ void step(double zr, double zi, double pr, double pi, double& nr, double& ni) {
    if constexpr (Formula == kFormulaBurningShip) {
        const double ar = fabs_(zr);
        const double ai = fabs_(zi);
        const double rs = ar * ar;
        const double is = ai * ai;
        const double cross = 2.0 * ar * ai;
        const double diff = rs - is;
        ni = cross + pi;
        nr = diff + pr;
    } else if constexpr (Formula == kFormulaTricorn) {
        const double rs = zr * zr;
        const double is = zi * zi;
        const double cross = -2.0 * zr * zi;
        const double diff = rs - is;
        ni = cross + pi;
        nr = diff + pr;
    } else {
        // Mandelbrot and Julia share the map; only the start point differs.
        nr = zr * zr - zi * zi + pr;
        ni = 2.0 * zr * zi + pi;
    }
}

__device__ bool direct_de(double zr, double zi, double dr, double di, const Fe& spacing, double& out_re,
                          double& out_im) {
    const Sc total = sc_from_fe(fe_from(zr, 0), fe_from(zi, 0));
    const Sc derivative = sc_from_fe(fe_from(dr, 0), fe_from(di, 0));
    const double mag = hypot(total.re, total.im);
    if (!(mag > 0.0) || !is_finite(mag)) return false;
    const double log_mag = log(mag) + static_cast<double>(total.e) * 0.693147180559945309417232121458176568;
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

// 2 a b for doubles a, b, formed as the product a*b with its exponent raised
// by one.  That equals the reference's (2 a) b bit for bit when a*b lies in
// the normal range away from its lowest binade (rounding commutes with the
// exact doubling there) and below the overflow binade; an exactly zero
// operand gives the signed zero of the product.  Everything else (underflow,
// subnormal, huge, infinite, NaN) returns false and the caller multiplies.
__device__ __forceinline__ bool twice_product(double a, double b, double& out) {
    const double product = a * b;
    const long long bits = __double_as_longlong(product);
    const unsigned biased = static_cast<unsigned>((bits >> 52) & 0x7ff);
    if (biased - 2u < 2044u) {
        out = __longlong_as_double(bits + (1ll << 52));
        return true;
    }
    out = product;
    const unsigned long long magnitude = 0x7fffffffffffffffull;
    return (static_cast<unsigned long long>(__double_as_longlong(a)) & magnitude) == 0
        || (static_cast<unsigned long long>(__double_as_longlong(b)) & magnitude) == 0;
}

__device__ __forceinline__ unsigned long long dbits(double v) {
    return static_cast<unsigned long long>(__double_as_longlong(v));
}

// The reference's escape test m2 > R^2 with m2 = RN(a + b), a = zr*zr and
// b = zi*zi (so a, b >= +0), decided on the bit patterns without an FP64
// instruction: a lone term above R^2 (or infinite / NaN) escapes, two terms
// at most R^2/2 cannot, and in between the exact sum is compared with the
// rounding midpoint above R^2 in integer units of half an ulp of R^2 (ties
// to even, as the FP64 add rounds).  R^2 is a normal double above 2.
__device__ __forceinline__ bool sum_exceeds(unsigned long long a, unsigned long long b, unsigned long long r2) {
    constexpr unsigned long long kMant = (1ull << 52) - 1;
    constexpr unsigned long long kMag = 0x7fffffffffffffffull;
    a &= kMag;
    b &= kMag;
    if (a < b) {
        const unsigned long long t = a;
        a = b;
        b = t;
    }
    if (a > r2) return true;
    if (a <= r2 - (1ull << 52)) return false;
    const int er = static_cast<int>(r2 >> 52);
    const unsigned long long mr = (r2 & kMant) | (1ull << 52);
    const int ea = static_cast<int>(a >> 52);
    const unsigned long long big = ((a & kMant) | (1ull << 52)) << (ea - er + 1);
    int eb = static_cast<int>(b >> 52);
    unsigned long long mb = b & kMant;
    if (eb == 0) {
        eb = 1;
    } else {
        mb |= 1ull << 52;
    }
    const int shift = eb - er + 1;
    unsigned long long small;
    bool below = false;  // bits of b under the unit
    if (shift >= 0) {
        small = mb << shift;
    } else if (shift > -64) {
        small = mb >> -shift;
        below = (mb & ((1ull << -shift) - 1)) != 0;
    } else {
        small = 0;
        below = mb != 0;
    }
    const unsigned long long sum = big + small;
    const unsigned long long midpoint = 2 * mr + 1;
    if (sum != midpoint) return sum > midpoint;
    return below || (mr & 1) != 0;
}

// Per-lane state of one pixel in flight.
struct Lane {
    double zr, zi;      // z_n
    double rs, is;      // zr*zr, zi*zi of z_n (the escape test's products)
    double pr, pi;      // additive parameter
    double dr, di;      // derivative (planes with DE only)
    double test1, test2;
    double escape2;
    unsigned long long saved_r, saved_i;  // cycle probe (Brent): z at the last power of two
    unsigned long long mark_r, mark_i;    // and z at the last multiple of 64 steps
    int it;             // completed steps
    int check_at;
    int max_iter;
    int stop_at;        // spill when `it` reaches this (phase budget)
    int field;
    int local;          // pixel index inside the field
};

// Step at which a fresh pixel is spilled (the cap when spilling is off).
__device__ __forceinline__ int budget_stop(const DirectBatch& b, int max_iter) {
    if (b.budget <= 0 || b.spill_capacity <= 0) return max_iter;
    return b.budget < max_iter ? b.budget : max_iter;
}

template <bool Planes>
__device__ void write_inside(const DirectParams& p, int local) {
    p.out[local] = static_cast<float>(static_cast<double>(p.max_iter) - p.output_bias);
    if (p.counts) p.counts[local] = static_cast<std::uint32_t>(p.max_iter);
    if constexpr (Planes) {
        p.p_iter[local] = p.max_iter;
        p.p_phase[local] = 0.0;
        p.p_dex[local] = 0.0;
        p.p_dey[local] = 0.0;
        p.p_t1[local] = 0.0;
        p.p_t2[local] = 0.0;
    }
}

// Smooth escape value n + 1 - log(log|z|)/log 2 (renderer.cpp:10108-10116).
__device__ float smooth_value(const DirectParams& p, int iteration, double m2) {
    const double safe2 = escape_r2_d(p.escape_mode) + 1.0e-7;
    const double safe = is_finite(m2) ? dmax(m2, safe2) : 1.7976931348623157e308;
    const double magnitude = sqrt(safe);
    return static_cast<float>((static_cast<double>(iteration + 1) - log(log(magnitude)) / kLogTwoD) - p.output_bias);
}

template <int Formula>
__device__ void write_escape_planes(const DirectParams& p, const Lane& l, double m2) {
    constexpr bool has_de = Formula == kFormulaMandelbrot || Formula == kFormulaJulia;
    const int local = l.local;
    p.out[local] = smooth_value(p, l.it, m2);
    if (p.counts) p.counts[local] = static_cast<std::uint32_t>(l.it + 1);
    p.p_iter[local] = l.it;
    double phase = 0.0;
    if (p.need_phase && is_finite(l.zr) && is_finite(l.zi)) {
        phase = atan2(l.zi, l.zr) / kTwoPi;
        phase -= floor(phase);
    }
    p.p_phase[local] = phase;
    double de_re = 0.0, de_im = 0.0;
    if (has_de && p.need_de && is_finite(l.zr) && is_finite(l.zi) && is_finite(l.dr) && is_finite(l.di)) {
        if (!direct_de(l.zr, l.zi, l.dr, l.di, fe_from(p.pixel_spacing, 0), de_re, de_im)) {
            de_re = 0.0;
            de_im = 0.0;
        }
    }
    p.p_dex[local] = de_re;
    p.p_dey[local] = de_im;
    p.p_t1[local] = l.test1;
    p.p_t2[local] = l.test2;
}

// Warp-private staging in shared memory.  Pixel starts and escapes happen
// on single lanes at scattered times; doing their FP64 work (the
// cardioid/bulb test, the smooth value's logs) there would issue a full warp
// instruction for one lane each time.  Instead the warp classifies 32 new
// pixels at once into a start stack and parks escaped pixels until 32 are
// waiting, then finishes them with every lane busy (ballot + popc compaction).
struct StartSlot {
    double cx, cy;
    int field, local;
};
struct ParkSlot {
    double rs, is;  // the escaping step's squares (|z|^2 = rs + is)
    int it, field, local, pad;
};
constexpr int kStage = 64;
struct WarpStage {
    StartSlot start[kStage];
    ParkSlot park[kStage];
};

// Warp-uniform queue state (every lane holds the same values).
struct WarpQueue {
    long long next, end;  // claimed pixel range not yet classified
    int field;            // field of `next` (search hint)
    int starts;           // pixels waiting in the start stack
    int parked;           // escapes waiting in the park buffer
    bool drained;         // the batch counter ran out
};

// Classify up to 32 pixels of the warp's claimed range (claiming a new chunk
// when it is empty): interior-culled pixels are written at once, the others
// pushed on the start stack with their coordinates.
template <int Formula, bool Planes>
__device__ void classify(const DirectBatch& b, WarpQueue& q, WarpStage& st, unsigned long long* claim,
                         unsigned lane, unsigned below, long long total) {
    constexpr unsigned kFull = 0xffffffffu;
    if (q.next >= q.end) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(claim, static_cast<unsigned long long>(b.chunk));
        base = __shfl_sync(kFull, base, 0);
        if (static_cast<long long>(base) >= total) {
            q.drained = true;
            return;
        }
        q.next = static_cast<long long>(base);
        q.end = q.next + b.chunk < total ? q.next + b.chunk : total;
    }
    const long long avail = q.end - q.next;
    const int n = avail < 32 ? static_cast<int>(avail) : 32;
    const long long g = q.next + lane;
    bool keep = false;
    double cx = 0.0, cy = 0.0;
    int f = q.field, local = 0;
    if (static_cast<int>(lane) < n) {
        while (g >= b.first[f + 1]) ++f;
        const DirectParams& p = b.field[f];
        local = static_cast<int>(g - b.first[f]);
        const int py = local / p.width;
        const int px = local - py * p.width;
        const double* coords = b.coords + b.coord_offset[f];
        cx = coords[px];
        cy = coords[p.width + py];
        keep = true;
        if constexpr (Formula == kFormulaMandelbrot) {
            if (b.interior_test[f]) {
                // renderer.cpp:10060-10066
                const double qq = (cx - 0.25) * (cx - 0.25) + cy * cy;
                const bool cardioid = qq * (qq + cx - 0.25) <= 0.25 * cy * cy;
                const bool bulb = (cx + 1.0) * (cx + 1.0) + cy * cy <= 0.0625;
                if (cardioid || bulb) keep = false;
            }
        }
        if (p.max_iter <= 0) keep = false;
        if (!keep) write_inside<Planes>(p, local);
    }
    q.field = __shfl_sync(kFull, f, n - 1);
    q.next += n;
    const unsigned kept = __ballot_sync(kFull, keep);
    if (keep) {
        StartSlot& slot = st.start[q.starts + __popc(kept & below)];
        slot.cx = cx;
        slot.cy = cy;
        slot.field = f;
        slot.local = local;
    }
    q.starts += __popc(kept);
    __syncwarp();
}

template <int Formula>
__device__ void begin_pixel(const DirectBatch& b, const StartSlot& slot, Lane& l) {
    constexpr bool julia = Formula == kFormulaJulia;
    const DirectParams& p = b.field[slot.field];
    l.field = slot.field;
    l.local = slot.local;
    l.zr = julia ? slot.cx : 0.0;
    l.zi = julia ? slot.cy : 0.0;
    l.rs = l.zr * l.zr;
    l.is = l.zi * l.zi;
    l.pr = julia ? p.julia_re : slot.cx;
    l.pi = julia ? p.julia_im : slot.cy;
    l.dr = julia ? 1.0 : 0.0;
    l.di = 0.0;
    l.test1 = 0.0;
    l.test2 = 0.0;
    l.escape2 = escape_r2_d(p.escape_mode);
    l.saved_r = dbits(l.zr);
    l.saved_i = dbits(l.zi);
    l.mark_r = l.saved_r;
    l.mark_i = l.saved_i;
    l.it = 0;
    l.check_at = 1;
    l.max_iter = p.max_iter;
    l.stop_at = budget_stop(b, p.max_iter);
}

// Resume a spilled pixel (it then runs to its end).  The entry was written
// by another SM during this launch: read it from L2 (ld.global.cg), never
// from a possibly stale L1 line.
template <int Formula>
__device__ void resume_pixel(const DirectBatch& b, const DirectSpill& e, Lane& l) {
    constexpr bool julia = Formula == kFormulaJulia;
    const int field = __ldcg(&e.field);
    const int local = __ldcg(&e.local);
    const DirectParams& p = b.field[field];
    l.field = field;
    l.local = local;
    l.zr = __ldcg(&e.zr);
    l.zi = __ldcg(&e.zi);
    l.rs = l.zr * l.zr;
    l.is = l.zi * l.zi;
    if (julia) {
        l.pr = p.julia_re;
        l.pi = p.julia_im;
    } else {
        const int py = local / p.width;
        const int px = local - py * p.width;
        const double* coords = b.coords + b.coord_offset[field];
        l.pr = coords[px];
        l.pi = coords[p.width + py];
    }
    l.dr = __ldcg(&e.dr);
    l.di = __ldcg(&e.di);
    l.test1 = __ldcg(&e.test1);
    l.test2 = __ldcg(&e.test2);
    l.escape2 = escape_r2_d(p.escape_mode);
    l.saved_r = __ldcg(&e.saved_r);
    l.saved_i = __ldcg(&e.saved_i);
    l.mark_r = __ldcg(&e.mark_r);
    l.mark_i = __ldcg(&e.mark_i);
    l.it = __ldcg(&e.it);
    l.check_at = __ldcg(&e.check_at);
    l.max_iter = p.max_iter;
    l.stop_at = p.max_iter;  // resumed pixels run to their end
}

// The smooth value with the logarithms in FP32 (the floatexp form's direct
// levels): the same formula, within a few float ulps of the FP64 value, at
// no FP64 cost.  Non-finite |z|^2 keeps the FP64 path.
__device__ float smooth_value_fast(const DirectParams& p, int iteration, double m2) {
    if (!is_finite(m2)) return smooth_value(p, iteration, m2);
    const double safe2 = escape_r2_d(p.escape_mode) + 1.0e-7;
    const float safe = static_cast<float>(dbits(m2) > dbits(safe2) ? m2 : safe2);
    const float log_mag = 0.5f * logf(safe);
    return (static_cast<float>(iteration + 1) - log2f(log_mag)) - static_cast<float>(p.output_bias);
}

__device__ void finish_parked(const DirectBatch& b, const ParkSlot& e) {
    const DirectParams& p = b.field[e.field];
    const double m2 = e.rs + e.is;
    p.out[e.local] = b.fast_smooth ? smooth_value_fast(p, e.it, m2) : smooth_value(p, e.it, m2);
    if (p.counts) p.counts[e.local] = static_cast<std::uint32_t>(e.it + 1);
}

// Direct field render over a batch of fields with lane refill.
//
// Restates render_direct_scalar_formula / render_direct_with_planes_formula
// (renderer.cpp:10054-10135, 10281-10438) pixel for pixel: the same
// coordinates, cardioid/bulb culling, the map z^2 + c with the reference's
// operation order (this translation unit is built without FMA contraction),
// escape at |z|^2 > R^2 and the smooth value.  Two rewrites leave every
// output bit unchanged:
//   * the squares zr*zr and zi*zi of the escape test are the next step's
//     squares, and 2 zr zi is formed as the product zr*zi with its exponent
//     raised by one (exact for normal numbers; the multiply otherwise);
//   * an orbit that returns bit for bit to an earlier z repeats forever and
//     can never escape, so it is settled as interior at once (interior
//     outputs do not depend on z); z is kept at every power of two (Brent's
//     probe, any period) and at every multiple of 64 steps (short periods
//     found within ~64 steps of the orbit settling).
// FP64 is the bottleneck on this part (1/64 of the FP32 rate), so a warp
// never waits on a finished lane: each warp claims chunks of pixels from a
// device counter over all fields of the batch and refills idle lanes every
// step from its start stack; escapes are parked and finished 32 at a time.
// Capped at 64 registers (a few spills): beside the FP32 queue on one SM, a
// block then takes as many registers as an FP32-queue block, so two of each
// kind fit where 80-register blocks left room for fewer.
template <int Formula, bool Planes>
__global__ void __launch_bounds__(128, 8) direct_queue_kernel(const __grid_constant__ DirectBatch b) {
    constexpr unsigned kFull = 0xffffffffu;
    __shared__ WarpStage stages[4];
    WarpStage& st = stages[threadIdx.x >> 5];
    const unsigned lane_id = threadIdx.x & 31u;
    const unsigned below = (1u << lane_id) - 1u;
    unsigned long long* claim = b.counter + kClaimFresh;
    unsigned long long* reserved = b.counter + kSpillReserved;
    unsigned long long* taken = b.counter + kSpillClaimed;
    const unsigned long long generation = *(b.counter + kGeneration);
    const long long total = b.first[b.count];
    WarpQueue q{0, 0, 0, 0, 0, false};
    bool active = false;
    bool resumed = false;  // the lane's pixel came from the spill list
    unsigned long long executed = 0;  // steps this lane computed for a pixel
    Lane l;
    l.field = 0;
    l.zr = l.zi = l.rs = l.is = l.pr = l.pi = 0.0;
    l.dr = l.di = l.test1 = l.test2 = 0.0;
    l.escape2 = 4.0;
    l.saved_r = l.saved_i = 0;
    l.it = 0;
    l.check_at = 1;
    l.max_iter = 0;
    l.stop_at = 0;
    l.local = 0;

    unsigned rounds = 0;
    while (true) {
        unsigned idle = __ballot_sync(kFull, !active);
        bool pending = false;  // spilled pixels exist that nobody has taken yet
        // The spill counters live in L2: look at them every 32nd refill round
        // (a long pixel waits a few dozen steps at most) or once the fresh
        // queue is drained, not on every step.
        const bool poll = (++rounds & 31u) == 0u || q.drained;
        if (idle != 0u && b.spill_capacity > 0 && poll) {
            // Spilled (long) pixels first: claim up to one per idle lane.
            unsigned long long base = 0, got = 0;
            if (lane_id == 0) {
                unsigned long long seen = *const_cast<volatile unsigned long long*>(taken);
                for (int attempt = 0; attempt < 64; ++attempt) {
                    unsigned long long made = *const_cast<volatile unsigned long long*>(reserved);
                    if (made > static_cast<unsigned long long>(b.spill_capacity)) {
                        made = static_cast<unsigned long long>(b.spill_capacity);
                    }
                    if (seen >= made) break;
                    const unsigned long long want = made - seen < static_cast<unsigned long long>(__popc(idle))
                                                        ? made - seen
                                                        : static_cast<unsigned long long>(__popc(idle));
                    const unsigned long long old = atomicCAS(taken, seen, seen + want);
                    if (old == seen) {
                        base = seen;
                        got = want;
                        break;
                    }
                    seen = old;
                }
            }
            base = __shfl_sync(kFull, base, 0);
            got = __shfl_sync(kFull, got, 0);
            const int rank = __popc(idle & below);
            const bool mine = ((idle >> lane_id) & 1u) != 0u && static_cast<unsigned long long>(rank) < got;
            if (mine) {
                // The producer reserved this slot before writing it; wait
                // (bounded) for its generation mark.
                const DirectSpill& e = b.spill[base + rank];
                bool ready = false;
                for (int spin = 0; spin < b.spin_limit; ++spin) {
                    if (*reinterpret_cast<const volatile unsigned long long*>(&e.ready) == generation) {
                        ready = true;
                        break;
                    }
                }
                __threadfence();
                if (ready) {
                    resume_pixel<Formula>(b, e, l);
                    active = true;
                    resumed = true;
                } else {
                    atomicExch(b.counter + kQueueError, 1ull);
                }
            }
            idle &= ~__ballot_sync(kFull, mine);
            pending = got != 0;
        }
        if (idle != 0u) {
            const int need = __popc(idle);
            while (q.starts < need && !q.drained) classify<Formula, Planes>(b, q, st, claim, lane_id, below, total);
            const int rank = __popc(idle & below);
            if (((idle >> lane_id) & 1u) != 0u && rank < q.starts) {
                begin_pixel<Formula>(b, st.start[q.starts - 1 - rank], l);
                active = true;
                resumed = false;
            }
            q.starts -= need < q.starts ? need : q.starts;
            __syncwarp();
        }
        if (__ballot_sync(kFull, active) == 0u) {
            if (pending) continue;
            // No work in hand: stop unless spilled pixels are waiting.
            bool waiting = false;
            if (b.spill_capacity > 0 && lane_id == 0) {
                unsigned long long made = *const_cast<volatile unsigned long long*>(reserved);
                if (made > static_cast<unsigned long long>(b.spill_capacity)) {
                    made = static_cast<unsigned long long>(b.spill_capacity);
                }
                waiting = *const_cast<volatile unsigned long long*>(taken) < made;
            }
            if (__shfl_sync(kFull, waiting, 0)) continue;
            // Drained: finish what is parked (fewer than 32) and stop.
            if constexpr (!Planes) {
                if (static_cast<int>(lane_id) < q.parked) finish_parked(b, st.park[lane_id]);
            }
            for (int o = 16; o > 0; o >>= 1) executed += __shfl_xor_sync(kFull, executed, o);
            if (lane_id == 0) atomicAdd(b.counter + kStepsExecuted, executed);
            break;
        }

        // Up to `steps` steps before the next refill: every lane computes
        // each step (an idle or settled lane on stale values that it then
        // discards: the FP64 pipe costs the same per warp instruction), and a
        // lane stops updating at its first event (escape, interior, budget).
        constexpr bool has_de = Formula == kFormulaMandelbrot || Formula == kFormulaJulia;
        bool running = active;
        bool escaped = false, inside = false, spill = false;
        double rs_at_escape = 0.0, is_at_escape = 0.0;
        const int steps = __all_sync(kFull, !active || resumed) ? b.long_steps : b.steps;
        for (int s = 0; s < steps; ++s) {
            if (!__any_sync(kFull, running)) break;
            executed += running ? 1u : 0u;
            if constexpr (Planes && has_de) {
                if (running && b.field[l.field].need_de) {
                    // d' = 2 z d + 1 (parameter plane) or 2 z d (Julia) on the
                    // pre-step z (renderer.cpp:336-338).
                    const double add_re = Formula == kFormulaJulia ? 0.0 : 1.0;
                    const double ndr = 2.0 * l.zr * l.dr - 2.0 * l.zi * l.di + add_re;
                    const double ndi = 2.0 * l.zr * l.di + 2.0 * l.zi * l.dr + 0.0;
                    l.dr = ndr;
                    l.di = ndi;
                }
            }
            const double ar = Formula == kFormulaBurningShip ? fabs_(l.zr) : l.zr;
            const double ai = Formula == kFormulaBurningShip ? fabs_(l.zi) : l.zi;
            double cross;
            const bool fast = twice_product(ar, ai, cross);
            if (__any_sync(kFull, running && !fast)) {
                if (!fast) cross = Formula == kFormulaTricorn ? -2.0 * l.zr * l.zi : 2.0 * ar * ai;
                else if (Formula == kFormulaTricorn) cross = -cross;
            } else if (Formula == kFormulaTricorn) {
                cross = -cross;
            }
            const double nr = (l.rs - l.is) + l.pr;
            const double ni = cross + l.pi;
            const double rs = nr * nr;
            const double is = ni * ni;
            if (!running) continue;
            l.zr = nr;
            l.zi = ni;
            l.rs = rs;
            l.is = is;
            if constexpr (Planes) {
                l.test2 = l.test1;
                l.test1 = rs + is;
            }
            if (sum_exceeds(dbits(rs), dbits(is), dbits(l.escape2))) {
                escaped = true;
                rs_at_escape = rs;
                is_at_escape = is;
                running = false;
                continue;
            }
            ++l.it;
            const unsigned long long br = dbits(l.zr), bi = dbits(l.zi);
            if ((br == l.saved_r && bi == l.saved_i) || (br == l.mark_r && bi == l.mark_i) || l.it >= l.max_iter) {
                inside = true;
                running = false;
                continue;
            }
            if (l.it == l.check_at) {
                l.saved_r = br;
                l.saved_i = bi;
                l.check_at = l.check_at < (1 << 30) ? l.check_at << 1 : l.check_at;
            }
            if ((l.it & 63) == 0) {
                l.mark_r = br;
                l.mark_i = bi;
            }
            if (l.it >= l.stop_at) {
                spill = true;
                running = false;
            }
        }
        if (inside) {
            write_inside<Planes>(b.field[l.field], l.local);
            active = false;
        }
        const unsigned spilling = __ballot_sync(kFull, spill);
        if (spilling != 0u) {
            // Hand lanes past the budget to the spill list (one reservation
            // per warp, the entry's generation mark written last); a full
            // list lets them run on here.
            const int leader = __ffs(spilling) - 1;
            unsigned long long base = 0;
            if (static_cast<int>(lane_id) == leader) {
                base = atomicAdd(reserved, static_cast<unsigned long long>(__popc(spilling)));
            }
            base = __shfl_sync(kFull, base, leader);
            if (spill) {
                const long long slot = static_cast<long long>(base) + __popc(spilling & below);
                if (slot < b.spill_capacity) {
                    DirectSpill& e = b.spill[slot];
                    e.zr = l.zr;
                    e.zi = l.zi;
                    e.dr = l.dr;
                    e.di = l.di;
                    e.test1 = l.test1;
                    e.test2 = l.test2;
                    e.saved_r = l.saved_r;
                    e.saved_i = l.saved_i;
                    e.mark_r = l.mark_r;
                    e.mark_i = l.mark_i;
                    e.it = l.it;
                    e.check_at = l.check_at;
                    e.field = l.field;
                    e.local = l.local;
                    __threadfence();
                    if (!b.withhold_publish) *reinterpret_cast<volatile unsigned long long*>(&e.ready) = generation;
                    active = false;
                } else {
                    l.stop_at = l.max_iter;
                }
            }
        }
        if constexpr (Planes) {
            if (escaped) {
                write_escape_planes<Formula>(b.field[l.field], l, rs_at_escape + is_at_escape);
                active = false;
            }
        } else {
            const unsigned esc = __ballot_sync(kFull, escaped);
            if (esc != 0u) {
                if (escaped) {
                    ParkSlot& slot = st.park[q.parked + __popc(esc & below)];
                    slot.rs = rs_at_escape;
                    slot.is = is_at_escape;
                    slot.it = l.it;
                    slot.field = l.field;
                    slot.local = l.local;
                    active = false;
                }
                q.parked += __popc(esc);
                __syncwarp();
                if (q.parked >= 32) {
                    finish_parked(b, st.park[q.parked - 32 + static_cast<int>(lane_id)]);
                    q.parked -= 32;
                    __syncwarp();
                }
            }
        }
    }
}

// Per-field coordinate tables (renderer.cpp:10185-10196): cx per column and
// cy per row, each centre + offset * span / size in double; also zeroes the
// batch's claim counter.
__global__ void direct_coords_kernel(const __grid_constant__ DirectBatch b) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < kGeneration) b.counter[i] = 0ull;
    if (i == kGeneration) b.counter[i] += 1ull;  // a new mark for this batch's spill entries
    for (int f = 0; f < b.count; ++f) {
        const DirectParams& p = b.field[f];
        const long long span = static_cast<long long>(p.width) + p.height;
        const long long start = b.coord_offset[f];
        if (i < start || i >= start + span) continue;
        const int k = static_cast<int>(i - start);
        double value;
        if (k < p.width) {
            const double x_origin = p.coordinate_mode == 1 ? static_cast<double>(p.width / 2)
                                                           : static_cast<double>(p.width - 1) / 2.0;
            const double x_offset = (static_cast<double>(k) - x_origin) * p.width_span / static_cast<double>(p.width);
            value = p.center_re + x_offset;
        } else {
            const int py = k - p.width;
            const double y_origin = p.coordinate_mode == 1 ? static_cast<double>(p.height / 2)
                                                           : static_cast<double>(p.height - 1) / 2.0;
            const double y_offset =
                -(static_cast<double>(py) - y_origin) * p.height_span / static_cast<double>(p.height);
            value = p.center_im + y_offset;
        }
        b.coords[i] = value;
    }
}

template <int Formula, bool Planes>
cudaError_t launch_queue(const DirectBatch& b, int sms, int blocks_per_sm, cudaStream_t s) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int blocks = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, direct_queue_kernel<Formula, Planes>, 128, 0);
        per_sm = blocks > 0 ? blocks : 1;
    }
    const long long pixels = b.first[b.count];
    const int use = blocks_per_sm > 0 && blocks_per_sm < per_sm ? blocks_per_sm : per_sm;
    long long grid = static_cast<long long>(sms) * use;
    const long long needed = (pixels + 127) / 128;
    if (grid > needed) grid = needed;
    if (grid < 1) grid = 1;
    direct_queue_kernel<Formula, Planes><<<static_cast<unsigned>(grid), 128, 0, s>>>(b);
    return cudaGetLastError();
}

template <bool Planes>
cudaError_t launch_formula(const DirectBatch& b, int formula, int sms, int blocks_per_sm, cudaStream_t s) {
    switch (formula) {
        case kFormulaMandelbrot: return launch_queue<kFormulaMandelbrot, Planes>(b, sms, blocks_per_sm, s);
        case kFormulaJulia: return launch_queue<kFormulaJulia, Planes>(b, sms, blocks_per_sm, s);
        case kFormulaBurningShip: return launch_queue<kFormulaBurningShip, Planes>(b, sms, blocks_per_sm, s);
        default: return launch_queue<kFormulaTricorn, Planes>(b, sms, blocks_per_sm, s);
    }
}

// Aurora palette lookup (write_colour_pixel, renderer.cpp:5210-5237): the
// palette index is smooth * ((size-1)/max_iter), the reference's double
// product of two floats, truncated and clamped; interior and non-finite
// pixels take the interior colour.  Four pixels per thread: 16 B of field in, 12 B of RGB out.
__global__ void __launch_bounds__(256) aurora_kernel(const float* __restrict__ field,
                                                     std::uint8_t* __restrict__ rgb, long long pixels,
                                                     const std::uint8_t* __restrict__ lut, int lut_size,
                                                     float index_scale, int max_iter, int vector_ok,
                                                     std::uint32_t interior) {
    const float limit = static_cast<float>(max_iter);
    const long long quads = vector_ok ? pixels / 4 : 0;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    auto colour = [&](float smooth, std::uint8_t* dst) {
        if (!isfinite(smooth) || smooth >= limit) {
            dst[0] = static_cast<std::uint8_t>(interior);
            dst[1] = static_cast<std::uint8_t>(interior >> 8);
            dst[2] = static_cast<std::uint8_t>(interior >> 16);
            return;
        }
        // trunc(double(smooth) * double(index_scale)), clamped: the product
        // of two floats is exact as p + e (FMA two-product), so it is
        // compared and truncated without FP64 (smooth is finite here).
        const float p = smooth * index_scale;
        const float e = __fmaf_rn(smooth, index_scale, -p);
        const float last_f = static_cast<float>(lut_size - 1);
        int k;
        if (p > last_f || (p == last_f && e >= 0.0f)) {
            k = lut_size - 1;
        } else if (!(p > 0.0f)) {
            k = 0;
        } else {
            const float f = floorf(p);
            k = static_cast<int>(f) - (p == f && e < 0.0f ? 1 : 0);
        }
        dst[0] = __ldg(lut + 3 * k);
        dst[1] = __ldg(lut + 3 * k + 1);
        dst[2] = __ldg(lut + 3 * k + 2);
    };
    for (long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; q < quads; q += stride) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(field) + q);
        std::uint8_t out[12];
        colour(v.x, out);
        colour(v.y, out + 3);
        colour(v.z, out + 6);
        colour(v.w, out + 9);
        std::uint32_t w0 = out[0] | (out[1] << 8) | (out[2] << 16) | (static_cast<std::uint32_t>(out[3]) << 24);
        std::uint32_t w1 = out[4] | (out[5] << 8) | (out[6] << 16) | (static_cast<std::uint32_t>(out[7]) << 24);
        std::uint32_t w2 = out[8] | (out[9] << 8) | (out[10] << 16) | (static_cast<std::uint32_t>(out[11]) << 24);
        uint3 packed = make_uint3(w0, w1, w2);
        // 12-byte store: the RGB buffer of a 4-pixel group starts at 12*q,
        // which is 4-byte aligned.
        std::uint32_t* dst = reinterpret_cast<std::uint32_t*>(rgb + 12 * q);
        __stcs(dst, packed.x);
        __stcs(dst + 1, packed.y);
        __stcs(dst + 2, packed.z);
    }
    // Tail pixels (count not divisible by four).
    const long long tail_start = quads * 4;
    for (long long i = tail_start + static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += stride) {
        colour(field[i], rgb + 3 * i);
    }
}

__global__ void stamp_time_kernel(unsigned long long* slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *slot = t;
}

}  // namespace

cudaError_t launch_stamp_time(unsigned long long* slot, cudaStream_t stream) {
    stamp_time_kernel<<<1, 1, 0, stream>>>(slot);
    return cudaGetLastError();
}

cudaError_t direct_queue_attributes(cudaFuncAttributes* attributes) {
    return cudaFuncGetAttributes(attributes, direct_queue_kernel<kFormulaMandelbrot, false>);
}

int direct_queue_occupancy() {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, direct_queue_kernel<kFormulaMandelbrot, false>, 128, 0);
    return blocks > 0 ? blocks : 1;
}

std::size_t direct_scratch_bytes(const DirectParams* fields, int count, long long spill_entries) {
    std::size_t doubles = 0;
    for (int f = 0; f < count; ++f) doubles += static_cast<std::size_t>(fields[f].width) + fields[f].height;
    std::size_t bytes = 256 + doubles * sizeof(double);
    if (spill_entries > 0) {
        bytes = (bytes + 255) / 256 * 256;
        bytes += static_cast<std::size_t>(spill_entries) * sizeof(DirectSpill);
    }
    return bytes;
}

// Interior culling can matter only where the view reaches the cardioid's or
// the period-2 bulb's bounding box (with a wide margin).
static bool view_meets_interior(const DirectParams& p) {
    const double half_w = 0.5 * p.width_span + 0.05, half_h = 0.5 * p.height_span + 0.05;
    const double x0 = p.center_re - half_w, x1 = p.center_re + half_w;
    const double y0 = p.center_im - half_h, y1 = p.center_im + half_h;
    const bool cardioid = x1 >= -0.80 && x0 <= 0.40 && y1 >= -0.70 && y0 <= 0.70;
    const bool bulb = x1 >= -1.30 && x0 <= -0.70 && y1 >= -0.30 && y0 <= 0.30;
    return cardioid || bulb;
}

namespace {
constexpr int kDefaultSpinLimit = 1 << 22;
thread_local int fault_spin_limit = kDefaultSpinLimit;
thread_local int fault_withhold_publish = 0;
}  // namespace

void set_direct_fault_injection(int spin_limit, int withhold_publish) {
    fault_spin_limit = spin_limit > 0 ? spin_limit : kDefaultSpinLimit;
    fault_withhold_publish = withhold_publish ? 1 : 0;
}

cudaError_t launch_direct_batch(const DirectParams* fields, int count, void* scratch, const QueueShape& shape,
                                long long spill_entries, cudaStream_t stream, bool fast_smooth) {
    if (count < 1 || count > kMaxDirectFields || !scratch) return cudaErrorInvalidValue;
    DirectBatch b{};
    b.spin_limit = fault_spin_limit;
    b.withhold_publish = fault_withhold_publish;
    b.count = count;
    b.fast_smooth = fast_smooth ? 1 : 0;
    b.counter = static_cast<unsigned long long*>(scratch);
    b.coords = reinterpret_cast<double*>(static_cast<char*>(scratch) + 256);
    b.chunk = shape.chunk > 0 ? shape.chunk : 64;
    const int formula = fields[0].formula;
    const bool planes = fields[0].p_iter != nullptr;
    long long pixels = 0, coords = 0;
    for (int f = 0; f < count; ++f) {
        if (fields[f].formula != formula || (fields[f].p_iter != nullptr) != planes) return cudaErrorInvalidValue;
        b.field[f] = fields[f];
        b.first[f] = pixels;
        b.coord_offset[f] = static_cast<int>(coords);
        b.interior_test[f] = formula == kFormulaMandelbrot && view_meets_interior(fields[f]) ? 1 : 0;
        pixels += static_cast<long long>(fields[f].width) * fields[f].height;
        coords += static_cast<long long>(fields[f].width) + fields[f].height;
    }
    b.first[count] = pixels;
    if (spill_entries > 0) {
        const std::size_t head = (256 + static_cast<std::size_t>(coords) * sizeof(double) + 255) / 256 * 256;
        b.spill = reinterpret_cast<DirectSpill*>(static_cast<char*>(scratch) + head);
        b.spill_capacity = spill_entries;
        b.budget = 256;
    }
    b.steps = shape.steps > 0 ? shape.steps : 2;
    b.long_steps = 16;
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    direct_coords_kernel<<<static_cast<unsigned>((coords + 255) / 256), 256, 0, stream>>>(b);
    cudaError_t status = cudaGetLastError();
    if (status != cudaSuccess) return status;
    return planes ? launch_formula<true>(b, formula, sms, shape.blocks_per_sm, stream)
                  : launch_formula<false>(b, formula, sms, shape.blocks_per_sm, stream);
}

cudaError_t launch_aurora(const float* field, std::uint8_t* rgb, long long pixels, const std::uint8_t* lut,
                          int lut_size, float index_scale, int max_iter, cudaStream_t stream,
                          std::uint32_t interior) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // The palette (up to 192 KiB) is read through L1: neighbouring pixels
    // take neighbouring entries.
    const long long quads = (pixels + 3) / 4;
    const int threads = 256;
    long long blocks = (quads + threads - 1) / threads;
    const long long cap = static_cast<long long>(sms) * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    const int vector_ok = (reinterpret_cast<std::uintptr_t>(field) % 16 == 0)
        && (reinterpret_cast<std::uintptr_t>(rgb) % 4 == 0);
    aurora_kernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(field, rgb, pixels, lut, lut_size,
                                                                              index_scale, max_iter, vector_ok,
                                                                              interior);
    return cudaGetLastError();
}

}  // namespace fgb
