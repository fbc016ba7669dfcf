// Direct (shallow) field render in plain double, one thread per pixel.
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

template <int Formula, bool Planes>
__global__ void __launch_bounds__(128) direct_kernel(const DirectParams p) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const long long index = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (index >= pixels) return;
    const int py = static_cast<int>(index / p.width);
    const int px = static_cast<int>(index - static_cast<long long>(py) * p.width);
    // Pixel coordinates (renderer.cpp:10185-10196): centre + offset * span / size.
    const double x_origin = p.coordinate_mode == 1 ? static_cast<double>(p.width / 2)
                                                   : static_cast<double>(p.width - 1) / 2.0;
    const double y_origin = p.coordinate_mode == 1 ? static_cast<double>(p.height / 2)
                                                   : static_cast<double>(p.height - 1) / 2.0;
    const double x_offset = (static_cast<double>(px) - x_origin) * p.width_span / static_cast<double>(p.width);
    const double y_offset = -(static_cast<double>(py) - y_origin) * p.height_span / static_cast<double>(p.height);
    const double cx = p.center_re + x_offset;
    const double cy = p.center_im + y_offset;
    const float inside = static_cast<float>(static_cast<double>(p.max_iter) - p.output_bias);
    auto mark_inside = [&] {
        p.out[index] = inside;
        if (p.counts) p.counts[index] = static_cast<std::uint32_t>(p.max_iter);
        if constexpr (Planes) {
            p.p_iter[index] = p.max_iter;
            p.p_phase[index] = 0.0;
            p.p_dex[index] = 0.0;
            p.p_dey[index] = 0.0;
            p.p_t1[index] = 0.0;
            p.p_t2[index] = 0.0;
        }
    };
    if constexpr (Formula == kFormulaMandelbrot) {
        const double q = (cx - 0.25) * (cx - 0.25) + cy * cy;
        const bool cardioid = q * (q + cx - 0.25) <= 0.25 * cy * cy;
        const bool bulb = (cx + 1.0) * (cx + 1.0) + cy * cy <= 0.0625;
        if (cardioid || bulb) {
            mark_inside();
            return;
        }
    }
    constexpr bool julia = Formula == kFormulaJulia;
    constexpr bool has_de = Formula == kFormulaMandelbrot || Formula == kFormulaJulia;
    double zr = julia ? cx : 0.0;
    double zi = julia ? cy : 0.0;
    const double pr = julia ? p.julia_re : cx;
    const double pi = julia ? p.julia_im : cy;
    double dr = julia ? 1.0 : 0.0;
    double di = 0.0;
    const double add_re = julia ? 0.0 : 1.0;
    double test1 = 0.0, test2 = 0.0;
    const double escape2 = escape_r2_d(p.escape_mode);
    const double safe2 = escape2 + 1.0e-7;
    const bool track_de = Planes && has_de && p.need_de;
    for (int iteration = 0; iteration < p.max_iter; ++iteration) {
        if (track_de) {
            // d' = 2 z d + 1 (parameter plane) or 2 z d (Julia), on the
            // pre-step z (renderer.cpp:336-338).
            const double ndr = 2.0 * zr * dr - 2.0 * zi * di + add_re;
            const double ndi = 2.0 * zr * di + 2.0 * zi * dr + 0.0;
            dr = ndr;
            di = ndi;
        }
        double nr, ni;
        step<Formula>(zr, zi, pr, pi, nr, ni);
        zr = nr;
        zi = ni;
        const double m2 = zr * zr + zi * zi;
        if constexpr (Planes) {
            test2 = test1;
            test1 = m2;
        }
        if (m2 > escape2 || !is_finite(m2)) {
            const double safe = is_finite(m2) ? dmax(m2, safe2) : 1.7976931348623157e308;
            const double magnitude = sqrt(safe);
            p.out[index] = static_cast<float>(
                (static_cast<double>(iteration + 1) - log(log(magnitude)) / kLogTwoD) - p.output_bias);
            if (p.counts) p.counts[index] = static_cast<std::uint32_t>(iteration + 1);
            if constexpr (Planes) {
                p.p_iter[index] = iteration;
                double phase = 0.0;
                if (p.need_phase && is_finite(zr) && is_finite(zi)) {
                    phase = atan2(zi, zr) / kTwoPi;
                    phase -= floor(phase);
                }
                p.p_phase[index] = phase;
                double de_re = 0.0, de_im = 0.0;
                if (track_de && is_finite(zr) && is_finite(zi) && is_finite(dr) && is_finite(di)) {
                    if (!direct_de(zr, zi, dr, di, fe_from(p.pixel_spacing, 0), de_re, de_im)) {
                        de_re = 0.0;
                        de_im = 0.0;
                    }
                }
                p.p_dex[index] = de_re;
                p.p_dey[index] = de_im;
                p.p_t1[index] = test1;
                p.p_t2[index] = test2;
            }
            return;
        }
    }
    mark_inside();
}

template <bool Planes>
cudaError_t launch_formula(const DirectParams& p, dim3 grid, dim3 block, cudaStream_t s) {
    switch (p.formula) {
        case kFormulaMandelbrot: direct_kernel<kFormulaMandelbrot, Planes><<<grid, block, 0, s>>>(p); break;
        case kFormulaJulia: direct_kernel<kFormulaJulia, Planes><<<grid, block, 0, s>>>(p); break;
        case kFormulaBurningShip: direct_kernel<kFormulaBurningShip, Planes><<<grid, block, 0, s>>>(p); break;
        default: direct_kernel<kFormulaTricorn, Planes><<<grid, block, 0, s>>>(p); break;
    }
    return cudaGetLastError();
}

// Aurora palette lookup (write_colour_pixel, renderer.cpp:5210-5237): the
// palette index is smooth * ((size-1)/max_iter) formed in double from a
// float32 scale, truncated and clamped; interior and non-finite pixels are
// black.  Four pixels per thread: 16 B of field in, 12 B of RGB out.
__global__ void __launch_bounds__(256) aurora_kernel(const float* __restrict__ field,
                                                     std::uint8_t* __restrict__ rgb, long long pixels,
                                                     const std::uint8_t* __restrict__ lut, int lut_size,
                                                     float index_scale, int max_iter, int vector_ok) {
    extern __shared__ std::uint8_t palette[];
    for (int i = threadIdx.x; i < lut_size * 3; i += blockDim.x) palette[i] = lut[i];
    __syncthreads();
    const float limit = static_cast<float>(max_iter);
    const long long quads = vector_ok ? pixels / 4 : 0;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    auto colour = [&](float smooth, std::uint8_t* dst) {
        if (!isfinite(smooth) || smooth >= limit) {
            dst[0] = 0;
            dst[1] = 0;
            dst[2] = 0;
            return;
        }
        const double scaled = static_cast<double>(smooth) * static_cast<double>(index_scale);
        const int k = scaled >= static_cast<double>(lut_size - 1)
            ? lut_size - 1
            : (!(scaled > 0.0) ? 0 : static_cast<int>(scaled));
        dst[0] = palette[3 * k];
        dst[1] = palette[3 * k + 1];
        dst[2] = palette[3 * k + 2];
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

cudaError_t launch_direct(const DirectParams& p, cudaStream_t stream) {
    const long long pixels = static_cast<long long>(p.width) * p.height;
    const dim3 block(128);
    const dim3 grid(static_cast<unsigned>((pixels + 127) / 128));
    const bool planes = p.p_iter != nullptr;
    return planes ? launch_formula<true>(p, grid, block, stream) : launch_formula<false>(p, grid, block, stream);
}

cudaError_t launch_aurora(const float* field, std::uint8_t* rgb, long long pixels, const std::uint8_t* lut,
                          int lut_size, float index_scale, int max_iter, cudaStream_t stream) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const long long quads = (pixels + 3) / 4;
    long long blocks = (quads + 255) / 256;
    const long long cap = static_cast<long long>(sms) * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    const std::size_t shared = static_cast<std::size_t>(lut_size) * 3;
    if (shared > 48 * 1024) {
        cudaFuncSetAttribute(aurora_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(shared));
    }
    const int vector_ok = (reinterpret_cast<std::uintptr_t>(field) % 16 == 0)
        && (reinterpret_cast<std::uintptr_t>(rgb) % 4 == 0);
    aurora_kernel<<<static_cast<unsigned>(blocks), 256, shared, stream>>>(field, rgb, pixels, lut, lut_size,
                                                                          index_scale, max_iter, vector_ok);
    return cudaGetLastError();
}

}  // namespace fgb
