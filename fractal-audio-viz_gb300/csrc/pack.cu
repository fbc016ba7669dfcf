// Video-frame handoff: RGB8 frames packed on the device into the layout the
// encoder pipe takes, so the host copies one finished buffer per frame.
//
// The reference writes rgb24 to FFmpeg's stdin, or rgb0 for NVENC's packed
// RGB input (visualizer.py:3203-3260, 12916-12942).  Formats here:
//   0 rgb24   the frame as is
//   1 rgb0    R, G, B, 0 per pixel
//   2 rgba    R, G, B, 255 per pixel
//   3 yuv420p BT.709 limited range, planes Y (W x H), U, V (ceil(W/2) x
//             ceil(H/2)); chroma from the mean of each 2x2 block
//   4 nv12    the same Y plane, then U/V interleaved
// The YUV conversion is the integer BT.709 form
//   Y = 16 + ((47 R + 157 G + 16 B + 128) >> 8)
//   U = 128 + ((-26 R - 86 G + 112 B + 128) >> 8)
//   V = 128 + ((112 R - 102 G - 10 B + 128) >> 8)
// (coefficients: the BT.709 matrix scaled to 8-bit studio swing, x 256,
// rounded so that each chroma row sums to zero: greys map to 128), chroma
// taken from the rounded mean of the 2x2 block's R, G, B.
// One thread per 2x2 block (any shape) or per 4x2 pixels with word accesses
// (the common shape); HBM-bound (3 B in, 1.5 B out per pixel for YUV).
#include <cuda_runtime.h>

#include <cstdint>

#include "device.h"

namespace fgb {
namespace {

__device__ __forceinline__ int luma(int r, int g, int b) { return 16 + ((47 * r + 157 * g + 16 * b + 128) >> 8); }
__device__ __forceinline__ int chroma_u(int r, int g, int b) { return 128 + ((-26 * r - 86 * g + 112 * b + 128) >> 8); }
__device__ __forceinline__ int chroma_v(int r, int g, int b) { return 128 + ((112 * r - 102 * g - 10 * b + 128) >> 8); }

__global__ void pack_rgbx_kernel(const std::uint8_t* __restrict__ rgb, std::uint32_t* __restrict__ out,
                                 long long pixels, std::uint32_t alpha) {
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < pixels;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const std::uint8_t* p = rgb + 3 * i;
        out[i] = static_cast<std::uint32_t>(p[0]) | (static_cast<std::uint32_t>(p[1]) << 8)
            | (static_cast<std::uint32_t>(p[2]) << 16) | (alpha << 24);
    }
}

// Four pixels per thread for 4-byte aligned RGB and 16-byte aligned output:
// three word loads, one 16-byte store; `quads` = pixels / 4 (the caller packs
// any remainder with pack_rgbx_kernel).
__global__ void pack_rgbx_wide_kernel(const std::uint8_t* __restrict__ rgb, uint4* __restrict__ out, long long quads,
                                      std::uint32_t alpha) {
    const std::uint32_t a = alpha << 24;
    for (long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; q < quads;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        const std::uint32_t* src = reinterpret_cast<const std::uint32_t*>(rgb + 12 * q);
        const std::uint32_t w0 = __ldg(src), w1 = __ldg(src + 1), w2 = __ldg(src + 2);
        // Bytes r0 g0 b0 r1 | g1 b1 r2 g2 | b2 r3 g3 b3.
        uint4 o;
        o.x = (w0 & 0xffffffu) | a;
        o.y = (w0 >> 24) | ((w1 & 0xffffu) << 8) | a;
        o.z = (w1 >> 16) | ((w2 & 0xffu) << 16) | a;
        o.w = (w2 >> 8) | a;
        out[q] = o;
    }
}

__global__ void pack_yuv_kernel(const std::uint8_t* __restrict__ rgb, std::uint8_t* __restrict__ out, int width,
                                int height, int interleaved) {
    const int cw = (width + 1) / 2, ch = (height + 1) / 2;
    const long long blocks = static_cast<long long>(cw) * ch;
    std::uint8_t* y_plane = out;
    std::uint8_t* u_plane = out + static_cast<long long>(width) * height;
    std::uint8_t* v_plane = u_plane + blocks;
    for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < blocks;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int by = static_cast<int>(k / cw), bx = static_cast<int>(k - static_cast<long long>(by) * cw);
        int sr = 0, sg = 0, sb = 0, n = 0;
        for (int dy = 0; dy < 2; ++dy) {
            const int y = 2 * by + dy;
            if (y >= height) continue;
            for (int dx = 0; dx < 2; ++dx) {
                const int x = 2 * bx + dx;
                if (x >= width) continue;
                const long long i = static_cast<long long>(y) * width + x;
                const int r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
                y_plane[i] = static_cast<std::uint8_t>(luma(r, g, b));
                sr += r;
                sg += g;
                sb += b;
                ++n;
            }
        }
        const int r = (sr + n / 2) / n, g = (sg + n / 2) / n, b = (sb + n / 2) / n;
        const std::uint8_t u = static_cast<std::uint8_t>(chroma_u(r, g, b));
        const std::uint8_t v = static_cast<std::uint8_t>(chroma_v(r, g, b));
        if (interleaved) {
            u_plane[2 * k] = u;
            u_plane[2 * k + 1] = v;
        } else {
            u_plane[k] = u;
            v_plane[k] = v;
        }
    }
}

// The same conversion for the common frame shape (width a multiple of 4,
// even height, 4-byte aligned buffers): one thread per 4x2 pixels, i.e. two
// chroma blocks side by side, with 4-byte loads and stores (three words of
// RGB per row in, one word of Y per row, one word of interleaved U/V or two
// half-words of U and V out).
__global__ void pack_yuv_wide_kernel(const std::uint8_t* __restrict__ rgb, std::uint8_t* __restrict__ out,
                                     int width, int height, int interleaved) {
    const int quads = width >> 2, rows = height >> 1;
    const long long units = static_cast<long long>(quads) * rows;
    const long long chroma_blocks = static_cast<long long>(width >> 1) * rows;
    std::uint8_t* y_plane = out;
    std::uint8_t* u_plane = out + static_cast<long long>(width) * height;
    std::uint8_t* v_plane = u_plane + chroma_blocks;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < units;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int by = static_cast<int>(t / quads), qx = static_cast<int>(t - static_cast<long long>(by) * quads);
        const int x0 = qx << 2;
        int sr[2] = {0, 0}, sg[2] = {0, 0}, sb[2] = {0, 0};
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const long long i = static_cast<long long>(2 * by + dy) * width + x0;
            const std::uint32_t* src = reinterpret_cast<const std::uint32_t*>(rgb + 3 * i);
            const std::uint32_t w0 = __ldg(src), w1 = __ldg(src + 1), w2 = __ldg(src + 2);
            // Bytes r0 g0 b0 r1 | g1 b1 r2 g2 | b2 r3 g3 b3.
            const int r[4] = {static_cast<int>(w0 & 255), static_cast<int>(w0 >> 24), static_cast<int>((w1 >> 16) & 255),
                              static_cast<int>((w2 >> 8) & 255)};
            const int g[4] = {static_cast<int>((w0 >> 8) & 255), static_cast<int>(w1 & 255),
                              static_cast<int>(w1 >> 24), static_cast<int>((w2 >> 16) & 255)};
            const int b[4] = {static_cast<int>((w0 >> 16) & 255), static_cast<int>((w1 >> 8) & 255),
                              static_cast<int>(w2 & 255), static_cast<int>(w2 >> 24)};
            std::uint32_t luma_word = 0;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                luma_word |= static_cast<std::uint32_t>(luma(r[p], g[p], b[p])) << (8 * p);
                sr[p >> 1] += r[p];
                sg[p >> 1] += g[p];
                sb[p >> 1] += b[p];
            }
            *reinterpret_cast<std::uint32_t*>(y_plane + i) = luma_word;
        }
        std::uint32_t u[2], v[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int r = (sr[c] + 2) >> 2, g = (sg[c] + 2) >> 2, b = (sb[c] + 2) >> 2;
            u[c] = static_cast<std::uint32_t>(chroma_u(r, g, b));
            v[c] = static_cast<std::uint32_t>(chroma_v(r, g, b));
        }
        const long long k = static_cast<long long>(by) * (width >> 1) + (qx << 1);  // first of the two blocks
        if (interleaved) {
            *reinterpret_cast<std::uint32_t*>(u_plane + 2 * k) = u[0] | (v[0] << 8) | (u[1] << 16) | (v[1] << 24);
        } else {
            *reinterpret_cast<std::uint16_t*>(u_plane + k) = static_cast<std::uint16_t>(u[0] | (u[1] << 8));
            *reinterpret_cast<std::uint16_t*>(v_plane + k) = static_cast<std::uint16_t>(v[0] | (v[1] << 8));
        }
    }
}

}  // namespace

std::size_t packed_frame_bytes(int width, int height, int format) {
    const std::size_t pixels = static_cast<std::size_t>(width) * height;
    const std::size_t chroma = static_cast<std::size_t>((width + 1) / 2) * ((height + 1) / 2);
    switch (format) {
        case 0: return pixels * 3;
        case 1:
        case 2: return pixels * 4;
        case 3:
        case 4: return pixels + 2 * chroma;
        default: return 0;
    }
}

cudaError_t launch_pack_frame(const std::uint8_t* rgb, int width, int height, int format, std::uint8_t* out,
                              cudaStream_t stream) {
    int device = 0, sms = 152;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const long long pixels = static_cast<long long>(width) * height;
    if (format == 0) return cudaMemcpyAsync(out, rgb, pixels * 3, cudaMemcpyDeviceToDevice, stream);
    const unsigned blocks = static_cast<unsigned>(sms) * 8;
    if (format == 1 || format == 2) {
        const std::uint32_t alpha = format == 2 ? 255u : 0u;
        if ((reinterpret_cast<std::uintptr_t>(rgb) & 3) == 0 && (reinterpret_cast<std::uintptr_t>(out) & 15) == 0
            && pixels >= 4) {
            const long long quads = pixels / 4;
            const unsigned wide = static_cast<unsigned>((quads + 255) / 256 < blocks ? (quads + 255) / 256 : blocks);
            pack_rgbx_wide_kernel<<<wide, 256, 0, stream>>>(rgb, reinterpret_cast<uint4*>(out), quads, alpha);
            const long long done = quads * 4;
            if (done < pixels) {
                pack_rgbx_kernel<<<1, 32, 0, stream>>>(rgb + 3 * done, reinterpret_cast<std::uint32_t*>(out) + done,
                                                       pixels - done, alpha);
            }
        } else {
            pack_rgbx_kernel<<<blocks, 256, 0, stream>>>(rgb, reinterpret_cast<std::uint32_t*>(out), pixels, alpha);
        }
    } else if (width % 4 == 0 && height % 2 == 0 && (reinterpret_cast<std::uintptr_t>(rgb) & 3) == 0
               && (reinterpret_cast<std::uintptr_t>(out) & 3) == 0) {
        const long long units = static_cast<long long>(width / 4) * (height / 2);
        const unsigned wide = static_cast<unsigned>((units + 255) / 256 < blocks ? (units + 255) / 256 : blocks);
        pack_yuv_wide_kernel<<<wide > 0 ? wide : 1, 256, 0, stream>>>(rgb, out, width, height, format == 4 ? 1 : 0);
    } else {
        pack_yuv_kernel<<<blocks, 256, 0, stream>>>(rgb, out, width, height, format == 4 ? 1 : 0);
    }
    return cudaGetLastError();
}

}  // namespace fgb
