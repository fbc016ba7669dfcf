// FMA-pipe throughput probe: the FP64 / FP32 roofline denominators for the
// iteration kernels, measured on the device the renders run on.  Each thread
// runs eight independent FMA chains; the result is 2 * FMAs / kernel time.
#include <cuda_runtime.h>

#include "fractal_gb300.h"
#include "runtime.h"

namespace fgb {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T* sink, int rounds, T a, T b) {
    T x0 = static_cast<T>(threadIdx.x), x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int r = 0; r < rounds; ++r) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    const T total = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (total == static_cast<T>(-1.2345)) sink[threadIdx.x] = total;  // keeps the chains live
}

template <typename T>
double measure(ThreadRuntime& rt, int rounds) {
    int device = 0, sms = 1;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8;
    T* sink = static_cast<T*>(scratch(rt, kScratchWork, 256 * sizeof(T)));
    fma_chains<T><<<blocks, 256, 0, rt.stream>>>(sink, 4, static_cast<T>(0.999), static_cast<T>(0.001));
    check_cuda(cudaGetLastError(), "FMA probe launch");
    check_cuda(cudaEventRecord(rt.start, rt.stream), "cudaEventRecord");
    fma_chains<T><<<blocks, 256, 0, rt.stream>>>(sink, rounds, static_cast<T>(0.999), static_cast<T>(0.001));
    check_cuda(cudaEventRecord(rt.stop, rt.stream), "cudaEventRecord");
    check_cuda(cudaStreamSynchronize(rt.stream), "FMA probe");
    float ms = 0.0f;
    check_cuda(cudaEventElapsedTime(&ms, rt.start, rt.stop), "cudaEventElapsedTime");
    const double fmas = static_cast<double>(blocks) * 256.0 * rounds * 16.0 * 8.0;
    return 2.0 * fmas / (static_cast<double>(ms) * 1.0e-3) / 1.0e12;
}

}  // namespace
}  // namespace fgb

extern "C" int fractal_gb300_fma_peak(int precision_bits, double* tflops) {
    try {
        if (!tflops || (precision_bits != 32 && precision_bits != 64)) return 1;
        fgb::ThreadRuntime& rt = fgb::thread_runtime();
        *tflops = precision_bits == 64 ? fgb::measure<double>(rt, 2048) : fgb::measure<float>(rt, 16384);
        return 0;
    } catch (...) {
        return 1;
    }
}
