// Tile-cost network: parameters, forward, backward and Adam on the GPU.
//
// Layers: h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = w3 . h2 + b3 with
// x the 320 features of a tile (mlp.h).  The three matrix products of a
// training step (x W1^T, h1 W2^T, and the backward products dZ2 W2,
// dZ2^T h1, dZ1^T x) run on the tensor cores through mlp::gemm with BF16
// operands and FP32 accumulation; everything else (output layer, loss,
// bias sums, ReLU backward for the output layer, Adam) is small and runs on
// the CUDA cores.  Intermediate activations and gradients are stored in
// BF16 where they feed a tensor-core product; the CPU check of the gradients
// (oracle/costnet.py) rounds at the same places.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "mlp.h"

namespace fgb {
namespace mlp {

namespace {

constexpr int kW1 = kHidden * kFeatures;
constexpr int kW2 = kHidden * kHidden;
constexpr std::size_t kParams = static_cast<std::size_t>(kW1) + kHidden + kW2 + kHidden + kHidden + 1;

// Offsets of each parameter block in the flat vector.
constexpr std::size_t kOffW1 = 0;
constexpr std::size_t kOffB1 = kOffW1 + kW1;
constexpr std::size_t kOffW2 = kOffB1 + kHidden;
constexpr std::size_t kOffB2 = kOffW2 + kW2;
constexpr std::size_t kOffW3 = kOffB2 + kHidden;
constexpr std::size_t kOffB3 = kOffW3 + kHidden;

__global__ void to_bf16_kernel(const float* src, __nv_bfloat16* dst, int rows, int cols, __nv_bfloat16* dst_t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int r = i / cols, c = i - r * cols;
    const __nv_bfloat16 v = __float2bfloat16_rn(src[i]);
    if (dst) dst[i] = v;
    if (dst_t) dst_t[static_cast<long long>(c) * rows + r] = v;
}

// x [batch x 320] -> x^T [320 x batch] (rows beyond 320 stay zero).
__global__ void transpose_bf16_kernel(const __nv_bfloat16* x, __nv_bfloat16* xt, int batch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch * kFeatures) return;
    const int b = i / kFeatures, f = i - b * kFeatures;
    xt[static_cast<long long>(f) * batch + b] = x[i];
}

// y[b] = sum_j h2[b][j] * w3[j] + b3 (BF16 inputs, FP32 sum).
__global__ void output_kernel(const __nv_bfloat16* h2, const __nv_bfloat16* w3, const float* b3, float* y,
                              int rows) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float sum = 0.0f;
    for (int j = lane; j < kHidden; j += 32) {
        sum += __bfloat162float(h2[static_cast<long long>(warp) * kHidden + j]) * __bfloat162float(w3[j]);
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) y[warp] = sum + b3[0];
}

// dy = 2 (y - t) / B and the batch loss (one block).
__global__ void loss_kernel(const float* y, const float* t, float* dy, float* loss, int batch) {
    __shared__ float partial[256];
    float sum = 0.0f;
    for (int b = threadIdx.x; b < batch; b += blockDim.x) {
        const float d = y[b] - t[b];
        dy[b] = 2.0f * d / static_cast<float>(batch);
        sum += d * d;
    }
    partial[threadIdx.x] = sum;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) partial[threadIdx.x] += partial[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = partial[0] / static_cast<float>(batch);
}

// Output-layer backward: dZ2 = dy w3 (where h2 > 0), in BF16 both ways.
__global__ void output_backward_kernel(const float* dy, const __nv_bfloat16* w3, const __nv_bfloat16* h2,
                                       __nv_bfloat16* dz2, __nv_bfloat16* dz2_t, int batch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch * kHidden) return;
    const int b = i / kHidden, j = i - b * kHidden;
    const float g = __bfloat162float(h2[i]) > 0.0f ? dy[b] * __bfloat162float(w3[j]) : 0.0f;
    const __nv_bfloat16 v = __float2bfloat16_rn(g);
    dz2[i] = v;
    dz2_t[static_cast<long long>(j) * batch + b] = v;
}

// Row sums of a [rows x cols] BF16 matrix (one warp per row): bias
// gradients from transposed layer gradients.
__global__ void row_sum_kernel(const __nv_bfloat16* m, float* out, int rows, int cols) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float sum = 0.0f;
    for (int c = lane; c < cols; c += 32) sum += __bfloat162float(m[static_cast<long long>(warp) * cols + c]);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) out[warp] = sum;
}

// gw3[j] = sum_b dy[b] h2[b][j]; gb3 = sum_b dy[b] (one warp per j, plus one).
__global__ void output_grad_kernel(const float* dy, const __nv_bfloat16* h2, float* gw3, float* gb3, int batch) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp > kHidden) return;
    float sum = 0.0f;
    for (int b = lane; b < batch; b += 32) {
        sum += warp == kHidden ? dy[b] : dy[b] * __bfloat162float(h2[static_cast<long long>(b) * kHidden + warp]);
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
        if (warp == kHidden) *gb3 = sum;
        else gw3[warp] = sum;
    }
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int n, float lr, float beta1, float beta2,
                            float c1, float c2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

template <typename T>
T* device_alloc(std::size_t count, std::string& why) {
    void* p = nullptr;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
        why = "cudaMalloc (cost network)";
        return nullptr;
    }
    cudaMemset(p, 0, count * sizeof(T));
    return static_cast<T*>(p);
}

unsigned blocks(long long n, int threads) { return static_cast<unsigned>((n + threads - 1) / threads); }

}  // namespace

struct CostNet {
    int device = -1;
    float* params = nullptr;  // FP32 masters, flat (kParams)
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    long long step = 0;
    __nv_bfloat16* w1 = nullptr;    // [256 x 320]
    __nv_bfloat16* w2 = nullptr;    // [256 x 256]
    __nv_bfloat16* w2_t = nullptr;  // [256 x 256]
    __nv_bfloat16* w3 = nullptr;    // [256]
    int* error = nullptr;
    float* loss = nullptr;
    // Workspace for `capacity` rows.
    int capacity = 0;
    __nv_bfloat16 *h1 = nullptr, *h1_t = nullptr, *h2 = nullptr, *dz2 = nullptr, *dz2_t = nullptr;
    __nv_bfloat16 *dz1 = nullptr, *dz1_t = nullptr, *x_t = nullptr;
    float *y = nullptr, *dy = nullptr;
};

namespace {

void free_workspace(CostNet* n) {
    for (void* p : {static_cast<void*>(n->h1), static_cast<void*>(n->h1_t), static_cast<void*>(n->h2),
                    static_cast<void*>(n->dz2), static_cast<void*>(n->dz2_t), static_cast<void*>(n->dz1),
                    static_cast<void*>(n->dz1_t), static_cast<void*>(n->x_t), static_cast<void*>(n->y),
                    static_cast<void*>(n->dy)}) {
        cudaFree(p);
    }
    n->h1 = n->h1_t = n->h2 = n->dz2 = n->dz2_t = n->dz1 = n->dz1_t = n->x_t = nullptr;
    n->y = n->dy = nullptr;
    n->capacity = 0;
}

bool reserve(CostNet* n, int rows, std::string& why) {
    if (rows <= n->capacity) return true;
    cudaDeviceSynchronize();
    free_workspace(n);
    const std::size_t r = static_cast<std::size_t>(rows);
    if (!(n->h1 = device_alloc<__nv_bfloat16>(r * kHidden, why)) || !(n->h1_t = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->h2 = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->dz2 = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->dz2_t = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->dz1 = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->dz1_t = device_alloc<__nv_bfloat16>(r * kHidden, why))
        || !(n->x_t = device_alloc<__nv_bfloat16>(r * 512, why))  // 320 rows used, 512 = two 256-row boxes
        || !(n->y = device_alloc<float>(r, why)) || !(n->dy = device_alloc<float>(r, why))) {
        free_workspace(n);
        return false;
    }
    n->capacity = rows;
    return true;
}

// Refresh the BF16 weight copies from the FP32 masters.
bool refresh(CostNet* n, cudaStream_t s, std::string& why) {
    to_bf16_kernel<<<blocks(kW1, 256), 256, 0, s>>>(n->params + kOffW1, n->w1, kHidden, kFeatures, nullptr);
    to_bf16_kernel<<<blocks(kW2, 256), 256, 0, s>>>(n->params + kOffW2, n->w2, kHidden, kHidden, n->w2_t);
    to_bf16_kernel<<<blocks(kHidden, 256), 256, 0, s>>>(n->params + kOffW3, n->w3, 1, kHidden, nullptr);
    const cudaError_t status = cudaGetLastError();
    if (status != cudaSuccess) {
        why = std::string("weight conversion: ") + cudaGetErrorString(status);
        return false;
    }
    return true;
}

Epilogue epilogue() {
    Epilogue e;
    std::memset(&e, 0, sizeof e);
    return e;
}

// Forward through both hidden layers and the output for `rows` rows.
bool forward(CostNet* n, const __nv_bfloat16* x, int rows, float* y, cudaStream_t s, std::string& why) {
    Epilogue e1 = epilogue();
    e1.bias = n->params + kOffB1;
    e1.relu = 1;
    e1.out_bf16 = n->h1;
    e1.ld_out = kHidden;
    e1.out_bf16_t = n->h1_t;
    e1.ld_out_t = rows;
    e1.rows = rows;
    e1.cols = kHidden;
    if (!gemm(GemmShape{x, n->w1, rows, kHidden, kFeatures, kHidden}, e1, n->error, s, why)) return false;
    Epilogue e2 = epilogue();
    e2.bias = n->params + kOffB2;
    e2.relu = 1;
    e2.out_bf16 = n->h2;
    e2.ld_out = kHidden;
    e2.rows = rows;
    e2.cols = kHidden;
    if (!gemm(GemmShape{n->h1, n->w2, rows, kHidden, kHidden, kHidden}, e2, n->error, s, why)) return false;
    output_kernel<<<blocks(static_cast<long long>(rows) * 32, 256), 256, 0, s>>>(n->h2, n->w3, n->params + kOffB3, y,
                                                                                 rows);
    return true;
}

bool check_error(CostNet* n, cudaStream_t s, std::string& why) {
    int flag = 0;
    if (cudaMemcpyAsync(&flag, n->error, sizeof flag, cudaMemcpyDeviceToHost, s) != cudaSuccess
        || cudaStreamSynchronize(s) != cudaSuccess) {
        why = "cost network: CUDA error after the GEMMs";
        return false;
    }
    if (flag) {
        why = "cost network: a tensor-core GEMM gave up waiting on its barrier";
        cudaMemsetAsync(n->error, 0, sizeof(int), s);
        return false;
    }
    return true;
}

}  // namespace

std::size_t parameter_count() { return kParams; }

CostNet* create(unsigned seed, std::string& why) {
    auto* n = new CostNet();
    cudaGetDevice(&n->device);
    if (!(n->params = device_alloc<float>(kParams, why)) || !(n->grads = device_alloc<float>(kParams, why))
        || !(n->adam_m = device_alloc<float>(kParams, why)) || !(n->adam_v = device_alloc<float>(kParams, why))
        || !(n->w1 = device_alloc<__nv_bfloat16>(kW1, why)) || !(n->w2 = device_alloc<__nv_bfloat16>(kW2, why))
        || !(n->w2_t = device_alloc<__nv_bfloat16>(kW2, why)) || !(n->w3 = device_alloc<__nv_bfloat16>(kHidden, why))
        || !(n->error = device_alloc<int>(1, why)) || !(n->loss = device_alloc<float>(1, why))) {
        destroy(n);
        return nullptr;
    }
    // He-uniform initial weights from a seeded 64-bit LCG (inputs beyond the
    // 258 real features start at zero), zero biases.
    std::vector<float> host(kParams, 0.0f);
    std::uint64_t state = 0x9E3779B97F4A7C15ull ^ (static_cast<std::uint64_t>(seed) * 0xD1B54A32D192ED03ull);
    auto uniform = [&state] {
        state = state * 6364136223846793005ull + 1442695040888963407ull;
        return static_cast<float>((state >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f;
    };
    const float a1 = std::sqrt(6.0f / static_cast<float>(kProbe + 2));
    for (int r = 0; r < kHidden; ++r) {
        for (int c = 0; c < kProbe + 2; ++c) host[kOffW1 + static_cast<std::size_t>(r) * kFeatures + c] = a1 * uniform();
    }
    const float a2 = std::sqrt(6.0f / static_cast<float>(kHidden));
    for (int i = 0; i < kW2; ++i) host[kOffW2 + i] = a2 * uniform();
    for (int i = 0; i < kHidden; ++i) host[kOffW3 + i] = 0.1f * a2 * uniform();
    if (!set_parameters(n, host.data(), host.size(), why)) {
        destroy(n);
        return nullptr;
    }
    return n;
}

void destroy(CostNet* n) {
    if (!n) return;
    cudaDeviceSynchronize();
    free_workspace(n);
    for (void* p : {static_cast<void*>(n->params), static_cast<void*>(n->grads), static_cast<void*>(n->adam_m),
                    static_cast<void*>(n->adam_v), static_cast<void*>(n->w1), static_cast<void*>(n->w2),
                    static_cast<void*>(n->w2_t), static_cast<void*>(n->w3), static_cast<void*>(n->error),
                    static_cast<void*>(n->loss)}) {
        cudaFree(p);
    }
    delete n;
}

bool get_parameters(CostNet* n, std::vector<float>& out, std::string& why) {
    out.resize(kParams);
    if (cudaMemcpy(out.data(), n->params, kParams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        why = "copy of cost-network parameters failed";
        return false;
    }
    return true;
}

bool set_parameters(CostNet* n, const float* values, std::size_t count, std::string& why) {
    if (count != kParams) {
        why = "cost network expects " + std::to_string(kParams) + " parameters";
        return false;
    }
    if (cudaMemcpy(n->params, values, kParams * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        why = "upload of cost-network parameters failed";
        return false;
    }
    cudaMemset(n->adam_m, 0, kParams * sizeof(float));
    cudaMemset(n->adam_v, 0, kParams * sizeof(float));
    n->step = 0;
    if (!refresh(n, nullptr, why)) return false;
    return cudaDeviceSynchronize() == cudaSuccess;
}

bool predict(CostNet* n, const __nv_bfloat16* x, int rows, float* out, cudaStream_t s, std::string& why) {
    if (rows <= 0 || rows % 128 != 0) {
        why = "cost-network rows must be a positive multiple of 128";
        return false;
    }
    if (!reserve(n, rows, why)) return false;
    if (!forward(n, x, rows, out, s, why)) return false;
    return check_error(n, s, why);
}

bool reserve_rows(CostNet* n, int rows, std::string& why) { return reserve(n, rows, why); }

bool predict_async(CostNet* n, const __nv_bfloat16* x, int rows, float* out, cudaStream_t s, std::string& why) {
    if (rows <= 0 || rows % 128 != 0 || rows > n->capacity) {
        why = "cost-network rows must be a positive multiple of 128 within the reserved workspace";
        return false;
    }
    return forward(n, x, rows, out, s, why);
}

bool train_step(CostNet* n, const __nv_bfloat16* x, const float* target, int batch, float learning_rate, bool update,
                float* loss, std::vector<float>* grads, cudaStream_t s, std::string& why) {
    if (batch <= 0 || batch % 128 != 0) {
        why = "cost-network batch must be a positive multiple of 128";
        return false;
    }
    if (!reserve(n, batch, why)) return false;
    if (!forward(n, x, batch, n->y, s, why)) return false;
    loss_kernel<<<1, 256, 0, s>>>(n->y, target, n->dy, n->loss, batch);
    // Output layer.
    output_grad_kernel<<<blocks(static_cast<long long>(kHidden + 1) * 32, 256), 256, 0, s>>>(
        n->dy, n->h2, n->grads + kOffW3, n->grads + kOffB3, batch);
    output_backward_kernel<<<blocks(static_cast<long long>(batch) * kHidden, 256), 256, 0, s>>>(
        n->dy, n->w3, n->h2, n->dz2, n->dz2_t, batch);
    // Second layer: dW2 = dZ2^T h1, db2 = row sums of dZ2^T.
    Epilogue g2 = epilogue();
    g2.out_f32 = n->grads + kOffW2;
    g2.ld_out = kHidden;
    g2.rows = kHidden;
    g2.cols = kHidden;
    if (!gemm(GemmShape{n->dz2_t, n->h1_t, kHidden, kHidden, batch, kHidden}, g2, n->error, s, why)) return false;
    row_sum_kernel<<<blocks(static_cast<long long>(kHidden) * 32, 256), 256, 0, s>>>(n->dz2_t, n->grads + kOffB2,
                                                                                    kHidden, batch);
    // dZ1 = (dZ2 W2) masked by h1 > 0.
    Epilogue d1 = epilogue();
    d1.mask = n->h1;
    d1.ld_mask = kHidden;
    d1.out_bf16 = n->dz1;
    d1.ld_out = kHidden;
    d1.out_bf16_t = n->dz1_t;
    d1.ld_out_t = batch;
    d1.rows = batch;
    d1.cols = kHidden;
    if (!gemm(GemmShape{n->dz2, n->w2_t, batch, kHidden, kHidden, kHidden}, d1, n->error, s, why)) return false;
    row_sum_kernel<<<blocks(static_cast<long long>(kHidden) * 32, 256), 256, 0, s>>>(n->dz1_t, n->grads + kOffB1,
                                                                                    kHidden, batch);
    // First layer: dW1 = dZ1^T x.
    transpose_bf16_kernel<<<blocks(static_cast<long long>(batch) * kFeatures, 256), 256, 0, s>>>(x, n->x_t, batch);
    Epilogue g1 = epilogue();
    g1.out_f32 = n->grads + kOffW1;
    g1.ld_out = kFeatures;
    g1.rows = kHidden;
    g1.cols = kFeatures;
    if (!gemm(GemmShape{n->dz1_t, n->x_t, kHidden, kFeatures, batch, 512}, g1, n->error, s, why)) return false;
    if (update) {
        ++n->step;
        const float beta1 = 0.9f, beta2 = 0.999f;
        const float c1 = 1.0f - std::pow(beta1, static_cast<float>(n->step));
        const float c2 = 1.0f - std::pow(beta2, static_cast<float>(n->step));
        adam_kernel<<<blocks(static_cast<long long>(kParams), 256), 256, 0, s>>>(
            n->params, n->grads, n->adam_m, n->adam_v, static_cast<int>(kParams), learning_rate, beta1, beta2, c1, c2,
            1e-8f);
        if (!refresh(n, s, why)) return false;
    }
    if (loss && cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
        why = "loss copy failed";
        return false;
    }
    if (grads) {
        grads->resize(kParams);
        if (cudaMemcpyAsync(grads->data(), n->grads, kParams * sizeof(float), cudaMemcpyDeviceToHost, s)
            != cudaSuccess) {
            why = "gradient copy failed";
            return false;
        }
    }
    return check_error(n, s, why);
}

}  // namespace mlp
}  // namespace fgb
