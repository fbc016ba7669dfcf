// Tile-cost network and its tensor-core GEMM (mlp.cu, costnet.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace fgb {
namespace mlp {

constexpr int kProbeSide = 16;                       // coarse probe per tile side
constexpr int kProbe = kProbeSide * kProbeSide;      // 256 probe counts
constexpr int kFeatures = 320;                       // 256 + log zoom + log cap, zero padded to 5 x 64
constexpr int kHidden = 256;
constexpr int kTile = 64;                            // tile side in pixels

// C = A * B^T.  A: [m x k] row-major BF16; B: [b_rows x k] row-major BF16 of
// which the first n rows are used (b_rows a multiple of 256, zero padded).
struct GemmShape {
    const void* a;
    const void* b;
    int m, n, k;
    int b_rows;
};

// Fused epilogue: x = acc (+ bias[col]) (ReLU) (x 0 where mask <= 0); store
// FP32 and/or BF16 row-major and/or BF16 transposed.  rows/cols bound the
// stores.
struct Epilogue {
    const float* bias;
    int relu;
    const __nv_bfloat16* mask;
    int ld_mask;
    float* out_f32;
    __nv_bfloat16* out_bf16;
    int ld_out;
    __nv_bfloat16* out_bf16_t;
    int ld_out_t;
    int rows;
    int cols;
};

bool gemm(const GemmShape& shape, const Epilogue& epilogue, int* error, cudaStream_t stream, std::string& why);

struct CostNet;

CostNet* create(unsigned seed, std::string& why);
void destroy(CostNet* net);
// Parameter vector order: W1 [256 x 320], b1 [256], W2 [256 x 256], b2 [256],
// w3 [256], b3 [1].
std::size_t parameter_count();
bool get_parameters(CostNet* net, std::vector<float>& out, std::string& why);
bool set_parameters(CostNet* net, const float* values, std::size_t count, std::string& why);
// x: device BF16 [rows x 320]; rows a multiple of 128.
bool predict(CostNet* net, const __nv_bfloat16* x, int rows, float* out, cudaStream_t stream, std::string& why);
// The same forward pass enqueued without synchronising (capturable in a
// graph once reserve_rows has sized the workspace); a GEMM that gave up
// waiting is reported by the next synchronous call.
bool reserve_rows(CostNet* net, int rows, std::string& why);
bool predict_async(CostNet* net, const __nv_bfloat16* x, int rows, float* out, cudaStream_t stream, std::string& why);
// One Adam step on mean squared error; `grads` (optional, host) receives the
// gradient in parameter order and `loss` the batch loss.  batch % 128 == 0.
bool train_step(CostNet* net, const __nv_bfloat16* x, const float* target, int batch, float learning_rate,
                bool update, float* loss, std::vector<float>* grads, cudaStream_t stream, std::string& why);

}  // namespace mlp
}  // namespace fgb
