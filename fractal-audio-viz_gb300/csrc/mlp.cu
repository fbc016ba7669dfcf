// Tile-cost network: a small MLP (258 inputs padded to 320, two hidden
// layers of 256 with ReLU, one output) that predicts the log render cost of
// a 64x64 tile from a 16x16 coarse probe of its iteration counts plus the
// field's log zoom and cap.  The persistent floatexp queue uses the
// predictions to start the heaviest tiles first; the network never touches
// a pixel value.
//
// The three matrix products of each forward/backward pass run on the
// tensor cores through hand-written tcgen05 kernels: BF16 operands staged in
// shared memory by TMA (cp.async.bulk.tensor, no swizzle, K-major core
// matrices), the FP32 accumulator in TMEM (128 lanes x up to 256 columns),
// read back with tcgen05.ld for a fused epilogue (bias, ReLU, ReLU mask,
// BF16 store in both orientations).  Weights are BF16 copies of FP32 master
// weights; Adam updates the masters.  Every wait on an mbarrier is bounded
// and reports through an error word instead of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mlp.h"

namespace fgb {
namespace mlp {
namespace {

constexpr int kBM = 128;             // rows per CTA (TMEM lanes)
constexpr int kBN = 256;             // columns per CTA (TMEM columns, FP32)
constexpr int kBK = 64;              // K per stage (8 core-matrix groups of 8)
constexpr int kGroups = kBK / 8;
constexpr unsigned kABytes = kGroups * kBM * 16;  // 16 KB
constexpr unsigned kBBytes = kGroups * kBN * 16;  // 32 KB
constexpr unsigned kSmemBytes = kABytes + kBBytes + 64 + 1024;
constexpr unsigned kSpinLimit = 1u << 24;

__device__ __forceinline__ std::uint32_t smem_addr(const void* p) {
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of
// 8 rows x 16 bytes; `lbo` = byte distance between core matrices along K,
// `sbo` = byte distance between 8-row groups along M/N.
__device__ __forceinline__ std::uint64_t matrix_desc(std::uint32_t address, std::uint32_t lbo, std::uint32_t sbo) {
    std::uint64_t d = 0;
    d |= static_cast<std::uint64_t>((address >> 4) & 0x3FFFu);
    d |= static_cast<std::uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<std::uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<std::uint64_t>(1) << 46;  // descriptor version
    return d;                                   // base offset 0, layout: no swizzle
}

// Instruction descriptor of tcgen05.mma kind::f16: D = F32, A = B = BF16,
// both K-major, M = 128, N = n.
__device__ __forceinline__ std::uint32_t instr_desc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<std::uint32_t>(n >> 3) << 17)
         | (static_cast<std::uint32_t>(kBM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(std::uint32_t bar, std::uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(std::uint32_t bar, std::uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(std::uint32_t bar, std::uint32_t parity) {
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        std::uint32_t done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(std::uint32_t dst, const CUtensorMap* map, int x, int y,
                                            std::uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<std::uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mma_bf16(std::uint32_t tmem, std::uint64_t a, std::uint64_t b, std::uint32_t idesc,
                                         std::uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(std::uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_load8(std::uint32_t taddr, float (&v)[8]) {
    std::uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// C[M x N] = A[M x K] * B[N x K]^T with A, B row-major BF16 (K contiguous),
// M a multiple of 128, N a multiple of 16, K a multiple of 64.  One CTA per
// 128 x 256 tile of C; single-stage TMA -> MMA loop over K.
__global__ void __launch_bounds__(128) umma_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                                                        const __grid_constant__ CUtensorMap tb, const Epilogue ep,
                                                        int n_total, int k_total, int* error) {
    extern __shared__ unsigned char dynamic_smem[];
    const std::uint32_t raw = smem_addr(dynamic_smem);
    const std::uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* base_ptr = dynamic_smem + (base - raw);
    const std::uint32_t a_addr = base;
    const std::uint32_t b_addr = base + kABytes;
    const std::uint32_t tma_bar = base + kABytes + kBBytes;
    const std::uint32_t mma_bar = tma_bar + 8;
    volatile std::uint32_t* tmem_slot = reinterpret_cast<volatile std::uint32_t*>(base_ptr + kABytes + kBBytes + 16);

    const int warp = static_cast<int>(threadIdx.x >> 5);
    const int lane = static_cast<int>(threadIdx.x & 31);
    const int m0 = static_cast<int>(blockIdx.x) * kBM;
    const int n0 = static_cast<int>(blockIdx.y) * kBN;
    const int n_cta = n_total - n0 < kBN ? n_total - n0 : kBN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(const_cast<std::uint32_t*>(tmem_slot))),
                     "r"(static_cast<std::uint32_t>(kBN))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 32) {
        mbar_init(tma_bar, 1);
        mbar_init(mma_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const std::uint32_t tmem = *tmem_slot;

    bool ok = true;
    std::uint32_t phase = 0;
    const int kblocks = k_total / kBK;
    for (int kb = 0; kb < kblocks; ++kb) {
        if (threadIdx.x == 0) {
            mbar_expect_tx(tma_bar, kABytes + kBBytes);
#pragma unroll
            for (int g = 0; g < kGroups; ++g) {
                tma_load_2d(a_addr + g * kBM * 16, &ta, kb * kBK + g * 8, m0, tma_bar);
                tma_load_2d(b_addr + g * kBN * 16, &tb, kb * kBK + g * 8, n0, tma_bar);
            }
        }
        const bool loaded = mbar_wait(tma_bar, phase);
        if (!__syncthreads_and(loaded)) {
            ok = false;
            break;
        }
        if (threadIdx.x == 0) {
            fence_after_sync();
            const std::uint32_t idesc = instr_desc(n_cta);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const std::uint64_t ad = matrix_desc(a_addr + kk * 2 * kBM * 16, kBM * 16, 128);
                const std::uint64_t bd = matrix_desc(b_addr + kk * 2 * kBN * 16, kBN * 16, 128);
                mma_bf16(tmem, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(mma_bar);
        }
        const bool done = mbar_wait(mma_bar, phase);
        if (!__syncthreads_and(done)) {
            ok = false;
            break;
        }
        phase ^= 1u;
    }

    fence_after_sync();
    if (ok) {
        const int row = m0 + warp * 32 + lane;
        for (int c = 0; c < n_cta; c += 8) {
            float v[8];
            tmem_load8(tmem + (static_cast<std::uint32_t>(warp * 32) << 16) + static_cast<std::uint32_t>(c), v);
            if (row >= ep.rows) continue;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int col = n0 + c + j;
                if (col >= ep.cols) continue;
                float x = v[j];
                if (ep.bias) x += ep.bias[col];
                if (ep.relu) x = x > 0.0f ? x : 0.0f;
                if (ep.mask) {
                    // ReLU backward: pass the gradient where the layer's
                    // activation was positive.
                    if (!(__bfloat162float(ep.mask[static_cast<long long>(row) * ep.ld_mask + col]) > 0.0f)) x = 0.0f;
                }
                if (ep.out_f32) ep.out_f32[static_cast<long long>(row) * ep.ld_out + col] = x;
                if (ep.out_bf16) ep.out_bf16[static_cast<long long>(row) * ep.ld_out + col] = __float2bfloat16_rn(x);
                if (ep.out_bf16_t) ep.out_bf16_t[static_cast<long long>(col) * ep.ld_out_t + row] = __float2bfloat16_rn(x);
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(error, 1);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(static_cast<std::uint32_t>(kBN))
                     : "memory");
    }
}

// ----------------------------------------------------------- host: maps

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q)
                == cudaSuccess
            && q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        }
    });
    return fn;
}

// Tensor map of a row-major BF16 matrix [rows x cols] (cols contiguous) read
// in boxes of 8 columns (16 bytes) x box_rows rows.
bool make_map(CUtensorMap& map, const void* base, int rows, int cols, int box_rows, std::string& why) {
    auto fn = encode_fn();
    if (!fn) {
        why = "cuTensorMapEncodeTiled is unavailable";
        return false;
    }
    if ((reinterpret_cast<std::uintptr_t>(base) & 15u) != 0 || (cols * 2) % 16 != 0) {
        why = "tensor map base or row pitch is not 16-byte aligned";
        return false;
    }
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(cols) * 2};
    const cuuint32_t box[2] = {8u, static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t element_strides[2] = {1u, 1u};
    const CUresult r = fn(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
                          element_strides, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        why = "cuTensorMapEncodeTiled failed (" + std::to_string(static_cast<int>(r)) + ")";
        return false;
    }
    return true;
}

}  // namespace

bool gemm(const GemmShape& s, const Epilogue& ep, int* error, cudaStream_t stream, std::string& why) {
    if (s.m <= 0 || s.m % kBM != 0 || s.n <= 0 || s.n % 16 != 0 || s.k <= 0 || s.k % kBK != 0) {
        why = "GEMM shape must be M % 128 == 0, N % 16 == 0, K % 64 == 0";
        return false;
    }
    if (s.b_rows < ((s.n + kBN - 1) / kBN) * kBN) {
        why = "GEMM B operand must hold whole 256-row boxes";
        return false;
    }
    CUtensorMap ta, tb;
    if (!make_map(ta, s.a, s.m, s.k, kBM, why) || !make_map(tb, s.b, s.b_rows, s.k, kBN, why)) return false;
    static bool attribute_set = false;
    if (!attribute_set) {
        if (cudaFuncSetAttribute(umma_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSmemBytes)) != cudaSuccess) {
            why = "cudaFuncSetAttribute (GEMM shared memory) failed";
            return false;
        }
        attribute_set = true;
    }
    const dim3 grid(static_cast<unsigned>(s.m / kBM), static_cast<unsigned>((s.n + kBN - 1) / kBN));
    umma_gemm_kernel<<<grid, 128, kSmemBytes, stream>>>(ta, tb, ep, s.n, s.k, error);
    const cudaError_t status = cudaGetLastError();
    if (status != cudaSuccess) {
        why = std::string("GEMM launch: ") + cudaGetErrorString(status);
        return false;
    }
    return true;
}

}  // namespace mlp
}  // namespace fgb
