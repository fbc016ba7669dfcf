// BLA hierarchy construction on the GPU.
//
// Level 0 holds one single-step map per reference index; level L merges the
// pairs of level L-1 (y after x).  Every level is a data-parallel map, one
// thread per output step, one launch per level; the builder form (FloatExp
// complex coefficients) ping-pongs between two device buffers while the
// compact render form is written straight into the table the kernels read.
// The arithmetic is bla_math.h compiled with --fmad=false, the same
// definitions the host builder uses, so both produce identical tables
// (build_bla / build_alternate_linear_bla / retarget_*, renderer.cpp:11336-
// 11868).  FP32 mirrors for the floatexp form are converted here as well.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bla_math.h"
#include "device.h"
#include "runtime.h"

namespace fgb {
namespace {

constexpr int kThreads = 128;

unsigned blocks_for(long long n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

__global__ void cubic_base_kernel(const fx::Fec* orbit, int count, BuilderCubic* builder, CubicStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const BuilderCubic s = cubic_base(orbit[i + 1]);
    builder[i] = s;
    out[i] = compact_cubic(s);
}

__global__ void cubic_merge_kernel(const BuilderCubic* prev, int count, fx::Fe radius, BuilderCubic* cur,
                                   CubicStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const BuilderCubic s = merge_cubic(prev[2 * i + 1], prev[2 * i], radius);
    cur[i] = s;
    out[i] = compact_cubic(s);
}

__global__ void linear_base_kernel(const fx::Fec* orbit, int count, BuilderLinear* builder, LinearStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const BuilderLinear s = linear_base(orbit[i + 1]);
    builder[i] = s;
    out[i] = compact_linear(s);
}

__global__ void linear_merge_kernel(const BuilderLinear* prev, int prev_count, int count, fx::Fe radius,
                                    BuilderLinear* cur, LinearStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int first = 2 * i;
    const BuilderLinear s = first + 1 < prev_count ? merge_linear(prev[first + 1], prev[first], radius) : prev[first];
    cur[i] = s;
    out[i] = compact_linear(s);
}

__global__ void alt_base_kernel(const fx::Fec* orbit, int first_index, int count, int formula, AltStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    out[i] = alt_base(orbit[first_index + i], formula);
}

__global__ void alt_merge_kernel(const AltStep* prev, int prev_count, int count, fx::Fe radius, AltStep* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int first = 2 * i;
    out[i] = first + 1 < prev_count ? merge_alt(prev[first + 1], prev[first], radius) : prev[first];
}

__global__ void cubic_retarget_kernel(const CubicStep* prev, CubicStep* cur, int count, fx::Fe radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const CubicStep& x = prev[2 * i];
    const CubicStep& y = prev[2 * i + 1];
    cur[i].r2 = retarget_radius(x.r2, y.r2, x.c[0], x.c[1], radius);
}

__global__ void linear_retarget_kernel(const LinearStep* prev, int prev_count, LinearStep* cur, int count,
                                       fx::Fe radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int first = 2 * i;
    if (first + 1 >= prev_count) {
        cur[i].r2 = prev[first].r2;
        return;
    }
    cur[i].r2 = retarget_radius(prev[first].r2, prev[first + 1].r2, prev[first].a, prev[first].b, radius);
}

__device__ f32x::F2e sc_to_f2e(const fx::Sc& v) {
    if (v.re == 0.0 && v.im == 0.0) return f32x::zero();
    return f32x::norm(static_cast<float>(v.re), static_cast<float>(v.im), v.e);
}

__device__ f32x::N1e fe_to_n1e(const fx::Fe& v) {
    f32x::N1e r;
    if (!fx::fe_finite(v)) {
        r.m = 3.0e38f;
        r.e = 0x3fffffff;
        return r;
    }
    if (v.m == 0.0) {
        r.m = 0.0f;
        r.e = 0;
        return r;
    }
    return f32x::n_norm(static_cast<float>(v.m), v.e);
}

__global__ void fx_cubic_kernel(const CubicStep* in, FxCubic* out, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    FxCubic c;
    for (int k = 0; k < 9; ++k) c.c[k] = sc_to_f2e(in[i].c[k]);
    c.r2 = fe_to_n1e(in[i].r2);
    c.len = in[i].len;
    c.pad = 0;
    out[i] = c;
}

__global__ void fx_linear_kernel(const LinearStep* in, FxLinear* out, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    FxLinear l;
    l.a = sc_to_f2e(in[i].a);
    l.b = sc_to_f2e(in[i].b);
    l.r2 = fe_to_n1e(in[i].r2);
    l.len = in[i].len;
    l.pad = 0;
    out[i] = l;
}

__global__ void fx_alt_kernel(const AltStep* in, FxAltStep* out, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    FxAltStep a;
    for (int k = 0; k < 8; ++k) {
        const fx::Fe v = in[i].c[k];
        a.c[k] = fx::fe_finite(v) ? f32x::r_norm(static_cast<float>(v.m), v.e)
                                  : f32x::r_make(v.m < 0.0 ? -3.0e38f : 3.0e38f, 0x3fffffff);
    }
    a.r2 = fe_to_n1e(in[i].r2);
    a.len = in[i].len;
    a.pad = 0;
    out[i] = a;
}

template <typename T>
T* device_alloc(std::size_t count, const char* what) {
    T* p = nullptr;
    if (count == 0) return nullptr;
    check_cuda(cudaMalloc(&p, count * sizeof(T)), what);
    return p;
}

struct Scoped {
    void* p = nullptr;
    ~Scoped() { cudaFree(p); }
};

// Level sizes of a hierarchy: halving (cubic) or halving rounded up with a
// pass-through tail (linear, alternate), up to the maximum block length.
std::vector<int> level_sizes(int base, int max_length, bool round_up) {
    std::vector<int> sizes;
    if (base <= 0) return sizes;
    sizes.push_back(base);
    for (int level = 1; (1LL << level) <= max_length; ++level) {
        const int prev = sizes.back();
        const int cur = round_up ? (prev + 1) / 2 : prev / 2;
        if (cur == 0) break;
        sizes.push_back(cur);
    }
    return sizes;
}

LevelIndex index_of(const std::vector<int>& sizes) {
    LevelIndex index;
    index.levels = static_cast<int>(sizes.size());
    int offset = 0;
    for (std::size_t l = 0; l < sizes.size(); ++l) {
        index.offset[l] = offset;
        index.count[l] = sizes[l];
        offset += sizes[l];
    }
    return index;
}

int total_of(const std::vector<int>& sizes) {
    int total = 0;
    for (int s : sizes) total += s;
    return total;
}

void build_linear(const fx::Fec* orbit, int base_count, const fx::Fe& radius, LinearStep** out, LevelIndex& index,
                  cudaStream_t stream) {
    const std::vector<int> sizes = level_sizes(base_count, kMaxSafeLinearBlaLength, true);
    if (sizes.size() > static_cast<std::size_t>(kMaxLevels)) throw Failure{"too many BLA levels"};
    index = index_of(sizes);
    *out = device_alloc<LinearStep>(static_cast<std::size_t>(total_of(sizes)), "cudaMalloc (linear BLA)");
    Scoped a, b;
    a.p = device_alloc<BuilderLinear>(static_cast<std::size_t>(base_count), "cudaMalloc (BLA builder)");
    b.p = device_alloc<BuilderLinear>(static_cast<std::size_t>((base_count + 1) / 2), "cudaMalloc (BLA builder)");
    BuilderLinear* prev = static_cast<BuilderLinear*>(a.p);
    BuilderLinear* cur = static_cast<BuilderLinear*>(b.p);
    linear_base_kernel<<<blocks_for(base_count), kThreads, 0, stream>>>(orbit, base_count, prev, *out);
    for (std::size_t l = 1; l < sizes.size(); ++l) {
        linear_merge_kernel<<<blocks_for(sizes[l]), kThreads, 0, stream>>>(prev, sizes[l - 1], sizes[l], radius, cur,
                                                                           *out + index.offset[l]);
        std::swap(prev, cur);
    }
    check_cuda(cudaGetLastError(), "linear BLA build");
    check_cuda(cudaStreamSynchronize(stream), "linear BLA build");
}

}  // namespace

// Mandelbrot hierarchies for one reference (build_bla, renderer.cpp:11612-11769).
void build_bla_on_device(ReferenceContext& ctx, int base_count) {
    ThreadRuntime& rt = thread_runtime();
    cudaStream_t stream = rt.stream;
    auto tables = std::make_shared<DeviceTables>();
    tables->device = rt.device;
    Scoped orbit;
    orbit.p = device_alloc<fx::Fec>(ctx.fast_orbit.size(), "cudaMalloc (builder orbit)");
    check_cuda(cudaMemcpy(orbit.p, ctx.fast_orbit.data(), ctx.fast_orbit.size() * sizeof(fx::Fec),
                          cudaMemcpyHostToDevice), "upload builder orbit");
    const fx::Fec* d_orbit = static_cast<const fx::Fec*>(orbit.p);
    // Cubic hierarchy up to 64 steps.
    const std::vector<int> sizes = level_sizes(base_count, kMaxSafeBlaLength, false);
    tables->cubic_index = index_of(sizes);
    tables->cubic = device_alloc<CubicStep>(static_cast<std::size_t>(total_of(sizes)), "cudaMalloc (cubic BLA)");
    {
        Scoped a, b;
        a.p = device_alloc<BuilderCubic>(static_cast<std::size_t>(base_count), "cudaMalloc (BLA builder)");
        b.p = device_alloc<BuilderCubic>(static_cast<std::size_t>(base_count / 2 + 1), "cudaMalloc (BLA builder)");
        BuilderCubic* prev = static_cast<BuilderCubic*>(a.p);
        BuilderCubic* cur = static_cast<BuilderCubic*>(b.p);
        cubic_base_kernel<<<blocks_for(base_count), kThreads, 0, stream>>>(d_orbit, base_count, prev, tables->cubic);
        for (std::size_t l = 1; l < sizes.size(); ++l) {
            cubic_merge_kernel<<<blocks_for(sizes[l]), kThreads, 0, stream>>>(
                prev, sizes[l], ctx.input_radius, cur, tables->cubic + tables->cubic_index.offset[l]);
            std::swap(prev, cur);
        }
        check_cuda(cudaGetLastError(), "cubic BLA build");
        check_cuda(cudaStreamSynchronize(stream), "cubic BLA build");
    }
    ctx.deep_input_radius = fx::fe_mul(ctx.input_radius, 1.0e-20);
    build_linear(d_orbit, base_count, ctx.input_radius, &tables->linear, tables->linear_index, stream);
    build_linear(d_orbit, base_count, ctx.deep_input_radius, &tables->deep_linear, tables->deep_linear_index, stream);
    ctx.device = tables;
    ctx.bla_on_device = true;
}

// Alternate-formula hierarchy (build_alternate_linear_bla, renderer.cpp:11414-11526).
void build_alt_bla_on_device(ReferenceContext& ctx, int first_index, int base_count) {
    ThreadRuntime& rt = thread_runtime();
    cudaStream_t stream = rt.stream;
    auto tables = std::make_shared<DeviceTables>();
    tables->device = rt.device;
    Scoped orbit;
    orbit.p = device_alloc<fx::Fec>(ctx.fast_orbit.size(), "cudaMalloc (builder orbit)");
    check_cuda(cudaMemcpy(orbit.p, ctx.fast_orbit.data(), ctx.fast_orbit.size() * sizeof(fx::Fec),
                          cudaMemcpyHostToDevice), "upload builder orbit");
    const std::vector<int> sizes = level_sizes(base_count, kMaxSafeLinearBlaLength, true);
    if (sizes.size() > static_cast<std::size_t>(kMaxLevels)) throw Failure{"too many BLA levels"};
    tables->alt_index = index_of(sizes);
    tables->alt = device_alloc<AltStep>(static_cast<std::size_t>(total_of(sizes)), "cudaMalloc (alternate BLA)");
    alt_base_kernel<<<blocks_for(base_count), kThreads, 0, stream>>>(static_cast<const fx::Fec*>(orbit.p), first_index,
                                                                      base_count, ctx.formula, tables->alt);
    for (std::size_t l = 1; l < sizes.size(); ++l) {
        alt_merge_kernel<<<blocks_for(sizes[l]), kThreads, 0, stream>>>(
            tables->alt + tables->alt_index.offset[l - 1], sizes[l - 1], sizes[l], ctx.alt_input_radius,
            tables->alt + tables->alt_index.offset[l]);
    }
    check_cuda(cudaGetLastError(), "alternate BLA build");
    check_cuda(cudaStreamSynchronize(stream), "alternate BLA build");
    ctx.device = tables;
    ctx.bla_on_device = true;
}

// Tier clone: copy the root's render tables and recompute only the radii for
// the new input radius (build_retargeted_bla, renderer.cpp:11803-11825).
void retarget_bla_on_device(ReferenceContext& ctx, const ReferenceContext& source) {
    const std::shared_ptr<DeviceTables> src = source.device;
    if (!src || !source.bla_on_device) throw Failure{"reference tier root has no device BLA tables"};
    ThreadRuntime& rt = thread_runtime();
    cudaStream_t stream = rt.stream;
    auto tables = std::make_shared<DeviceTables>();
    tables->device = src->device;
    auto copy_levels = [&](const auto* from, const LevelIndex& index, auto** to) {
        using T = std::remove_const_t<std::remove_pointer_t<decltype(from)>>;
        int total = 0;
        for (int l = 0; l < index.levels; ++l) total += index.count[l];
        *to = device_alloc<T>(static_cast<std::size_t>(total), "cudaMalloc (retargeted BLA)");
        if (total > 0) {
            check_cuda(cudaMemcpyAsync(*to, from, static_cast<std::size_t>(total) * sizeof(T), cudaMemcpyDeviceToDevice,
                                       stream), "copy BLA tables");
        }
    };
    copy_levels(src->cubic, src->cubic_index, &tables->cubic);
    tables->cubic_index = src->cubic_index;
    copy_levels(src->linear, src->linear_index, &tables->linear);
    tables->linear_index = src->linear_index;
    // The deep tier is retargeted from the root's normal linear levels.
    copy_levels(src->linear, src->linear_index, &tables->deep_linear);
    tables->deep_linear_index = src->linear_index;
    for (int l = 1; l < tables->cubic_index.levels; ++l) {
        const int n = tables->cubic_index.count[l];
        cubic_retarget_kernel<<<blocks_for(n), kThreads, 0, stream>>>(
            tables->cubic + tables->cubic_index.offset[l - 1], tables->cubic + tables->cubic_index.offset[l], n,
            ctx.input_radius);
    }
    ctx.deep_input_radius = fx::fe_mul(ctx.input_radius, 1.0e-20);
    const struct {
        LinearStep* table;
        const LevelIndex* index;
        fx::Fe radius;
    } linear_sets[2] = {{tables->linear, &tables->linear_index, ctx.input_radius},
                        {tables->deep_linear, &tables->deep_linear_index, ctx.deep_input_radius}};
    for (const auto& set : linear_sets) {
        for (int l = 1; l < set.index->levels; ++l) {
            const int n = set.index->count[l];
            linear_retarget_kernel<<<blocks_for(n), kThreads, 0, stream>>>(
                set.table + set.index->offset[l - 1], set.index->count[l - 1], set.table + set.index->offset[l], n,
                set.radius);
        }
    }
    check_cuda(cudaGetLastError(), "BLA retarget");
    check_cuda(cudaStreamSynchronize(stream), "BLA retarget");
    ctx.device = tables;
    ctx.bla_on_device = true;
}

// FP32 mirrors of device-resident compact tables.
void convert_fx_levels(DeviceTables& dev, cudaStream_t stream) {
    auto total = [](const LevelIndex& index) {
        int t = 0;
        for (int l = 0; l < index.levels; ++l) t += index.count[l];
        return t;
    };
    const int nc = total(dev.cubic_index);
    const int nl = total(dev.linear_index);
    const int nd = total(dev.deep_linear_index);
    const int na = total(dev.alt_index);
    dev.fx_cubic = device_alloc<FxCubic>(static_cast<std::size_t>(nc), "cudaMalloc (FP32 cubic BLA)");
    dev.fx_linear = device_alloc<FxLinear>(static_cast<std::size_t>(nl), "cudaMalloc (FP32 linear BLA)");
    dev.fx_deep_linear = device_alloc<FxLinear>(static_cast<std::size_t>(nd), "cudaMalloc (FP32 linear BLA)");
    if (nc) fx_cubic_kernel<<<blocks_for(nc), kThreads, 0, stream>>>(dev.cubic, dev.fx_cubic, nc);
    if (nl) fx_linear_kernel<<<blocks_for(nl), kThreads, 0, stream>>>(dev.linear, dev.fx_linear, nl);
    if (nd) fx_linear_kernel<<<blocks_for(nd), kThreads, 0, stream>>>(dev.deep_linear, dev.fx_deep_linear, nd);
    if (na) {
        dev.fx_alt = device_alloc<FxAltStep>(static_cast<std::size_t>(na), "cudaMalloc (FP32 alternate BLA)");
        fx_alt_kernel<<<blocks_for(na), kThreads, 0, stream>>>(dev.alt, dev.fx_alt, na);
    }
    check_cuda(cudaGetLastError(), "FP32 table conversion");
    check_cuda(cudaStreamSynchronize(stream), "FP32 table conversion");
}

}  // namespace fgb
