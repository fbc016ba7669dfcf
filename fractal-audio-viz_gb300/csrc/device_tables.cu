// Upload of one reference's tables to HBM, once per handle generation.
//
// A handle's tables are immutable after creation, so the device copy is made
// on the first render that needs it and shared by every later render of the
// same handle (the reference keys its OpenCL cache on the generation the
// same way, renderer.cpp:9077-9245).
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "runtime.h"

namespace fgb {

DeviceTables::~DeviceTables() {
    // Freed on the owning device; errors at process teardown are ignored.
    int current = -1;
    cudaGetDevice(&current);
    if (device >= 0 && current != device) cudaSetDevice(device);
    cudaFree(orbit);
    cudaFree(cubic);
    cudaFree(linear);
    cudaFree(deep_linear);
    cudaFree(alt);
    cudaFree(series);
    cudaFree(fx_orbit);
    cudaFree(fx_cubic);
    cudaFree(fx_linear);
    cudaFree(fx_deep_linear);
    cudaFree(fx_alt);
    cudaFree(fx_series);
    cudaFree(fx_index);
    if (device >= 0 && current >= 0 && current != device) cudaSetDevice(current);
}

namespace {

template <typename T>
T* upload(const std::vector<T>& host) {
    if (host.empty()) return nullptr;
    T* device = nullptr;
    check_cuda(cudaMalloc(&device, host.size() * sizeof(T)), "cudaMalloc (reference tables)");
    check_cuda(cudaMemcpy(device, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice),
               "cudaMemcpy (reference tables)");
    return device;
}

template <typename T>
T* upload_levels(const std::vector<std::vector<T>>& levels, LevelIndex& index) {
    if (levels.size() > static_cast<std::size_t>(kMaxLevels)) {
        throw Failure{"BLA hierarchy has more levels than the device index holds"};
    }
    std::vector<T> flat;
    index = LevelIndex{};
    index.levels = static_cast<int>(levels.size());
    for (std::size_t level = 0; level < levels.size(); ++level) {
        index.offset[level] = static_cast<int>(flat.size());
        index.count[level] = static_cast<int>(levels[level].size());
        flat.insert(flat.end(), levels[level].begin(), levels[level].end());
    }
    return upload(flat);
}

f32x::F2e to_f2e(const fx::Sc& v) {
    if (v.re == 0.0 && v.im == 0.0) return f32x::zero();
    return f32x::norm(static_cast<float>(v.re), static_cast<float>(v.im), v.e);
}

f32x::N1e to_n1e(const fx::Fe& v) {
    if (v.m == 0.0 || !fx::fe_finite(v)) {
        f32x::N1e r;
        r.m = fx::fe_finite(v) ? 0.0f : 3.0e38f;
        r.e = fx::fe_finite(v) ? 0 : 0x3fffffff;
        return r;
    }
    return f32x::n_norm(static_cast<float>(v.m), v.e);
}

f32x::R1e to_r1e(const fx::Fe& v) {
    if (!fx::fe_finite(v)) return f32x::r_make(v.m < 0.0 ? -3.0e38f : 3.0e38f, 0x3fffffff);
    return f32x::r_norm(static_cast<float>(v.m), v.e);
}

float plain_float(double mantissa, int exponent) {
    const double v = fx::scale2(mantissa, exponent);
    const double a = v < 0 ? -v : v;
    if (!(a < 3.0e38)) return v < 0 ? -3.0e38f : 3.0e38f;
    if (a < 1.0e-37) return 0.0f;
    return static_cast<float>(v);
}

}  // namespace

void convert_fx_levels(DeviceTables& dev, cudaStream_t stream);

// FP32 mirrors of the tables for the floatexp form, made once per handle.
void floatexp_tables(ReferenceContext& ctx, DeviceTables& dev) {
    std::lock_guard<std::mutex> lock(ctx.device_mutex);
    if (dev.fx_ready) return;
    const OrbitData& orbit = *ctx.orbit;
    std::vector<FxOrbitRec> records(orbit.scaled.size());
    for (std::size_t i = 0; i < records.size(); ++i) {
        const fx::Sc& z = orbit.scaled[i];
        FxOrbitRec& r = records[i];
        std::memset(&r, 0, sizeof r);
        r.zr = plain_float(z.re, z.e);
        r.zi = plain_float(z.im, z.e);
        r.z = to_f2e(z);
        if (ctx.formula == kFormulaMandelbrot) {
            const fx::Nrm n = fx::sc_norm2(z);
            r.z2 = to_n1e(fx::fe_make(n.m, n.e));
        } else {
            r.z2 = f32x::n_from_r(to_r1e(i < orbit.escape_margin.size() ? orbit.escape_margin[i] : fx::Fe{0.0, 0}));
        }
    }
    dev.fx_orbit = upload(records);
    auto cubic_levels = [&](const std::vector<std::vector<CubicStep>>& levels) {
        std::vector<std::vector<FxCubic>> out;
        for (const auto& level : levels) {
            auto& dst = out.emplace_back();
            for (const CubicStep& s : level) {
                FxCubic c{};
                for (int k = 0; k < 9; ++k) c.c[k] = to_f2e(s.c[k]);
                c.r2 = to_n1e(s.r2);
                c.len = s.len;
                dst.push_back(c);
            }
        }
        return out;
    };
    auto linear_levels = [&](const std::vector<std::vector<LinearStep>>& levels) {
        std::vector<std::vector<FxLinear>> out;
        for (const auto& level : levels) {
            auto& dst = out.emplace_back();
            for (const LinearStep& s : level) {
                FxLinear l{};
                l.a = to_f2e(s.a);
                l.b = to_f2e(s.b);
                l.r2 = to_n1e(s.r2);
                l.len = s.len;
                dst.push_back(l);
            }
        }
        return out;
    };
    auto alt_levels = [&](const std::vector<std::vector<AltStep>>& levels) {
        std::vector<std::vector<FxAltStep>> out;
        for (const auto& level : levels) {
            auto& dst = out.emplace_back();
            for (const AltStep& s : level) {
                FxAltStep a{};
                for (int k = 0; k < 8; ++k) a.c[k] = to_r1e(s.c[k]);
                a.r2 = to_n1e(s.r2);
                a.len = s.len;
                dst.push_back(a);
            }
        }
        return out;
    };
    if (ctx.bla_on_device) {
        convert_fx_levels(dev, thread_runtime().stream);
    } else {
        LevelIndex unused;
        dev.fx_cubic = upload_levels(cubic_levels(ctx.cubic), unused);
        dev.fx_linear = upload_levels(linear_levels(ctx.linear), unused);
        dev.fx_deep_linear = upload_levels(linear_levels(ctx.deep_linear), unused);
        dev.fx_alt = upload_levels(alt_levels(ctx.alt), unused);
    }
    const std::vector<LevelIndex> indexes = {dev.cubic_index, dev.linear_index, dev.deep_linear_index,
                                             dev.alt_index};
    dev.fx_index = upload(indexes);
    std::vector<f32x::F2e> series;
    for (const fx::Sc& c : ctx.series.coeff) series.push_back(to_f2e(c));
    dev.fx_series = upload(series);
    dev.fx_ready = true;
}

std::shared_ptr<DeviceTables> device_tables(ReferenceContext& ctx) {
    const int device = current_device();
    std::lock_guard<std::mutex> lock(ctx.device_mutex);
    if (ctx.device && ctx.device->device != device) {
        if (ctx.bla_on_device) throw Failure{"reference tables were built on another CUDA device"};
        ctx.device.reset();
    }
    if (!ctx.device) ctx.device = std::make_shared<DeviceTables>();
    DeviceTables& t = *ctx.device;
    t.device = device;
    if (t.orbit == nullptr) {
        const std::vector<OrbitRec> records = make_orbit_records(ctx);
        t.orbit = upload(records);
        t.orbit_size = static_cast<int>(records.size());
        t.series = upload(ctx.series.coeff);
        t.series_terms = static_cast<int>(ctx.series.coeff.size());
        if (!ctx.bla_on_device) {
            t.cubic = upload_levels(ctx.cubic, t.cubic_index);
            t.linear = upload_levels(ctx.linear, t.linear_index);
            t.deep_linear = upload_levels(ctx.deep_linear, t.deep_linear_index);
            t.alt = upload_levels(ctx.alt, t.alt_index);
        }
    }
    return ctx.device;
}

}  // namespace fgb
