// Floatexp form (FP32 mantissa / int32 exponent deltas).
#include "device.h"
#include "fractal_gb300.h"
#include "runtime.h"

namespace fgb {

void render_floatexp_from_reference(ReferenceContext&, const Outputs&, int, int, const char*, int, int, int,
                                    const FractalRenderOptions&, ThreadRuntime&, cudaStream_t) {
    throw Failure{"floatexp form is not available yet"};
}

}  // namespace fgb
