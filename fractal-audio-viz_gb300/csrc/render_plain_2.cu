// Plain-form Mandelbrot kernel variant: planes=false, stats=true.
#include "render_plain.cuh"

namespace fgb {
template cudaError_t launch_plain_variant<false, true>(const PlainParams&, cudaStream_t);
}  // namespace fgb
