// Plain-form Mandelbrot kernel variant: planes=true, stats=true.
#include "render_plain.cuh"

namespace fgb {
template cudaError_t launch_plain_variant<true, true>(const PlainParams&, cudaStream_t);
}  // namespace fgb
