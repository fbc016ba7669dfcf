// Plain-form Mandelbrot kernel variant: planes=false, stats=false.
#include "render_plain.cuh"

namespace fgb {
template cudaError_t launch_plain_variant<false, false>(const PlainParams&, cudaStream_t);
}  // namespace fgb
