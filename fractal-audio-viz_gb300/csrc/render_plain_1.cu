// Plain-form Mandelbrot kernel variant: planes=true, stats=false.
#include "render_plain.cuh"

namespace fgb {
template cudaError_t launch_plain_variant<true, false>(const PlainParams&, cudaStream_t);
}  // namespace fgb
