// Dispatch to the plain-form Mandelbrot kernel variants (one per translation
// unit so the four instantiations compile in parallel).
#include "device.h"

namespace fgb {

template <bool Planes, bool Stats>
cudaError_t launch_plain_variant(const PlainParams& p, cudaStream_t stream);

cudaError_t launch_plain_mandelbrot(const PlainParams& p, bool planes, bool stats, cudaStream_t stream) {
    if (planes) {
        return stats ? launch_plain_variant<true, true>(p, stream) : launch_plain_variant<true, false>(p, stream);
    }
    return stats ? launch_plain_variant<false, true>(p, stream) : launch_plain_variant<false, false>(p, stream);
}

}  // namespace fgb
