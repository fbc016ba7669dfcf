// Plain form for julia / burning-ship / tricorn.
#include "device.h"

namespace fgb {

cudaError_t launch_plain_alternate(const AltParams&, bool, bool, cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace fgb
