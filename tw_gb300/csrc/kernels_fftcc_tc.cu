// Tensor-core FFT-CC (tcgen05 DFT GEMMs).  Placeholder until implemented:
// reports unsupported so the engine uses the FP32 SIMT DFT kernel.
#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

bool fftcc_tc_supported(const Geom&) { return false; }

cudaError_t launch_fftcc_tc(const Geom&, const uint8_t*, const uint8_t*, const int2*, int, float*, float*, float*,
                            uint8_t*, unsigned*, cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace twdic
