// march_tc.cu -- FP16 tensor-core march (tcgen05 MLP).  Placeholder until
// the tensor-core kernel lands: the launcher reports "not supported" so a
// context created with NES_PREC_FP16_TC fails loudly instead of silently
// falling back to another path.
#include "kernels.h"

namespace nes {

size_t tc_weight_bytes() { return 16; }
void pack_tc_weights(const float*, uint8_t* out) {
  for (int i = 0; i < 16; ++i) out[i] = 0;
}

cudaError_t launch_march_tc(const ViewBatch&, const DevScene&, const DevScratch&, int, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace nes
