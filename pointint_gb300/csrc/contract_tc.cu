// Volume contraction on tcgen05 tensor cores (BF16 hi+lo split, FP32 accumulation).
#include <cuda_runtime.h>
#include "pi_internal.h"

namespace pi {

size_t contract_tc_ws_bytes(int64_t, int) { return 0; }

int launch_contract_tc(const pi_kgrid_impl*, const float2*, int, double*, void*, size_t, cudaStream_t) {
  return fail(PI_ERR_UNSUPPORTED, "tensor-core contraction not built yet");
}

}  // namespace pi
