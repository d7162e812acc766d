// Split-precision tensor-core engine (placeholder until the tcgen05 path lands).
#include "kernels.h"

namespace ctr {

int twosided_split(int, int, int, int, const double*, const double*, int, const std::vector<TwoSidedRow>&,
                   const std::vector<float>&, const std::vector<int32_t>&, int, double*, cudaStream_t) {
  return fail(CTR_ERR_UNSUPPORTED, "split-precision engine not built yet");
}

}  // namespace ctr

extern "C" int ctr_split_available(void) { return 0; }
