// BF16 tcgen05 level evaluator (placeholder until the tensor-core kernel lands).
#include "level.cuh"

namespace mpl {

int launch_level_bf16(const LevelArgs& a, cudaStream_t s) {
  (void)a;
  (void)s;
  return MPL_ERR_UNSUPPORTED;
}

}  // namespace mpl
