// Reverse-mode input-gradient kernels (template in level_rgrad.cuh), BF16
// and FP16 operands, 16-feature epilogue units.
#include "level_rgrad.cuh"

namespace mpl {
int launch_level_rgrad(const LevelArgs& a, bool f16, cudaStream_t s) {
  return f16 ? rgrad::launch<__half>(a, s) : rgrad::launch<__nv_bfloat16>(a, s);
}
}  // namespace mpl
