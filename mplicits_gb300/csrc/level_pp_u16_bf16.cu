// Two-tile tensor-core level kernels: 16-feature epilogue units, BF16 operands.
#include "level_pp.cuh"

namespace mpl {
int launch_level_pp_u16_bf16(const LevelArgs& a, cudaStream_t s) {
  return pp::launch_unit<16, __nv_bfloat16>(a, s);
}
}  // namespace mpl
