// Two-tile tensor-core level kernels with first-layer warps (4 or 8):
// 32-feature epilogue units, FP16 operands.
#include "level_l0w.cuh"

namespace mpl {
int launch_level_l0w_u32_f16(const LevelArgs& a, int layer0_warps, cudaStream_t s) {
  return layer0_warps == 8 ? l0w::launch_unit<32, 8, __half>(a, s)
                           : l0w::launch_unit<32, 4, __half>(a, s);
}
}  // namespace mpl
