// Two-tile tensor-core level kernels: 32-feature epilogue units, FP16 operands.
#include "level_pp.cuh"

namespace mpl {
int launch_level_pp_u32_f16(const LevelArgs& a, cudaStream_t s) {
  return pp::launch_unit<32, __half>(a, s);
}
}  // namespace mpl
