// Two-tile tensor-core level kernels: 16-feature epilogue units, FP16 operands.
#include "level_pp.cuh"

namespace mpl {
int launch_level_pp_u16_f16(const LevelArgs& a, cudaStream_t s) {
  return pp::launch_unit<16, __half>(a, s);
}
}  // namespace mpl
