// Tensor-core level kernels: 32-feature epilogue units, F16 operands.
#include "level_bf16.cuh"

namespace mpl {
int launch_level_tc_u32_f16(const LevelArgs& a, cudaStream_t s) {
  return bf16::launch_unit<32, __half>(a, s);
}
}  // namespace mpl
