// Reverse-mode input-gradient kernels with 32-feature epilogue units.
#include "level_rgrad.cuh"

namespace mpl {
int launch_level_rgrad_u32(const LevelArgs& a, bool f16, cudaStream_t s) {
  return f16 ? rgrad::launch<32, __half>(a, s) : rgrad::launch<32, __nv_bfloat16>(a, s);
}
}  // namespace mpl
