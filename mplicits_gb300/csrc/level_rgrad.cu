// Reverse-mode input-gradient kernels (template in level_rgrad.cuh), BF16
// and FP16 operands, 16-feature epilogue units (32-feature units in
// level_rgrad_u32.cu); the unit follows MPL_OPT_BF16_EPILOGUE_UNIT, as the
// forward kernels' does.
#include "level_rgrad.cuh"

namespace mpl {
int launch_level_rgrad_u32(const LevelArgs& a, bool f16, cudaStream_t s);

int launch_level_rgrad(const LevelArgs& a, bool f16, cudaStream_t s) {
  if (option_value(MPL_OPT_BF16_EPILOGUE_UNIT) == 32) return launch_level_rgrad_u32(a, f16, s);
  return f16 ? rgrad::launch<16, __half>(a, s) : rgrad::launch<16, __nv_bfloat16>(a, s);
}
}  // namespace mpl
