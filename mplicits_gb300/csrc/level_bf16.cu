// Dispatch of the BF16 tcgen05 level kernels (kernel template in
// level_bf16.cuh): the epilogue unit width is a tuning option.
#include "level.cuh"

namespace mpl {

int launch_level_bf16_u16(const LevelArgs& a, cudaStream_t s);
int launch_level_bf16_u32(const LevelArgs& a, cudaStream_t s);

int launch_level_bf16(const LevelArgs& a, cudaStream_t s) {
  if (a.lay.nh == 0) return launch_level_fp32(a, s);  // no hidden GEMM to run in BF16
  return option_value(MPL_OPT_BF16_EPILOGUE_UNIT) == 32 ? launch_level_bf16_u32(a, s)
                                                        : launch_level_bf16_u16(a, s);
}

}  // namespace mpl
