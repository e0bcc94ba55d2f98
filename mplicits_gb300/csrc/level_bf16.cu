// Dispatch of the tensor-core level kernels (templates in level_bf16.cuh,
// level_pp.cuh and level_rgrad.cuh): operand type by precision (BF16 or
// FP16), epilogue unit width by MPL_OPT_BF16_EPILOGUE_UNIT, one or two tiles
// in flight per CTA by MPL_OPT_TC_TILES_IN_FLIGHT, the first layer in warps of
// its own or in the drains by MPL_OPT_TC_LAYER0_WARPS, and for the input gradient
// the reverse-mode kernel (MPL_OPT_TC_GRAD_REVERSE, levels with one or two
// hidden GEMMs) or the forward-mode tangent rows of the level kernels.
#include "level.cuh"

namespace mpl {

int launch_level_tc_u16_bf16(const LevelArgs& a, cudaStream_t s);
int launch_level_tc_u32_bf16(const LevelArgs& a, cudaStream_t s);
int launch_level_tc_u16_f16(const LevelArgs& a, cudaStream_t s);
int launch_level_tc_u32_f16(const LevelArgs& a, cudaStream_t s);
int launch_level_pp_u16_bf16(const LevelArgs& a, cudaStream_t s);
int launch_level_pp_u32_bf16(const LevelArgs& a, cudaStream_t s);
int launch_level_pp_u16_f16(const LevelArgs& a, cudaStream_t s);
int launch_level_pp_u32_f16(const LevelArgs& a, cudaStream_t s);
int launch_level_l0w_u16_bf16(const LevelArgs& a, int layer0_warps, cudaStream_t s);
int launch_level_l0w_u32_bf16(const LevelArgs& a, int layer0_warps, cudaStream_t s);
int launch_level_l0w_u16_f16(const LevelArgs& a, int layer0_warps, cudaStream_t s);
int launch_level_l0w_u32_f16(const LevelArgs& a, int layer0_warps, cudaStream_t s);
int launch_level_rgrad(const LevelArgs& a, bool f16, cudaStream_t s);

int launch_level_tc(const LevelArgs& a, bool f16, cudaStream_t s) {
  if (a.lay.nh == 0) return launch_level_fp32(a, s);  // no hidden GEMM for the tensor cores
  if (a.grad && option_value(MPL_OPT_TC_GRAD_REVERSE) == 1) {
    const int st = launch_level_rgrad(a, f16, s);
    if (st != MPL_ERR_UNSUPPORTED) return st;
  }
  const bool u32 = option_value(MPL_OPT_BF16_EPILOGUE_UNIT) == 32;
  if (option_value(MPL_OPT_TC_TILES_IN_FLIGHT) == 2) {
    // two tiles per CTA where the level's constants fit next to two A tiles,
    // with the first layer in warps of its own or in the epilogue's drains
    int st;
    const int nl = (int)option_value(MPL_OPT_TC_LAYER0_WARPS);
    if (nl == 4 || nl == 8) {
      if (f16) st = u32 ? launch_level_l0w_u32_f16(a, nl, s) : launch_level_l0w_u16_f16(a, nl, s);
      else st = u32 ? launch_level_l0w_u32_bf16(a, nl, s) : launch_level_l0w_u16_bf16(a, nl, s);
    } else {
      if (f16) st = u32 ? launch_level_pp_u32_f16(a, s) : launch_level_pp_u16_f16(a, s);
      else st = u32 ? launch_level_pp_u32_bf16(a, s) : launch_level_pp_u16_bf16(a, s);
    }
    if (st != MPL_ERR_UNSUPPORTED) return st;
  }
  if (f16) return u32 ? launch_level_tc_u32_f16(a, s) : launch_level_tc_u16_f16(a, s);
  return u32 ? launch_level_tc_u32_bf16(a, s) : launch_level_tc_u16_bf16(a, s);
}

int launch_level_bf16(const LevelArgs& a, cudaStream_t s) { return launch_level_tc(a, false, s); }

int launch_level_f16(const LevelArgs& a, cudaStream_t s) { return launch_level_tc(a, true, s); }

}  // namespace mpl
