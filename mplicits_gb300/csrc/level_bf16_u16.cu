// BF16 level kernels with 16-feature epilogue units (16 epilogue warps).
#include "level_bf16.cuh"

namespace mpl {
int launch_level_bf16_u16(const LevelArgs& a, cudaStream_t s) { return bf16::launch_unit<16>(a, s); }
}  // namespace mpl
