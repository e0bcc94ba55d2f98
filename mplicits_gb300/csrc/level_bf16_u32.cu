// BF16 level kernels with 32-feature epilogue units (8 epilogue warps).
#include "level_bf16.cuh"

namespace mpl {
int launch_level_bf16_u32(const LevelArgs& a, cudaStream_t s) { return bf16::launch_unit<32>(a, s); }
}  // namespace mpl
