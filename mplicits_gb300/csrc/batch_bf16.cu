// Batched kernel instantiations, BF16 operands.
#include "batch_launch.h"

namespace mpl {
namespace batch {
int launch_u16_s2_bf16(const Args& a, int c, cudaStream_t s) { return launch<2, 16, __nv_bfloat16>(a, c, s); }
int launch_u16_s3_bf16(const Args& a, int c, cudaStream_t s) { return launch<3, 16, __nv_bfloat16>(a, c, s); }
int launch_u32_s2_bf16(const Args& a, int c, cudaStream_t s) { return launch<2, 32, __nv_bfloat16>(a, c, s); }
int launch_u32_s3_bf16(const Args& a, int c, cudaStream_t s) { return launch<3, 32, __nv_bfloat16>(a, c, s); }
}  // namespace batch
}  // namespace mpl
