// Batched kernel instantiations, FP16 operands.
#include "batch_launch.h"

namespace mpl {
namespace batch {
int launch_u16_s2_f16(const Args& a, int c, cudaStream_t s) { return launch<2, 16, __half>(a, c, s); }
int launch_u16_s3_f16(const Args& a, int c, cudaStream_t s) { return launch<3, 16, __half>(a, c, s); }
int launch_u32_s2_f16(const Args& a, int c, cudaStream_t s) { return launch<2, 32, __half>(a, c, s); }
int launch_u32_s3_f16(const Args& a, int c, cudaStream_t s) { return launch<3, 32, __half>(a, c, s); }
}  // namespace batch
}  // namespace mpl
