// Two-tile batched kernel instantiations, FP16 operands.
#include "batch_launch.h"

namespace mpl {
namespace batch {
int launch_p_u32_f16(const Args& a, int WP, int c, cudaStream_t s) { return launch_l0w<32, 8, __half>(a, WP, c, s); }
}  // namespace batch
}  // namespace mpl
