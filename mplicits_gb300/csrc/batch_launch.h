// Instantiations of the batched kernel (batch.cuh), one translation unit per
// operand type so that they compile in parallel.
#pragma once

#include "batch.cuh"

namespace mpl {
namespace batch {

int launch_u16_s2_bf16(const Args& a, int ctas, cudaStream_t s);
int launch_u16_s3_bf16(const Args& a, int ctas, cudaStream_t s);
int launch_u32_s2_bf16(const Args& a, int ctas, cudaStream_t s);
int launch_u32_s3_bf16(const Args& a, int ctas, cudaStream_t s);
int launch_u16_s2_f16(const Args& a, int ctas, cudaStream_t s);
int launch_u16_s3_f16(const Args& a, int ctas, cudaStream_t s);
int launch_u32_s2_f16(const Args& a, int ctas, cudaStream_t s);
int launch_u32_s3_f16(const Args& a, int ctas, cudaStream_t s);

}  // namespace batch
}  // namespace mpl
