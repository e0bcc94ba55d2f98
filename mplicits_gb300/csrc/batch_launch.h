// Instantiations of the batched kernels (batch.cuh: one tile per CTA;
// batch_l0w.cuh: two tiles per CTA with first-layer warps), one translation
// unit per kernel family and operand type so that they compile in parallel.
#pragma once

#include "batch.cuh"
#include "batch_l0w.cuh"

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
int launch_p_u32_bf16(const Args& a, int WP, int ctas, cudaStream_t s);
int launch_p_u32_f16(const Args& a, int WP, int ctas, cudaStream_t s);

}  // namespace batch
}  // namespace mpl
