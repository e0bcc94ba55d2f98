// Per-ray pieces of the sphere tracer shared by the launch-per-level loop
// (trace.cu) and the persistent marching kernel (trace_march.cu), so both
// give every ray the same arithmetic.
#pragma once

#include "common.cuh"

namespace mpl {

// Appends `value` for the lanes with `keep` set (a full warp calls it).
__device__ __forceinline__ void warp_append(bool keep, int32_t value, int32_t* out,
                                            int32_t* count, int64_t capacity) {
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) {
    const int64_t pos = (int64_t)base + __popc(m & ((1u << lane) - 1u));
    if (pos < capacity) out[pos] = value;
  }
}

// One marching step with SDF value s of a ray at o moving along d
// (renderer/cuda/kernels.cu:315-398): |s| < eps is a hit (state 1);
// otherwise the ray advances by s along d, and a ray outside the bounding
// sphere moving outwards is a miss (state 2); on the last step of the budget
// a ray still marching stops (state 3).  Returns the new state (0: marching).
__device__ __forceinline__ int march_step(float s, float (&o)[3], const float (&d)[3], float eps,
                                          float R, bool last) {
  if (fabsf(s) < eps) return 1;
  float od = 0.f, oo = 0.f;
  for (int c = 0; c < 3; ++c) {
    o[c] = __fmaf_rn(d[c], s, o[c]);
    od = __fmaf_rn(o[c], d[c], od);
    oo = __fmaf_rn(o[c], o[c], oo);
  }
  if (oo > R * R && od > 0.0f) return 2;
  return last ? 3 : 0;  // 3: step budget exhausted
}

// march_step on ray r of the frame's arrays (position, direction, state);
// returns its new state.
__device__ __forceinline__ int march_ray(float s, int64_t r, float* __restrict__ org,
                                         const float* __restrict__ dir,
                                         int32_t* __restrict__ state, float eps, float R,
                                         bool last) {
  float o[3] = {org[3 * r + 0], org[3 * r + 1], org[3 * r + 2]};
  const float d[3] = {dir[3 * r + 0], dir[3 * r + 1], dir[3 * r + 2]};
  const int st = march_step(s, o, d, eps, R, last);
  if (st != 1)
    for (int c = 0; c < 3; ++c) org[3 * r + c] = o[c];
  if (st != 0) state[r] = st;
  return st;
}

}  // namespace mpl
