// Arguments shared by the level-evaluation kernels.
#pragma once

#include "common.cuh"

namespace mpl {

struct LevelArgs {
  const char* packed;
  PackLayout lay;
  float omega[MPL_MAX_LAYERS];
  MplPoints pts;
  const int32_t* index;  // nullable
  const int32_t* n_dev;  // nullable
  int64_t n;
  float* S;
  int32_t store_mode;
  int32_t has_band;
  float band_delta;
  float band_lower;
  int32_t* band_out;
  int32_t* band_count;
  int64_t band_capacity;
  int* status;  // device status word
  int32_t grad;  // also compute df/dx (forward mode) into G
  float* G;      // [*, 3] gradients, indexed like S (nullable in grad mode)
  // training: pre-activations a_l of every layer and row, FP32 plain GRAD
  // kernel only: pre[((l * n + q) * 4 + row) * WP + j] (row 0 value with bias,
  // rows 1..3 the tangents d/dx, d/dy, d/dz without bias)
  float* pre;
};

__device__ __forceinline__ int64_t level_point_count(const LevelArgs& a) {
  int64_t n = a.n;
  if (a.n_dev) {
    int64_t m = (int64_t)(*a.n_dev);
    n = m < n ? m : n;
  }
  return n < 0 ? 0 : n;
}

// Coordinates of point p (grid index or row of the point list).
__device__ __forceinline__ void point_coords(const LevelArgs& a, int64_t p, float& x, float& y,
                                             float& z) {
  if (a.pts.kind == MPL_POINTS_GRID) {
    grid_point(p, a.pts.grid_n, a.pts.voxel_size, a.pts.offset[0], a.pts.offset[1],
               a.pts.offset[2], x, y, z);
  } else {
    x = a.pts.xyz[3 * p + 0];
    y = a.pts.xyz[3 * p + 1];
    z = a.pts.xyz[3 * p + 2];
  }
}

__device__ __forceinline__ void load_point(const LevelArgs& a, int64_t q, int64_t& p, float& x,
                                           float& y, float& z) {
  p = a.index ? (int64_t)a.index[q] : q;
  point_coords(a, p, x, y, z);
}

// Stores f into S[p] (or adds it) and appends p to the band list when
// |S[p]| < delta.  Called by every lane of a full warp; `valid` masks lanes
// without a point.
__device__ __forceinline__ void store_and_band(const LevelArgs& a, bool valid, int64_t p,
                                               float f);

// As store_and_band, with the value S[p] held before this level already read
// (MPL_ACCUMULATE; ignored in MPL_STORE), so that its load can be issued early.
__device__ __forceinline__ void store_and_band_old(const LevelArgs& a, bool valid, int64_t p,
                                                   float f, float old) {
  float s = f;
  if (valid) {
    if (a.store_mode == MPL_ACCUMULATE) s = __fadd_rn(old, f);
    a.S[p] = s;
  }
  if (a.has_band) {
    const bool keep = valid && fabsf(s) < a.band_delta && fabsf(s) >= a.band_lower;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(a.band_count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) {
      const int64_t pos = (int64_t)base + __popc(m & ((1u << lane) - 1u));
      if (pos < a.band_capacity) a.band_out[pos] = (int32_t)p;
    }
  }
}

__device__ __forceinline__ void store_and_band(const LevelArgs& a, bool valid, int64_t p,
                                               float f) {
  float s = f;
  if (valid) {
    if (a.store_mode == MPL_ACCUMULATE) s = __fadd_rn(a.S[p], f);
    a.S[p] = s;
  }
  if (a.has_band) {
    const bool keep = valid && fabsf(s) < a.band_delta && fabsf(s) >= a.band_lower;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(a.band_count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) {
      const int64_t pos = (int64_t)base + __popc(m & ((1u << lane) - 1u));
      if (pos < a.band_capacity) a.band_out[pos] = (int32_t)p;
    }
  }
}

int launch_level_fp32(const LevelArgs& a, cudaStream_t s);
int launch_level_bf16(const LevelArgs& a, cudaStream_t s);
int launch_level_f16(const LevelArgs& a, cudaStream_t s);

}  // namespace mpl
