// Band compaction, i3d/meshing.py:222-231 (`idx = |sdf_base| < delta`
// followed by the boolean gather `sample_subset[idx]`): a warp-ballot
// stream compaction of the points of a delta-band into an index list.
// HBM-bound: 4 B read per candidate, 4 B written per kept point.
#include "level.cuh"

namespace mpl {

__global__ void band_compact_kernel(const float* __restrict__ S, const int32_t* __restrict__ index,
                                    const int32_t* __restrict__ n_dev, int64_t n, float delta,
                                    float lower,
                                    int32_t* __restrict__ out, int32_t* __restrict__ count,
                                    int64_t capacity) {
  if (n_dev) {
    const int64_t m = *n_dev;
    n = m < n ? m : n;
  }
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // every lane of a warp runs the same number of iterations (ballot safety)
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) - lane;
  for (int64_t base = warp0; base < n; base += stride) {
    const int64_t q = base + lane;
    bool keep = false;
    int64_t p = 0;
    if (q < n) {
      p = index ? (int64_t)index[q] : q;
      const float v = fabsf(S[p]);
      keep = v < delta && v >= lower;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int b = 0;
    if (lane == 0 && m) b = atomicAdd(count, __popc(m));
    b = __shfl_sync(0xffffffffu, b, 0);
    if (keep) {
      const int64_t pos = (int64_t)b + __popc(m & ((1u << lane) - 1u));
      if (pos < capacity) out[pos] = (int32_t)p;
    }
  }
}

// max_j |S_j| as float bits: for non-negative floats the unsigned order of
// the bits is the numeric order, and a NaN's bits (0x7fc00000 and up) lie
// above +inf's, so one NaN makes the result NaN, as torch's max does.
__global__ void abs_max_kernel(const float* __restrict__ S, int64_t n,
                               unsigned int* __restrict__ out) {
  unsigned int m = 0u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned int v = __float_as_uint(S[i]) & 0x7fffffffu;
    m = v > m ? v : m;
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_abs_max(const float* S, int64_t n, float* out, void* stream) {
  if (!out || n < 0 || (n > 0 && !S)) return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float), s));
  if (n == 0) return MPL_OK;
  const int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  abs_max_kernel<<<(unsigned)blocks, threads, 0, s>>>(S, n, reinterpret_cast<unsigned int*>(out));
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_band_compact(const float* S, const int32_t* index, const int32_t* n_dev,
                                int64_t n, const MplBand* band, void* stream) {
  if (!S || !band || !band->out_index || !band->count_dev || n < 0 || n > INT32_MAX)
    return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(band->count_dev, 0, sizeof(int32_t), s));
  if (n == 0) return MPL_OK;
  const int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  band_compact_kernel<<<(unsigned)blocks, threads, 0, s>>>(S, index, n_dev, n, band->delta,
                                                           band->lower, band->out_index,
                                                           band->count_dev,
                                                           band->capacity);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
