// Grid coordinates of gen_mc_coordinate_grid (i3d/meshing.py:11-69) written
// to memory.  The level kernels generate the same coordinates in registers;
// this entry point exists for callers that want the coordinate tensor itself.
#include "level.cuh"

namespace mpl {

__global__ void grid_points_kernel(MplPoints pts, const int32_t* __restrict__ index, int64_t n,
                                   float* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const int64_t p = index ? (int64_t)index[q] : q;
    float x, y, z;
    grid_point(p, pts.grid_n, pts.voxel_size, pts.offset[0], pts.offset[1], pts.offset[2], x,
               y, z);
    out[3 * q + 0] = x;
    out[3 * q + 1] = y;
    out[3 * q + 2] = z;
  }
}

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_grid_points(const MplPoints* pts, const int32_t* index, int64_t n, float* out,
                               void* stream) {
  if (!pts || !out || n < 0 || pts->kind != MPL_POINTS_GRID || pts->grid_n < 2)
    return MPL_ERR_INVALID_ARG;
  if (n == 0) return MPL_OK;
  int64_t blocks = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  grid_points_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(*pts, index, n, out);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
