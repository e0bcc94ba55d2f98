// Multiscale sphere tracing: ray generation, the per-step update with
// active-ray compaction, and headless shading.  Restates the reference
// renderer's InitializeRays_kernel (renderer/cuda/kernels.cu:400-487),
// IterateSphereTracing_kernel (kernels.cu:315-398) and Shade_kernel
// (kernels.cu:122-275) without its OpenGL window and pixel buffer.  The
// level evaluations between steps are mpl_level_forward launches on the
// active-ray list (with band gating through their fused band lists), so a
// step only touches rays still marching and the finer levels only rays
// inside their bands (the reference evaluates every level for every pixel).
#include "level.cuh"
#include "trace.cuh"

namespace mpl {

namespace {

struct Basis {
  float eye[3], s[3], u[3], f[3];
  float tx, ty;  // tan(fov/2) * aspect, tan(fov/2)
};

// Pixel (i, j): NDC x = 2i/W - 1, y = 1 - 2j/H (row 0 at the top), the
// eye-space direction (x tan(fov/2) aspect, y tan(fov/2), -1) rotated by the
// look-at basis; the origin moves to the bounding sphere of radius R when
// the eye is outside it (kernels.cu:454-477).  Rays that miss the sphere
// are marked missed right away.
__global__ void trace_init_kernel(Basis b, int W, int H, float R, float* __restrict__ org,
                                  float* __restrict__ dir, int32_t* __restrict__ state,
                                  int32_t* __restrict__ active, int32_t* __restrict__ count) {
  const int64_t P = (int64_t)W * H;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~int64_t(31);
  for (int64_t base = warp0; base < P; base += stride) {
    const int64_t r = base + (threadIdx.x & 31);
    bool keep = false;
    if (r < P) {
      const int i = (int)(r % W), j = (int)(r / W);
      const float nx = 2.0f * (float)i / (float)W - 1.0f;
      const float ny = 1.0f - 2.0f * (float)j / (float)H;
      const float ex = nx * b.tx, ey = ny * b.ty;
      float d[3];
      for (int c = 0; c < 3; ++c) d[c] = b.s[c] * ex + b.u[c] * ey + b.f[c];
      const float inv = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      for (int c = 0; c < 3; ++c) d[c] *= inv;
      float o[3] = {b.eye[0], b.eye[1], b.eye[2]};
      const float bb = o[0] * d[0] + o[1] * d[1] + o[2] * d[2];
      const float cc = o[0] * o[0] + o[1] * o[1] + o[2] * o[2] - R * R;
      bool hits_sphere = true;
      if (cc > 0.0f) {
        const float disc = bb * bb - cc;
        if (bb < 0.0f && disc > 0.0f) {
          const float t = -bb - sqrtf(disc);
          for (int c = 0; c < 3; ++c) o[c] += t * d[c];
        } else {
          hits_sphere = false;
        }
      }
      for (int c = 0; c < 3; ++c) {
        org[3 * r + c] = o[c];
        dir[3 * r + c] = d[c];
      }
      state[r] = hits_sphere ? 0 : 2;
      keep = hits_sphere;
    }
    warp_append(keep, (int32_t)r, active, count, P);
  }
}

// One marching step for the active rays: |S| < eps is a hit; otherwise the
// ray advances by S along its direction (kernels.cu:315-398 with the sum of
// the levels evaluated for that ray), and a ray that leaves the bounding
// sphere moving outwards is a miss.  Still-active rays go to active_out,
// hits to hit_out.
__global__ void trace_step_kernel(const float* __restrict__ S, const int32_t* __restrict__ active,
                                  const int32_t* __restrict__ count, int64_t cap_in,
                                  float* __restrict__ org, const float* __restrict__ dir,
                                  int32_t* __restrict__ state, float eps, float R, int32_t last,
                                  int32_t* __restrict__ active_out, int32_t* __restrict__ count_out,
                                  int32_t* __restrict__ hit_out, int32_t* __restrict__ hit_count,
                                  int64_t capacity) {
  int64_t n = *count;
  n = n < cap_in ? n : cap_in;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~int64_t(31);
  for (int64_t base = warp0; base < n; base += stride) {
    const int64_t q = base + (threadIdx.x & 31);
    bool keep = false, hit = false;
    int32_t r = 0;
    if (q < n) {
      r = active[q];
      const int st = march_ray(S[r], r, org, dir, state, eps, R, last != 0);
      hit = st == 1;
      keep = st == 0;
    }
    warp_append(keep, r, active_out, count_out, capacity);
    warp_append(hit, r, hit_out, hit_count, capacity);
  }
}

// Phong shading of the hits (kernels.cu:191-268): light along the view
// direction, ka 1 x ambient 0.2, kd 1 x diffuse 0.54, ks 0.5 x specular 1,
// shininess 35; misses are white.  Pixels: RGBA8 packed little-endian.
__global__ void trace_shade_kernel(const float* __restrict__ org, const float* __restrict__ dir,
                                   const float* __restrict__ G, const int32_t* __restrict__ state,
                                   int64_t P, int32_t mode, uint32_t* __restrict__ image) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P) return;
  auto pack = [](float cr, float cg, float cb) {
    auto q = [](float v) { return (uint32_t)(fminf(fmaxf(v, 0.f), 1.f) * 255.0f); };
    return (255u << 24) | (q(cb) << 16) | (q(cg) << 8) | q(cr);
  };
  const bool inside = fabsf(org[3 * r]) < 1.f && fabsf(org[3 * r + 1]) < 1.f &&
                      fabsf(org[3 * r + 2]) < 1.f;
  if (state[r] != 1 || !inside) {
    image[r] = pack(1.f, 1.f, 1.f);
    return;
  }
  float n[3] = {G[3 * r], G[3 * r + 1], G[3 * r + 2]};
  const float len = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const float il = len > 0.f ? 1.f / len : 0.f;
  for (int c = 0; c < 3; ++c) n[c] *= il;
  if (mode == 0) {  // normal display
    image[r] = pack(fabsf(n[0]), fabsf(n[2]), fabsf(n[1]));
    return;
  }
  float l[3] = {-dir[3 * r], -dir[3 * r + 1], -dir[3 * r + 2]};
  const float nl = l[0] * n[0] + l[1] * n[1] + l[2] * n[2];
  float refl[3];
  for (int c = 0; c < 3; ++c) refl[c] = 2.f * nl * n[c] - l[c];
  const float diff = fmaxf(nl, 0.f);
  const float rv = l[0] * refl[0] + l[1] * refl[1] + l[2] * refl[2];
  const float spec = fmaxf(powf(fmaxf(rv, 0.f), 35.f), 0.f);
  const float c = 0.2f + 1.f * diff * 0.54f + 0.5f * spec;
  image[r] = pack(c, c, c);
}

Basis make_basis(const MplCamera& cam) {
  Basis b;
  float f[3], s[3], u[3];
  for (int c = 0; c < 3; ++c) f[c] = cam.target[c] - cam.eye[c];
  float fl = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (int c = 0; c < 3; ++c) f[c] /= fl;
  s[0] = f[1] * cam.up[2] - f[2] * cam.up[1];
  s[1] = f[2] * cam.up[0] - f[0] * cam.up[2];
  s[2] = f[0] * cam.up[1] - f[1] * cam.up[0];
  float sl = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  for (int c = 0; c < 3; ++c) s[c] /= sl;
  u[0] = s[1] * f[2] - s[2] * f[1];
  u[1] = s[2] * f[0] - s[0] * f[2];
  u[2] = s[0] * f[1] - s[1] * f[0];
  const float th = tanf(0.5f * cam.fov_y_deg * 3.14159265358979f / 180.f);
  for (int c = 0; c < 3; ++c) {
    b.eye[c] = cam.eye[c];
    b.s[c] = s[c];
    b.u[c] = u[c];
    b.f[c] = f[c];
  }
  b.ty = th;
  b.tx = th * (float)cam.width / (float)cam.height;
  return b;
}

}  // namespace

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_trace_init(const MplCamera* cam, float radius, float* origins, float* dirs,
                              int32_t* state, int32_t* active, int32_t* count, void* stream) {
  if (!cam || !origins || !dirs || !state || !active || !count) return MPL_ERR_INVALID_ARG;
  if (cam->width <= 0 || cam->height <= 0 || cam->fov_y_deg <= 0.f || cam->fov_y_deg >= 180.f)
    return MPL_ERR_INVALID_ARG;
  const int64_t P = (int64_t)cam->width * cam->height;
  if (P > INT32_MAX) return MPL_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(int32_t), s));
  int64_t blocks = (P + 255) / 256;
  if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
  trace_init_kernel<<<(unsigned)blocks, 256, 0, s>>>(make_basis(*cam), cam->width, cam->height,
                                                     radius, origins, dirs, state, active, count);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_trace_step(const float* S, const int32_t* active, const int32_t* count,
                              int64_t n_max, float* origins, const float* dirs, int32_t* state,
                              float eps, float radius, int32_t last_step, int32_t* active_out,
                              int32_t* count_out, int32_t* hit_out, int32_t* hit_count,
                              int64_t capacity, void* stream) {
  if (!S || !active || !count || !origins || !dirs || !state || !active_out || !count_out ||
      !hit_out || !hit_count || n_max < 0)
    return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(count_out, 0, sizeof(int32_t), s));
  if (n_max == 0) return MPL_OK;
  int64_t blocks = (n_max + 255) / 256;
  if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
  trace_step_kernel<<<(unsigned)blocks, 256, 0, s>>>(S, active, count, n_max, origins, dirs,
                                                     state, eps, radius, last_step, active_out,
                                                     count_out, hit_out, hit_count, capacity);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_trace_shade(const float* origins, const float* dirs, const float* G,
                               const int32_t* state, int64_t P, int32_t mode, uint32_t* image,
                               void* stream) {
  if (!origins || !dirs || !G || !state || !image || P < 0) return MPL_ERR_INVALID_ARG;
  if (P == 0) return MPL_OK;
  trace_shade_kernel<<<(unsigned)((P + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      origins, dirs, G, state, P, mode, image);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
