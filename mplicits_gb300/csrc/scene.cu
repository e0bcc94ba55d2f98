// Triangle scene and the tubular-neighbourhood deltas (calc_deltas).
//
// experiment_scripts/utils.py:46-89 bisects, for every vertex v with unit
// normal n, the radius delta of the largest ball q = v + delta * n that still
// touches the mesh only near v: each iteration asks the unsigned distance D
// from q to the mesh (an open3d RaycastingScene, built at
// experiment_scripts/train_sdf_on_neighborhood.py:145-146) and halves the step
// and steps back when |delta - D| > eps, else steps forward, while
// max(delta) < max_delta.
//
// Scene: a uniform grid of cubic cells over the mesh's bounding box (one cell
// of margin on every side).  Each cell lists the triangles whose bounding box,
// grown by a relative 1e-5, overlaps it; the lists are stored in cell order as
// the triangles' corner coordinates (three float4 per entry) beside one
// bounding sphere per entry (a separate float4 array, read first), so a query
// reads a cell's triangles as one contiguous run and computes the exact
// distance only for entries whose sphere comes near enough.  Built on the
// device by a count pass, an exclusive scan and a fill pass.
//
// Distance: the closest point of each triangle by the Voronoi-region method
// of C. Ericson, "Real-Time Collision Detection" (2005), section 5.1.5, in
// float32 with every rounding explicit (__f*_rn, fmaf where written), so the
// CPU oracle that writes the same operations gets the same bits.  A query
// visits the cells within a radius R of q in shells of growing Chebyshev
// distance from q's cell, skipping cells whose box is farther than R.
//
// Decision of one bisection step (shrink_step_warp): |delta - D| > eps for the
// minimum D is rewritten as "some triangle nearer than delta - eps, or none
// within delta + eps" (exact in float32, see shrink_step_warp), so the search
// stops at the first near triangle and, once one triangle within delta + eps
// is found, ignores everything beyond delta - eps.  The result equals the
// brute-force minimum's comparison bit for bit.
//
// One launch per iteration: the stopping rule max(delta) < max_delta couples
// all vertices, so launch i reads the maximum left by launch i - 1 (a float
// per iteration, reduced with one atomic per warp) and returns at once when it
// is reached, passing the value on; no host round trip.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cstring>

#include "common.cuh"

struct MplScene {
  int device;
  float lo[3];
  float h;
  int32_t dim[3];
  int64_t n_faces;
  int64_t n_refs;
  uint32_t* start;  // [cells + 1] offsets into tris (in entries)
  float4* tris;     // [n_refs * 3] corners a, b, c (w unused)
  float4* bound;    // [n_refs] bounding sphere: centre, radius
};

namespace mpl {
namespace scene {

constexpr int kThreads = 256;
constexpr int64_t kMaxDim = 1024;
constexpr int64_t kMaxCells = int64_t(1) << 25;
constexpr int64_t kMaxRefs = int64_t(1) << 31;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kThreads * kScanItems;

struct View {
  float lo[3];
  float h;
  int32_t dim[3];
  const uint32_t* __restrict__ start;
  const float4* __restrict__ tris;
  const float4* __restrict__ bound;
};

// ---- the exact float32 point-triangle distance -----------------------------
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 sub(V3 a, V3 b) {
  return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ float dot(V3 u, V3 v) {
  return __fmaf_rn(u.z, v.z, __fmaf_rn(u.y, v.y, __fmul_rn(u.x, v.x)));
}
// p - (s * u + o), per component
__device__ __forceinline__ V3 off_axpy(V3 p, float s, V3 u, V3 o) {
  return {__fsub_rn(p.x, __fmaf_rn(s, u.x, o.x)), __fsub_rn(p.y, __fmaf_rn(s, u.y, o.y)),
          __fsub_rn(p.z, __fmaf_rn(s, u.z, o.z))};
}

__device__ __forceinline__ float tri_dist2(V3 p, V3 a, V3 b, V3 c) {
  const V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
  const float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) return dot(ap, ap);
  const V3 bp = sub(p, b);
  const float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.f && d4 <= d3) return dot(bp, bp);
  const float vc = __fmaf_rn(d1, d4, -__fmul_rn(d3, d2));
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
    const V3 e = off_axpy(p, __fdiv_rn(d1, __fsub_rn(d1, d3)), ab, a);
    return dot(e, e);
  }
  const V3 cp = sub(p, c);
  const float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.f && d5 <= d6) return dot(cp, cp);
  const float vb = __fmaf_rn(d5, d2, -__fmul_rn(d1, d6));
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
    const V3 e = off_axpy(p, __fdiv_rn(d2, __fsub_rn(d2, d6)), ac, a);
    return dot(e, e);
  }
  const float va = __fmaf_rn(d3, d6, -__fmul_rn(d5, d4));
  const float e43 = __fsub_rn(d4, d3), e56 = __fsub_rn(d5, d6);
  if (va <= 0.f && e43 >= 0.f && e56 >= 0.f) {
    const V3 e = off_axpy(p, __fdiv_rn(e43, __fadd_rn(e43, e56)), sub(c, b), b);
    return dot(e, e);
  }
  const float denom = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(va, vb), vc));
  const float v = __fmul_rn(vb, denom), w = __fmul_rn(vc, denom);
  const V3 e = {__fsub_rn(p.x, __fmaf_rn(ac.x, w, __fmaf_rn(ab.x, v, a.x))),
                __fsub_rn(p.y, __fmaf_rn(ac.y, w, __fmaf_rn(ab.y, v, a.y))),
                __fsub_rn(p.z, __fmaf_rn(ac.z, w, __fmaf_rn(ab.z, v, a.z)))};
  return dot(e, e);
}

__device__ __forceinline__ int cell_of(float x, float lo, float h, int dim) {
  const float f = floorf(__fdiv_rn(__fsub_rn(x, lo), h));
  if (!(f >= 0.f)) return 0;
  if (f >= (float)(dim - 1)) return dim - 1;
  return (int)f;
}

__device__ __forceinline__ bool finite3(V3 q) {
  return isfinite(q.x) && isfinite(q.y) && isfinite(q.z);
}

// squared distance from q to the box of cell (x, y, z)
__device__ __forceinline__ float cell_box_d2(const View& S, V3 q, int x, int y, int z) {
  auto gap = [&](float v, float lo, int i) {
    const float a = lo + S.h * (float)i, b = lo + S.h * (float)(i + 1);
    return v < a ? a - v : (v > b ? v - b : 0.f);
  };
  const float gx = gap(q.x, S.lo[0], x), gy = gap(q.y, S.lo[1], y), gz = gap(q.z, S.lo[2], z);
  return gx * gx + gy * gy + gz * gz;
}

// Visits the cells within R of q in shells of growing Chebyshev distance from
// q's cell (clamped to the grid); visit(cell, box_d2) returns true to stop.
template <class Visit>
__device__ __forceinline__ void walk_cells(const View& S, V3 q, float R, Visit&& visit) {
  int lo[3], hi[3], c[3];
  const float qa[3] = {q.x, q.y, q.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = cell_of(qa[k] - R, S.lo[k], S.h, S.dim[k]);
    hi[k] = cell_of(qa[k] + R, S.lo[k], S.h, S.dim[k]);
    c[k] = cell_of(qa[k], S.lo[k], S.h, S.dim[k]);
  }
  int rmax = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) rmax = max(rmax, max(c[k] - lo[k], hi[k] - c[k]));
  for (int r = 0; r <= rmax; ++r) {
    const int z0 = max(lo[2], c[2] - r), z1 = min(hi[2], c[2] + r);
    const int y0 = max(lo[1], c[1] - r), y1 = min(hi[1], c[1] + r);
    for (int z = z0; z <= z1; ++z) {
      const bool zs = (z == c[2] - r) || (z == c[2] + r);
      for (int y = y0; y <= y1; ++y) {
        const bool full = zs || (y == c[1] - r) || (y == c[1] + r);
        // a full row of the shell, or only its two end cells
        const int xs = full ? max(lo[0], c[0] - r) : c[0] - r;
        const int xe = full ? min(hi[0], c[0] + r) : c[0] + r;
        const int xstep = full ? 1 : max(2 * r, 1);
        for (int x = xs; x <= xe; x += xstep) {
          if (x < lo[0] || x > hi[0]) continue;
          const int64_t cell = ((int64_t)z * S.dim[1] + y) * S.dim[0] + x;
          if (visit(cell, cell_box_d2(S, q, x, y, z))) return;
        }
      }
    }
  }
}

__device__ __forceinline__ float entry_dist(const View& S, V3 q, uint32_t e) {
  const float4 A = S.tris[3 * (int64_t)e], B = S.tris[3 * (int64_t)e + 1],
               C = S.tris[3 * (int64_t)e + 2];
  return __fsqrt_rn(tri_dist2(q, {A.x, A.y, A.z}, {B.x, B.y, B.z}, {C.x, C.y, C.z}));
}

// squared distance from q to an entry's bounding-sphere centre
__device__ __forceinline__ float centre_d2(V3 q, float4 b) {
  const float dx = q.x - b.x, dy = q.y - b.y, dz = q.z - b.z;
  return dx * dx + dy * dy + dz * dz;
}

// margin added to a search radius: far above the rounding of the cell, box
// and sphere arithmetic at the coordinates' magnitude
__device__ __forceinline__ float margin(V3 q, float h) {
  return 1e-5f * (fmaxf(fabsf(q.x), fmaxf(fabsf(q.y), fabsf(q.z))) + h);
}

// Minimum distance from q over the triangles within R of q (INFINITY when
// none).  An entry whose bounding sphere lies farther than the best so far
// cannot lower it and is skipped; the minimum is the same.
__device__ float nearest(const View& S, V3 q, float R) {
  const float m = margin(q, S.h);
  float best = INFINITY;
  walk_cells(S, q, R, [&](int64_t cell, float box_d2) {
    const float lim = fminf(best * 1.0001f + m, R);
    if (box_d2 > lim * lim) return false;
    const uint32_t e0 = S.start[cell], e1 = S.start[cell + 1];
    for (uint32_t e = e0; e < e1; ++e) {
      const float4 b = S.bound[e];
      const float l = (fminf(best * 1.0001f + m, R) + b.w) * 1.00002f;
      if (centre_d2(q, b) > l * l) continue;
      const float d = entry_dist(S, q, e);
      if (d < best) best = d;
    }
    return false;
  });
  return best;
}

// One bisection decision, |delta - D| > eps for D the minimum distance over
// all triangles, in float32.  With d_t each triangle's distance and the
// rounded differences monotone in d_t, it equals
//   (some t has delta - d_t > eps)  or  (no t has d_t - delta <= eps):
// the first ("close") ends the search; the second needs one witness
// ("touch").  Triangles farther than delta + eps can be neither; once a
// witness is found, only triangles nearer than delta - eps still matter.
// Both radii carry a margin, so the skips (cells by box, entries by bounding
// sphere) never drop a triangle that could change the answer.
//
// One query per warp; the close/touch flags are combined with __any_sync
// (they do not depend on the visiting order).
__device__ bool shrink_step_warp(const View& S, V3 q, float delta, float eps, int lane) {
  const float m = margin(q, S.h);
  const float r_touch = (delta + eps) * 1.0001f + m;
  const float r_close = fmaxf(delta - eps, 0.f) * 1.0001f + m;
  const int y0 = cell_of(q.y - r_touch, S.lo[1], S.h, S.dim[1]);
  const int z0 = cell_of(q.z - r_touch, S.lo[2], S.h, S.dim[2]);
  const int ny = cell_of(q.y + r_touch, S.lo[1], S.h, S.dim[1]) - y0 + 1;
  const int nz = cell_of(q.z + r_touch, S.lo[2], S.h, S.dim[2]) - z0 + 1;
  const int rows = ny * nz;
  const float inv_ny = 1.f / (float)ny;
  bool touch = false;
  // Rows of cells (y, z) are contiguous in the entry lists, so the entries of
  // the x-segment a row shares with the ball are one range: each lane takes a
  // row, and a warp prefix sum over the ranges hands the entries out one per
  // lane.
  for (int base = 0; base < rows; base += 32) {
    const float lim = touch ? r_close : r_touch;
    const int k = base + lane;
    uint32_t e0 = 0, cnt = 0;
    if (k < rows) {
      // k -> (y, z): a float quotient and exact integer corrections
      int zq = (int)((float)k * inv_ny);
      int yr = k - zq * ny;
      while (yr < 0) --zq, yr += ny;
      while (yr >= ny) ++zq, yr -= ny;
      const int y = y0 + yr, z = z0 + zq;
      const float ya = S.lo[1] + S.h * (float)y, yb = ya + S.h;
      const float za = S.lo[2] + S.h * (float)z, zb = za + S.h;
      const float gy = q.y < ya ? ya - q.y : (q.y > yb ? q.y - yb : 0.f);
      const float gz = q.z < za ? za - q.z : (q.z > zb ? q.z - zb : 0.f);
      const float w2 = lim * lim - gy * gy - gz * gz;
      if (w2 >= 0.f) {
        const float w = sqrtf(w2);
        const int xa = cell_of(q.x - w, S.lo[0], S.h, S.dim[0]);
        const int xb = cell_of(q.x + w, S.lo[0], S.h, S.dim[0]);
        const int64_t row = ((int64_t)z * S.dim[1] + y) * S.dim[0];
        e0 = S.start[row + xa];
        cnt = S.start[row + xb + 1] - e0;
      }
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const uint32_t T = __shfl_sync(0xffffffffu, incl, 31);
    for (uint32_t j0 = 0; j0 < T; j0 += 32) {
      const uint32_t j = j0 + lane;
      // the owning row's lane: the first lane whose inclusive count exceeds j
      int L = 0;
#pragma unroll
      for (int st = 16; st; st >>= 1)
        if (__shfl_sync(0xffffffffu, incl, L + st - 1) <= j) L += st;
      const uint32_t oi = __shfl_sync(0xffffffffu, incl, L & 31);
      const uint32_t oc = __shfl_sync(0xffffffffu, cnt, L & 31);
      const uint32_t oe = __shfl_sync(0xffffffffu, e0, L & 31);
      bool c_close = false, c_touch = false;
      if (j < T) {
        const uint32_t e = oe + (j - (oi - oc));
        const float4 b = S.bound[e];
        const float l = ((touch ? r_close : r_touch) + b.w) * 1.00002f;
        if (centre_d2(q, b) <= l * l) {
          const float d = entry_dist(S, q, e);
          c_close = __fsub_rn(delta, d) > eps;
          c_touch = __fsub_rn(d, delta) <= eps;
        }
      }
      if (__any_sync(0xffffffffu, c_close)) return true;
      touch = touch || __any_sync(0xffffffffu, c_touch);
    }
  }
  return !touch;
}

// ---- scene build -----------------------------------------------------------
__device__ __forceinline__ uint32_t ord(float f) {  // order-preserving float key
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float unord(uint32_t k) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
#else
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

// stats: [0..2] min keys, [3..5] max keys, [6..7] sum of edge lengths (double)
__global__ void bounds_kernel(const float* __restrict__ pos, int64_t nv,
                              const int32_t* __restrict__ faces, int64_t nf, uint32_t* keys,
                              double* edge_sum, int* bad_index) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  double es = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += stride) {
    int32_t f[3] = {faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]};
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 3; ++j) ok &= f[j] >= 0 && f[j] < nv;
    if (!ok) {
      atomicExch(bad_index, 1);
      continue;
    }
    float p[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) p[j][k] = pos[3 * (int64_t)f[j] + k];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        mn[k] = fminf(mn[k], p[j][k]);
        mx[k] = fmaxf(mx[k], p[j][k]);
      }
      const int j1 = (j + 1) % 3;
      const float dx = p[j1][0] - p[j][0], dy = p[j1][1] - p[j][1], dz = p[j1][2] - p[j][2];
      es += sqrt((double)dx * dx + (double)dy * dy + (double)dz * dz);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  for (int o = 16; o; o >>= 1) es += __shfl_xor_sync(0xffffffffu, es, o);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (mn[k] <= mx[k]) {
        atomicMin(&keys[k], ord(mn[k]));
        atomicMax(&keys[3 + k], ord(mx[k]));
      }
    }
    atomicAdd(edge_sum, es);
  }
}

__device__ __forceinline__ void tri_cells(const View& S, const float* __restrict__ pos,
                                          const int32_t* __restrict__ faces, int64_t t,
                                          int (&a)[3], int (&b)[3], float4 (&corner)[3]) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int64_t v = faces[3 * t + j];
    const float x = pos[3 * v], y = pos[3 * v + 1], z = pos[3 * v + 2];
    corner[j] = make_float4(x, y, z, 0.f);
    mn[0] = fminf(mn[0], x), mn[1] = fminf(mn[1], y), mn[2] = fminf(mn[2], z);
    mx[0] = fmaxf(mx[0], x), mx[1] = fmaxf(mx[1], y), mx[2] = fmaxf(mx[2], z);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float m = 1e-5f * (fabsf(mn[k]) + fabsf(mx[k]) + S.h);
    a[k] = cell_of(mn[k] - m, S.lo[k], S.h, S.dim[k]);
    b[k] = cell_of(mx[k] + m, S.lo[k], S.h, S.dim[k]);
  }
}

__global__ void count_kernel(View S, const float* __restrict__ pos,
                             const int32_t* __restrict__ faces, int64_t nf, uint32_t* counts,
                             unsigned long long* total) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long n = 0;
  if (t < nf) {
    int a[3], b[3];
    float4 cr[3];
    tri_cells(S, pos, faces, t, a, b, cr);
    for (int z = a[2]; z <= b[2]; ++z)
      for (int y = a[1]; y <= b[1]; ++y)
        for (int x = a[0]; x <= b[0]; ++x)
          atomicAdd(&counts[((int64_t)z * S.dim[1] + y) * S.dim[0] + x], 1u);
    n = (unsigned long long)(b[0] - a[0] + 1) * (b[1] - a[1] + 1) * (b[2] - a[2] + 1);
  }
  for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(total, n);
}

// exclusive scan of n uint32 counts in three passes (blocks of kScanBlock)
__global__ void scan_blocks(const uint32_t* __restrict__ in, uint32_t* out, int64_t n,
                            uint32_t* block_sums) {
  __shared__ uint32_t warp_tot[kThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems], s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    v[j] = base + j < n ? in[base + j] : 0u;
    s += v[j];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  uint32_t woff = 0;
  for (int w = 0; w < warp; ++w) woff += warp_tot[w];
  uint32_t run = woff + incl - s;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == kThreads - 1) block_sums[blockIdx.x] = run;
}

__global__ void scan_top(uint32_t* block_sums, int64_t nb) {
  // one block: a sequential chunk per thread, then a scan of the chunk sums
  __shared__ uint32_t tot[kThreads];
  const int64_t per = (nb + kThreads - 1) / kThreads;
  const int64_t b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
  uint32_t s = 0;
  for (int64_t b = b0; b < b1; ++b) s += block_sums[b];
  tot[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int i = 0; i < kThreads; ++i) {
      const uint32_t t = tot[i];
      tot[i] = run;
      run += t;
    }
  }
  __syncthreads();
  uint32_t run = tot[threadIdx.x];
  for (int64_t b = b0; b < b1; ++b) {
    const uint32_t t = block_sums[b];
    block_sums[b] = run;
    run += t;
  }
}

__global__ void scan_add(uint32_t* out, int64_t n, const uint32_t* __restrict__ block_sums,
                         uint32_t total) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += block_sums[i / kScanBlock];
  if (i == n) out[n] = total;
}

__global__ void fill_kernel(View S, const float* __restrict__ pos,
                            const int32_t* __restrict__ faces, int64_t nf, uint32_t* cursor,
                            float4* tris, float4* bound) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  int a[3], b[3];
  float4 cr[3];
  tri_cells(S, pos, faces, t, a, b, cr);
  // bounding sphere about the centroid, grown past its own rounding
  const float cx = (cr[0].x + cr[1].x + cr[2].x) / 3.f, cy = (cr[0].y + cr[1].y + cr[2].y) / 3.f,
              cz = (cr[0].z + cr[1].z + cr[2].z) / 3.f;
  float r2 = 0.f;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float dx = cr[j].x - cx, dy = cr[j].y - cy, dz = cr[j].z - cz;
    r2 = fmaxf(r2, dx * dx + dy * dy + dz * dz);
  }
  const float rad = sqrtf(r2) * 1.0001f +
                    1e-5f * (fmaxf(fabsf(cx), fmaxf(fabsf(cy), fabsf(cz))) + S.h);
  const float4 sphere = make_float4(cx, cy, cz, rad);
  for (int z = a[2]; z <= b[2]; ++z)
    for (int y = a[1]; y <= b[1]; ++y)
      for (int x = a[0]; x <= b[0]; ++x) {
        const uint32_t e = atomicAdd(&cursor[((int64_t)z * S.dim[1] + y) * S.dim[0] + x], 1u);
        tris[3 * (int64_t)e] = cr[0];
        tris[3 * (int64_t)e + 1] = cr[1];
        tris[3 * (int64_t)e + 2] = cr[2];
        bound[e] = sphere;
      }
}

// ---- queries ----------------------------------------------------------------
__global__ void distance_kernel(View S, const float* __restrict__ pts, int64_t n,
                                float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V3 q = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  if (!finite3(q)) {
    out[i] = __int_as_float(0x7fc00000);
    return;
  }
  // grow the radius until the nearest triangle found lies inside it (no
  // unvisited triangle can then be nearer), or it reaches every cell: rmax
  // is the distance to the grid's farthest corner
  const float qa[3] = {q.x, q.y, q.z};
  float far2 = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float a = fabsf(qa[k] - S.lo[k]), b = fabsf(qa[k] - (S.lo[k] + S.h * S.dim[k]));
    far2 += fmaxf(a, b) * fmaxf(a, b);
  }
  const float rmax = sqrtf(far2) * 1.001f + S.h;
  float r = S.h;
  float best;
  for (;;) {
    best = nearest(S, q, r * 1.0001f + margin(q, S.h));
    if (best <= r || r >= rmax) break;
    r = fminf(r * 4.f, rmax);
  }
  out[i] = best;
}

// calc_deltas: normalise normals, copy the rows, append delta = step0
__global__ void deltas_init(const float* __restrict__ v, int64_t M, int C, float step0,
                            float* __restrict__ out, float* __restrict__ step, float* maxd) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) maxd[0] = step0;
  if (i >= M) return;
  const float* r = v + i * C;
  float* o = out + i * (C + 1);
  for (int k = 0; k < C; ++k) o[k] = r[k];
  const float len = __fsqrt_rn(
      __fadd_rn(__fadd_rn(__fmul_rn(r[3], r[3]), __fmul_rn(r[4], r[4])), __fmul_rn(r[5], r[5])));
  o[3] = __fdiv_rn(r[3], len);
  o[4] = __fdiv_rn(r[4], len);
  o[5] = __fdiv_rn(r[5], len);
  o[C] = step0;
  step[i] = step0;
}

// one bisection step, one vertex per warp at a time; maxd[it] is the maximum
// delta before it, maxd[it + 1] collects the maximum after it
// (zero-initialised; deltas are positive whenever the loop runs, so the
// float bits order as integers; one atomic per block)
__global__ void __launch_bounds__(kThreads, 5) deltas_iter(View S, const float* __restrict__ v,
                                                        int64_t M, int C, float max_delta,
                                                        float eps, float* __restrict__ out,
                                                        float* __restrict__ step, float* maxd,
                                                        int it) {
  const float before = maxd[it];
  if (!(before < max_delta)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) maxd[it + 1] = before;
    return;
  }
  __shared__ float wmax_s[kThreads / 32];
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float wmax = 0.f;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < M; i += nwarps) {
    float* o = out + i * (C + 1);
    const float delta = o[C];
    const V3 q = {__fadd_rn(v[i * C], __fmul_rn(delta, o[3])),
                  __fadd_rn(v[i * C + 1], __fmul_rn(delta, o[4])),
                  __fadd_rn(v[i * C + 2], __fmul_rn(delta, o[5]))};
    const bool shrink = finite3(q) && shrink_step_warp(S, q, delta, eps, lane);
    float s = step[i];
    if (shrink) s = __fmul_rn(s, 0.5f);
    const float nd = shrink ? __fsub_rn(delta, s) : __fadd_rn(delta, s);
    __syncwarp();
    if (lane == 0) {
      step[i] = s;
      o[C] = nd;
    }
    wmax = fmaxf(wmax, nd);
  }
  if (lane == 0) wmax_s[threadIdx.x >> 5] = wmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < kThreads / 32; ++w) b = fmaxf(b, wmax_s[w]);
    if (b > 0.f) atomicMax((int*)&maxd[it + 1], __float_as_int(b));
  }
}

__global__ void deltas_count(const float* __restrict__ maxd, int n_iters, float max_delta,
                             int32_t* iterations) {
  int n = 0;
  for (int i = 0; i < n_iters; ++i) n += maxd[i] < max_delta ? 1 : 0;
  *iterations = n;
}

inline View view(const MplScene* s) {
  View v;
  for (int k = 0; k < 3; ++k) v.lo[k] = s->lo[k], v.dim[k] = s->dim[k];
  v.h = s->h;
  v.start = s->start;
  v.tris = s->tris;
  v.bound = s->bound;
  return v;
}

inline unsigned blocks(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// queries run on the device that holds the scene's grid
inline int check_device(const MplScene* s) {
  int dev = -1;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return MPL_ERR_CUDA;
  }
  return dev == s->device ? MPL_OK : MPL_ERR_INVALID_ARG;
}

}  // namespace scene
}  // namespace mpl

using namespace mpl;
using namespace mpl::scene;

extern "C" int mpl_scene_create(const float* positions_dev, int64_t n_positions,
                                const int32_t* faces_dev, int64_t n_faces, float cell,
                                MplScene** out, void* stream) {
  if (!out) return MPL_ERR_INVALID_ARG;
  *out = nullptr;
  if (!positions_dev || !faces_dev || n_positions < 3 || n_faces < 1 || !(cell >= 0.f))
    return MPL_ERR_INVALID_ARG;
  if (n_faces >= kMaxRefs) return MPL_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  MPL_CUDA_TRY(cudaGetDevice(&dev));

  // bounds, mean edge length, face-index check
  struct Stats {
    uint32_t keys[6];
    int bad;
    int pad;
    double edge_sum;
  };
  Stats* st = nullptr;
  MPL_CUDA_TRY(cudaMalloc(&st, sizeof(Stats)));
  Stats init;
  for (int k = 0; k < 3; ++k) init.keys[k] = 0xffffffffu, init.keys[3 + k] = 0u;
  init.bad = 0;
  init.pad = 0;
  init.edge_sum = 0.0;
  Stats host;
  cudaError_t e = cudaMemcpyAsync(st, &init, sizeof(Stats), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int64_t nb_want = blocks(n_faces), nb_cap = (int64_t)sm_count() * 8;
    const unsigned nb = (unsigned)(nb_want < nb_cap ? nb_want : nb_cap);
    bounds_kernel<<<nb, kThreads, 0, s>>>(positions_dev, n_positions, faces_dev, n_faces,
                                          st->keys, &st->edge_sum, &st->bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&host, st, sizeof(Stats), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(st);
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return MPL_ERR_CUDA;
  }
  if (host.bad) return MPL_ERR_INVALID_ARG;
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = unord(host.keys[k]);
    hi[k] = unord(host.keys[3 + k]);
    if (!isfinite(lo[k]) || !isfinite(hi[k])) return MPL_ERR_INVALID_ARG;
  }
  float h = cell;
  if (h <= 0.f) h = (float)(2.0 * host.edge_sum / (3.0 * (double)n_faces));
  float ext = 0.f;
  for (int k = 0; k < 3; ++k) ext = fmaxf(ext, hi[k] - lo[k]);
  if (!(h > 0.f)) h = ext > 0.f ? ext : 1.f;
  // bound the cell count: each dimension <= kMaxDim, the product <= kMaxCells
  int64_t dim[3], cells = 0;
  for (int guard = 0; guard < 64; ++guard) {
    cells = 1;
    for (int k = 0; k < 3; ++k) {
      dim[k] = (int64_t)((hi[k] - lo[k]) / h) + 3;
      cells *= dim[k];
    }
    if (cells <= kMaxCells && dim[0] <= kMaxDim && dim[1] <= kMaxDim && dim[2] <= kMaxDim) break;
    h *= 1.25f;
  }

  MplScene* sc = new MplScene();
  sc->device = dev;
  sc->h = h;
  for (int k = 0; k < 3; ++k) sc->lo[k] = lo[k] - h, sc->dim[k] = (int32_t)dim[k];
  sc->n_faces = n_faces;
  const int64_t nb = (cells + kScanBlock - 1) / kScanBlock;
  uint32_t *counts = nullptr, *bsum = nullptr;
  unsigned long long* total = nullptr;
  unsigned long long total_h = 0;
  auto fail = [&](cudaError_t err) {
    set_last_cuda_error(err);
    cudaFree(counts);
    cudaFree(bsum);
    cudaFree(total);
    cudaFree(sc->start);
    cudaFree(sc->tris);
    cudaFree(sc->bound);
    delete sc;
    return MPL_ERR_CUDA;
  };
  if ((e = cudaMalloc(&counts, sizeof(uint32_t) * cells)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&sc->start, sizeof(uint32_t) * (cells + 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&bsum, sizeof(uint32_t) * nb)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&total, sizeof(unsigned long long))) != cudaSuccess) return fail(e);
  if ((e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * cells, s)) != cudaSuccess) return fail(e);
  if ((e = cudaMemsetAsync(total, 0, sizeof(unsigned long long), s)) != cudaSuccess)
    return fail(e);
  View v = view(sc);
  count_kernel<<<blocks(n_faces), kThreads, 0, s>>>(v, positions_dev, faces_dev, n_faces, counts,
                                                    total);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpyAsync(&total_h, total, sizeof(total_h), cudaMemcpyDeviceToHost, s)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e);
  if (total_h >= (unsigned long long)kMaxRefs) {
    fail(cudaSuccess);
    return MPL_ERR_UNSUPPORTED;
  }
  sc->n_refs = (int64_t)total_h;
  scan_blocks<<<(unsigned)nb, kThreads, 0, s>>>(counts, sc->start, cells, bsum);
  scan_top<<<1, kThreads, 0, s>>>(bsum, nb);
  scan_add<<<blocks(cells + 1), kThreads, 0, s>>>(sc->start, cells, bsum, (uint32_t)total_h);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&sc->tris, sizeof(float4) * 3 * (total_h > 0 ? total_h : 1))) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaMalloc(&sc->bound, sizeof(float4) * (total_h > 0 ? total_h : 1))) != cudaSuccess)
    return fail(e);
  // counts becomes the fill cursor
  if ((e = cudaMemcpyAsync(counts, sc->start, sizeof(uint32_t) * cells, cudaMemcpyDeviceToDevice,
                           s)) != cudaSuccess)
    return fail(e);
  v = view(sc);
  fill_kernel<<<blocks(n_faces), kThreads, 0, s>>>(v, positions_dev, faces_dev, n_faces, counts,
                                                   sc->tris, sc->bound);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e);
  cudaFree(counts);
  cudaFree(bsum);
  cudaFree(total);
  *out = sc;
  return MPL_OK;
}

extern "C" int mpl_scene_destroy(MplScene* scene) {
  if (!scene) return MPL_OK;
  // queries still queued on any stream read the grid: let them finish
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(scene->start);
  cudaFree(scene->tris);
  cudaFree(scene->bound);
  delete scene;
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return MPL_ERR_CUDA;
  }
  return MPL_OK;
}

extern "C" int mpl_scene_info(const MplScene* scene, float* lo3, float* cell, int32_t* dims3,
                              int64_t* n_refs) {
  if (!scene) return MPL_ERR_INVALID_ARG;
  for (int k = 0; k < 3; ++k) {
    if (lo3) lo3[k] = scene->lo[k];
    if (dims3) dims3[k] = scene->dim[k];
  }
  if (cell) *cell = scene->h;
  if (n_refs) *n_refs = scene->n_refs;
  return MPL_OK;
}

extern "C" int mpl_scene_compute_distance(const MplScene* scene, const float* points_dev,
                                          int64_t n, float* out_dev, void* stream) {
  if (!scene || n < 0 || (n > 0 && (!points_dev || !out_dev))) return MPL_ERR_INVALID_ARG;
  if (n == 0) return MPL_OK;
  const int dst = check_device(scene);
  if (dst != MPL_OK) return dst;
  const View v = view(scene);
  distance_kernel<<<blocks(n), kThreads, 0, (cudaStream_t)stream>>>(v, points_dev, n, out_dev);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_calc_deltas_scratch_bytes(int64_t n_vertices, int32_t n_iters,
                                             int64_t* bytes) {
  if (!bytes || n_vertices < 1 || n_iters < 1) return MPL_ERR_INVALID_ARG;
  *bytes = ((n_iters + 1 + 63) / 64) * 256 + n_vertices * (int64_t)sizeof(float);
  return MPL_OK;
}

extern "C" int mpl_calc_deltas(const MplScene* scene, const float* vertices_dev,
                               int64_t n_vertices, int32_t cols, float max_delta, float step0,
                               int32_t n_iters, float eps, void* scratch_dev, float* out_dev,
                               int32_t* iterations_dev, void* stream) {
  if (!scene || !vertices_dev || !out_dev || !scratch_dev || n_vertices < 1 || cols < 6 ||
      n_iters < 1 || !isfinite(max_delta) || !isfinite(step0) || !(eps >= 0.f))
    return MPL_ERR_INVALID_ARG;
  if (((uintptr_t)scratch_dev & 255) != 0) return MPL_ERR_INVALID_ARG;
  const int dst = check_device(scene);
  if (dst != MPL_OK) return dst;
  cudaStream_t s = (cudaStream_t)stream;
  float* maxd = (float*)scratch_dev;
  float* step = (float*)((char*)scratch_dev + ((n_iters + 1 + 63) / 64) * 256);
  MPL_CUDA_TRY(cudaMemsetAsync(maxd, 0, sizeof(float) * (n_iters + 1), s));
  deltas_init<<<blocks(n_vertices), kThreads, 0, s>>>(vertices_dev, n_vertices, cols, step0,
                                                      out_dev, step, maxd);
  MPL_LAUNCH_CHECK();
  const View v = view(scene);
  // one warp per vertex, about 16 resident blocks per SM's worth of warps
  const int64_t want = (n_vertices + kThreads / 32 - 1) / (kThreads / 32);
  const unsigned nblk = (unsigned)(want < (int64_t)sm_count() * 16 ? want : (int64_t)sm_count() * 16);
  for (int it = 0; it < n_iters; ++it) {
    deltas_iter<<<nblk, kThreads, 0, s>>>(v, vertices_dev, n_vertices, cols, max_delta, eps,
                                          out_dev, step, maxd, it);
    MPL_LAUNCH_CHECK();
  }
  if (iterations_dev) {
    deltas_count<<<1, 1, 0, s>>>(maxd, n_iters, max_delta, iterations_dev);
    MPL_LAUNCH_CHECK();
  }
  return MPL_OK;
}
