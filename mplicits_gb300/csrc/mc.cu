// Marching cubes on the GPU, replacing the CPU call to scikit-image's
// marching_cubes in convert_sdf_samples_to_ply (i3d/meshing.py:291-313)
// and the 512 MiB device->host copy before it (i3d/meshing.py:242).
//
// The volume is C-order [N][N][N]; a *row* is the N points (i, j, 0..N-1).
//   count:  one warp per row classifies its points (crossing edges owned by
//           each point) and cells (case -> triangle count) and writes the
//           row totals;
//   scan:   exclusive prefix sums of the row totals (int64);
//   emit:   one CTA per non-empty row rebuilds the in-row vertex prefixes of
//           the four rows a cell touches with warp scans, writes the row's
//           vertices and its triangles.
// Output order is canonical (see mplicits.h) and matches the CPU restatement
// in oracle/mc.c bit for bit: all arithmetic is float32 with explicit
// round-to-nearest intrinsics and no contraction.
#include <atomic>
#include <mutex>

#include "common.cuh"
#include "mc_tables.h"

namespace mpl {

namespace {

__constant__ unsigned char c_tri_count[256];
__constant__ signed char c_tri_edges[256][MPL_MC_MAX_TRIS * 3];
__constant__ signed char c_edge[12][7];

struct McWork {
  int32_t* row_v;   // [N*N]
  int32_t* row_t;   // [N*N]
  int64_t* pre_v;   // [N*N]
  int64_t* pre_t;   // [N*N]
  int64_t* blk;     // [2 * nblk]
  int64_t* totals;  // [2]
};

constexpr int kScanChunk = 2048;  // rows per scan block

__host__ __device__ inline int64_t mc_nblk(int64_t N) {
  return (N * N + kScanChunk - 1) / kScanChunk;
}

__host__ __device__ inline McWork mc_work(void* base, int64_t N) {
  McWork w;
  char* p = (char*)base;
  const int64_t R = N * N;
  w.row_v = (int32_t*)p;
  p += align256(R * 4);
  w.row_t = (int32_t*)p;
  p += align256(R * 4);
  w.pre_v = (int64_t*)p;
  p += align256(R * 8);
  w.pre_t = (int64_t*)p;
  p += align256(R * 8);
  w.blk = (int64_t*)p;
  p += align256(2 * mc_nblk(N) * 8);
  w.totals = (int64_t*)p;
  return w;
}

__host__ inline int64_t mc_work_bytes(int64_t N) {
  const int64_t R = N * N;
  return align256(R * 4) * 2 + align256(R * 8) * 2 + align256(2 * mc_nblk(N) * 8) + 256;
}

// Four consecutive values of a row line starting at k (a multiple of 4):
// one 16-byte load when the grid size is a multiple of 4 (every line then
// starts 16-byte aligned), otherwise scalar loads; entries past N are 0.
__device__ __forceinline__ void load4(const float* __restrict__ line, int64_t k, int64_t N,
                                      bool vec, float (&v)[4]) {
  if (vec && k + 3 < N) {
    const float4 f = *reinterpret_cast<const float4*>(line + k);
    v[0] = f.x;
    v[1] = f.y;
    v[2] = f.z;
    v[3] = f.w;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = k + e < N ? line[k + e] : 0.f;
  }
}

// Sign bits (S < iso) of the four values of a lane (bits 0..3) and of the
// value that follows them (bit 4, a separate load that hits the same or the
// next cache line).
__device__ __forceinline__ uint32_t sign5(const float* __restrict__ line, int64_t k, int64_t N,
                                          bool vec, float iso) {
  float v[4];
  load4(line, k, N, vec, v);
  const float nx = k + 4 < N ? line[k + 4] : 0.f;
  uint32_t b = 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) b |= (v[e] < iso ? 1u : 0u) << e;
  return b | ((k + 4 < N && nx < iso) ? 16u : 0u);
}

// One warp per row (i, j), 128 points per step (4 per lane): crossing edges
// owned by each point (along i, j, k, in that order of the mask bits) and the
// triangle count of each cell (i, j, k) -> (i+1, j+1, k+1).
__global__ void mc_count_kernel(const float* __restrict__ S, int64_t N, float iso, McWork w) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (r >= N * N) return;
  const int64_t i = r / N, j = r % N;
  const bool has_i = i + 1 < N, has_j = j + 1 < N;
  const bool vec = (N & 3) == 0;
  const float* L00 = S + (i * N + j) * N;
  const float* L10 = L00 + N * N;
  const float* L01 = L00 + N;
  const float* L11 = L10 + N;
  int nv = 0, nt = 0;
  for (int64_t k0 = 0; k0 < N; k0 += 128) {
    const int64_t k = k0 + 4 * lane;
    const uint32_t a = sign5(L00, k, N, vec, iso);
    const uint32_t b = has_i ? sign5(L10, k, N, vec, iso) : 0u;
    const uint32_t c = has_j ? sign5(L01, k, N, vec, iso) : 0u;
    const uint32_t d = has_i && has_j ? sign5(L11, k, N, vec, iso) : 0u;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (k + e >= N) break;
      const uint32_t s0 = (a >> e) & 1u;
      int m = 0;
      if (has_i && (((b >> e) & 1u) != s0)) m |= 1;
      if (has_j && (((c >> e) & 1u) != s0)) m |= 2;
      if (k + e + 1 < N && (((a >> (e + 1)) & 1u) != s0)) m |= 4;
      nv += __popc(m);
      if (has_i && has_j && k + e + 1 < N) {
        // corner q: (i + (q & 1), j + ((q >> 1) & 1), k + e + (q >> 2))
        const uint32_t cs = ((a >> e) & 1u) | (((b >> e) & 1u) << 1) | (((c >> e) & 1u) << 2) |
                            (((d >> e) & 1u) << 3) | (((a >> (e + 1)) & 1u) << 4) |
                            (((b >> (e + 1)) & 1u) << 5) | (((c >> (e + 1)) & 1u) << 6) |
                            (((d >> (e + 1)) & 1u) << 7);
        nt += c_tri_count[cs];
      }
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    nv += __shfl_xor_sync(0xffffffffu, nv, o);
    nt += __shfl_xor_sync(0xffffffffu, nt, o);
  }
  if (lane == 0) {
    w.row_v[r] = nv;
    w.row_t[r] = nt;
  }
}

// block-wide exclusive scan of one int64 per thread (blockDim.x a multiple
// of 32, at most 256)
__device__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warp_sums[lane] = s;
  }
  __syncthreads();
  const int64_t before = wid > 0 ? warp_sums[wid - 1] : 0;
  if (total) *total = warp_sums[nw - 1];
  __syncthreads();
  return before + x - v;
}

// phase 1: per-block exclusive scan of kScanChunk rows (256 threads x 8)
__global__ void mc_scan_blocks(int64_t N, McWork w) {
  const int64_t R = N * N;
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + threadIdx.x * 8;
  int64_t lv[8], lt[8], sv = 0, st = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int64_t r = base + q;
    lv[q] = r < R ? w.row_v[r] : 0;
    lt[q] = r < R ? w.row_t[r] : 0;
    sv += lv[q];
    st += lt[q];
  }
  int64_t tv, tt;
  int64_t ov = block_exclusive_scan(sv, &tv);
  int64_t ot = block_exclusive_scan(st, &tt);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int64_t r = base + q;
    if (r < R) {
      w.pre_v[r] = ov;
      w.pre_t[r] = ot;
    }
    ov += lv[q];
    ot += lt[q];
  }
  if (threadIdx.x == 0) {
    w.blk[2 * blockIdx.x] = tv;
    w.blk[2 * blockIdx.x + 1] = tt;
  }
}

// phase 2: one CTA scans the block totals in place, writes the grand totals
__global__ void mc_scan_top(int64_t nblk, McWork w, int64_t* counts_out) {
  int64_t carry_v = 0, carry_t = 0;
  for (int64_t b0 = 0; b0 < nblk; b0 += blockDim.x) {
    const int64_t b = b0 + threadIdx.x;
    const int64_t v = b < nblk ? w.blk[2 * b] : 0;
    const int64_t t = b < nblk ? w.blk[2 * b + 1] : 0;
    int64_t tv, tt;
    const int64_t ev = block_exclusive_scan(v, &tv);
    const int64_t et = block_exclusive_scan(t, &tt);
    if (b < nblk) {
      w.blk[2 * b] = carry_v + ev;
      w.blk[2 * b + 1] = carry_t + et;
    }
    carry_v += tv;
    carry_t += tt;
  }
  if (threadIdx.x == 0) {
    w.totals[0] = carry_v;
    w.totals[1] = carry_t;
    if (counts_out) {
      counts_out[0] = carry_v;
      counts_out[1] = carry_t;
    }
  }
}

// phase 3: add block offsets
__global__ void mc_scan_add(int64_t N, McWork w) {
  const int64_t R = N * N;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int64_t b = r / kScanChunk;
  w.pre_v[r] += w.blk[2 * b];
  w.pre_t[r] += w.blk[2 * b + 1];
}

__device__ __forceinline__ float grad_axis(const float* __restrict__ S, int64_t N,
                                           const int64_t idx[3], int axis) {
  int64_t lo[3] = {idx[0], idx[1], idx[2]};
  int64_t hi[3] = {idx[0], idx[1], idx[2]};
  if (idx[axis] > 0) lo[axis] -= 1;
  if (idx[axis] + 1 < N) hi[axis] += 1;
  const float d = __fsub_rn(S[(hi[0] * N + hi[1]) * N + hi[2]], S[(lo[0] * N + lo[1]) * N + lo[2]]);
  return __fdiv_rn(d, (float)(hi[axis] - lo[axis]));
}

constexpr int kEmitThreads = 128;
constexpr int kMaxN = 1024;

// One CTA (4 warps) per row r = (i, j); rows without vertices or triangles
// return at once.
//   1. warp w walks line (i + (w >> 1), j + (w & 1)), 128 points per step:
//      the crossing-edge mask and sign bit of each point and its in-line
//      vertex prefix (warp scan), into shared memory;
//   2. the vertices of line (i, j) (interpolation, central-difference
//      normals);
//   3. the triangles of the cells of row (i, j): each thread takes four
//      consecutive cells, the cases come from the sign bits of the four
//      lines, one block scan orders them.
__global__ void __launch_bounds__(kEmitThreads) mc_emit_kernel(
    const float* __restrict__ S, int64_t N, float iso, float vs, float o0, float o1, float o2,
    McWork w, float* __restrict__ verts, float* __restrict__ normals, float* __restrict__ values,
    int32_t* __restrict__ faces, int64_t max_verts, int64_t max_tris) {
  // in-line vertex prefix (< 3 kMaxN) and, per point, the crossing-edge mask
  // (bits 0-2: along i, j, k) with the point's sign S < iso in bit 3
  __shared__ int16_t pre[4][kMaxN];
  __shared__ uint8_t msk[4][kMaxN];
  const int64_t r = blockIdx.x;
  const int64_t i = r / N, j = r % N;
  if (w.row_v[r] == 0 && w.row_t[r] == 0) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const float org[3] = {o0, o1, o2};

  // 1. masks, prefixes and signs of the four lines
  {
    const int64_t ri = i + (wid >> 1), rj = j + (wid & 1);
    if (ri < N && rj < N) {
      const bool vec = (N & 3) == 0;
      const bool has_i = ri + 1 < N, has_j = rj + 1 < N;
      const float* L = S + (ri * N + rj) * N;
      int32_t carry = 0;
      for (int64_t k0 = 0; k0 < N; k0 += 128) {
        const int64_t k = k0 + 4 * lane;
        const uint32_t a = sign5(L, k, N, vec, iso);
        const uint32_t b = has_i ? sign5(L + N * N, k, N, vec, iso) : 0u;
        const uint32_t c = has_j ? sign5(L + N, k, N, vec, iso) : 0u;
        int m[4], cnt = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const uint32_t s0 = (a >> e) & 1u;
          int me = 0;
          if (k + e < N) {
            if (has_i && (((b >> e) & 1u) != s0)) me |= 1;
            if (has_j && (((c >> e) & 1u) != s0)) me |= 2;
            if (k + e + 1 < N && (((a >> (e + 1)) & 1u) != s0)) me |= 4;
          }
          m[e] = me;
          cnt += __popc(me);
        }
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        int run = carry + x - cnt;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (k + e < N) {
            pre[wid][k + e] = (int16_t)run;
            msk[wid][k + e] = (uint8_t)(m[e] | (((a >> e) & 1u) << 3));
          }
          run += __popc(m[e]);
        }
        carry += __shfl_sync(0xffffffffu, x, 31);
      }
    }
  }
  __syncthreads();

  // 2. vertices of line (i, j)
  const int64_t vbase = w.pre_v[r];
  for (int64_t k = threadIdx.x; k < N; k += kEmitThreads) {
    const int m = msk[0][k] & 7;
    if (!m) continue;
    int64_t v = vbase + pre[0][k];
    const int64_t p = (i * N + j) * N + k;
    for (int a = 0; a < 3; ++a) {
      if (!(m & (1 << a))) continue;
      if (v < max_verts) {
        const int64_t idx0[3] = {i, j, k};
        int64_t idx1[3] = {i, j, k};
        idx1[a] += 1;
        const float v0 = S[p];
        const float v1 = S[(idx1[0] * N + idx1[1]) * N + idx1[2]];
        const float t = __fdiv_rn(__fsub_rn(iso, v0), __fsub_rn(v1, v0));
        float n[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float c = (float)idx0[d];
          if (d == a) c = __fadd_rn(c, t);
          verts[3 * v + d] = __fadd_rn(__fmul_rn(c, vs), org[d]);
          const float g0 = grad_axis(S, N, idx0, d);
          const float g1 = grad_axis(S, N, idx1, d);
          n[d] = __fadd_rn(g0, __fmul_rn(t, __fsub_rn(g1, g0)));
        }
        float l2 = __fmul_rn(n[0], n[0]);
        l2 = __fadd_rn(l2, __fmul_rn(n[1], n[1]));
        l2 = __fadd_rn(l2, __fmul_rn(n[2], n[2]));
        const float len = __fsqrt_rn(l2);
#pragma unroll
        for (int d = 0; d < 3; ++d)
          normals[3 * v + d] = len > 0.0f ? __fdiv_rn(n[d], len) : 0.0f;
        if (values) values[v] = v0 > v1 ? v0 : v1;
      }
      ++v;
    }
  }

  // 3. triangles of the cells of row (i, j), four consecutive cells a thread
  if (i + 1 >= N || j + 1 >= N) return;
  int64_t tcarry = w.pre_t[r];
  for (int64_t k0 = 0; k0 < N - 1; k0 += 4 * kEmitThreads) {
    const int64_t kb = k0 + 4 * threadIdx.x;
    int cs[4], nts[4], ntot = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t k = kb + e;
      int c = 0;
      if (k < N - 1) {
        // corner q: (i + (q & 1), j + ((q >> 1) & 1), k + (q >> 2)); line (di, dj) = di * 2 + dj
#pragma unroll
        for (int q = 0; q < 8; ++q)
          c |= (int)((msk[((q & 1) << 1) | ((q >> 1) & 1)][k + (q >> 2)] >> 3) & 1) << q;
      }
      cs[e] = c;
      nts[e] = k < N - 1 ? c_tri_count[c] : 0;
      ntot += nts[e];
    }
    int64_t tot;
    int64_t t = tcarry + block_exclusive_scan(ntot, &tot);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t k = kb + e;
      for (int q = 0; q < nts[e]; ++q, ++t) {
        if (t >= max_tris) break;
#pragma unroll
        for (int sidx = 0; sidx < 3; ++sidx) {
          const int ed = c_tri_edges[cs[e]][3 * q + sidx];
          const int axis = c_edge[ed][0];
          const int row = c_edge[ed][1] * 2 + c_edge[ed][2];
          const int64_t kk = k + c_edge[ed][3];
          const int64_t rr = (i + c_edge[ed][1]) * N + (j + c_edge[ed][2]);
          const int64_t vid = w.pre_v[rr] + pre[row][kk] +
                              __popc((int)msk[row][kk] & ((1 << axis) - 1));
          faces[3 * t + sidx] = (int32_t)vid;
        }
      }
    }
    tcarry += tot;
  }
}

// Per-device one-time set-up (case tables here, the no-allocation
// workspace's address below): the flags are read without a lock on the fast
// path; the first calls on a device, from any number of host threads,
// serialise on g_setup_mutex, so the upload happens once.
std::atomic<bool> g_tables_loaded[64];
std::mutex g_setup_mutex;

int ensure_tables() {
  int dev = 0;
  MPL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return MPL_ERR_INVALID_ARG;
  if (g_tables_loaded[dev].load(std::memory_order_acquire)) return MPL_OK;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_tables_loaded[dev].load(std::memory_order_relaxed)) return MPL_OK;
  MPL_CUDA_TRY(cudaMemcpyToSymbol(c_tri_count, MPL_MC_TRI_COUNT, sizeof(MPL_MC_TRI_COUNT)));
  MPL_CUDA_TRY(cudaMemcpyToSymbol(c_tri_edges, MPL_MC_TRI_EDGES, sizeof(MPL_MC_TRI_EDGES)));
  MPL_CUDA_TRY(cudaMemcpyToSymbol(c_edge, MPL_MC_EDGE, sizeof(MPL_MC_EDGE)));
  g_tables_loaded[dev].store(true, std::memory_order_release);
  return MPL_OK;
}

}  // namespace

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_mc_workspace_bytes(int64_t N, int64_t* bytes) {
  if (!bytes || N < 2 || N > kMaxN) return N > kMaxN ? MPL_ERR_UNSUPPORTED : MPL_ERR_INVALID_ARG;
  *bytes = mc_work_bytes(N);
  return MPL_OK;
}

extern "C" int mpl_mc_count(const float* S, int64_t N, float iso, void* workspace,
                            int64_t* counts_dev, void* stream) {
  if (!S || !workspace || N < 2) return MPL_ERR_INVALID_ARG;
  if (N > kMaxN) return MPL_ERR_UNSUPPORTED;
  if (((uintptr_t)workspace & 255) != 0) return MPL_ERR_INVALID_ARG;
  int st = ensure_tables();
  if (st != MPL_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  McWork w = mc_work(workspace, N);
  const int64_t R = N * N;
  mc_count_kernel<<<(unsigned)((R + 7) / 8), 256, 0, s>>>(S, N, iso, w);
  MPL_LAUNCH_CHECK();
  const int64_t nblk = mc_nblk(N);
  mc_scan_blocks<<<(unsigned)nblk, 256, 0, s>>>(N, w);
  MPL_LAUNCH_CHECK();
  mc_scan_top<<<1, 256, 0, s>>>(nblk, w, counts_dev);
  MPL_LAUNCH_CHECK();
  mc_scan_add<<<(unsigned)((R + 255) / 256), 256, 0, s>>>(N, w);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_mc_emit(const float* S, int64_t N, float iso, float voxel_size,
                           const float* origin, const void* workspace, float* verts,
                           float* normals, float* values, int32_t* faces, int64_t max_verts,
                           int64_t max_tris, void* stream) {
  if (!S || !workspace || !origin || N < 2) return MPL_ERR_INVALID_ARG;
  if (N > kMaxN) return MPL_ERR_UNSUPPORTED;
  if ((max_verts > 0 && (!verts || !normals)) || (max_tris > 0 && !faces))
    return MPL_ERR_INVALID_ARG;
  int st = ensure_tables();
  if (st != MPL_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  McWork w = mc_work(const_cast<void*>(workspace), N);
  mc_emit_kernel<<<(unsigned)(N * N), kEmitThreads, 0, s>>>(
      S, N, iso, voxel_size, origin[0], origin[1], origin[2], w, verts, normals, values, faces,
      max_verts, max_tris);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// ---------------------------------------------------------------------------
// Marching cubes without any allocation, for callers that cannot allocate
// device memory.  A real-time frame loop cannot afford cudaMalloc/cudaFree,
// which synchronise the whole device, and a host that hands this library
// only buffers it registered itself (an engine plug-in, or a foreign-language
// binding without access to a CUDA allocator) has no way to provide the
// workspace mpl_mc_count/mpl_mc_emit need.  This entry point keeps that
// workspace in a fixed file-scope device array instead, sized for grids up
// to kStaticMaxN^3, which every GPU that loads the library holds until the
// process exits.
// ---------------------------------------------------------------------------
namespace mpl {

namespace {

constexpr int64_t kStaticMaxN = 256;

constexpr int64_t static_align256(int64_t x) { return (x + 255) & ~int64_t(255); }

constexpr int64_t static_ws_bytes(int64_t N) {
  return static_align256(N * N * 4) * 2 + static_align256(N * N * 8) * 2 +
         static_align256(2 * ((N * N + kScanChunk - 1) / kScanChunk) * 8) + 256;
}

// 1.5 MiB: the count/prefix workspace of a 256^3 grid.
__device__ __align__(256) unsigned char g_mc_static_ws[static_ws_bytes(kStaticMaxN)];

// Device address of g_mc_static_ws on the current device.  In host code the
// symbol itself is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
int static_ws_address(void** out) {
  static std::atomic<void*> cached[64];
  int dev = 0;
  MPL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return MPL_ERR_INVALID_ARG;
  void* p = cached[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    p = cached[dev].load(std::memory_order_relaxed);
    if (!p) {
      MPL_CUDA_TRY(cudaGetSymbolAddress(&p, g_mc_static_ws));
      cached[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return MPL_OK;
}

}  // namespace

}  // namespace mpl

extern "C" int mpl_mc_noalloc(const float* S, int64_t N, float iso, float voxel_size,
                              const float* origin, float* verts, float* normals, float* values,
                              int32_t* faces, int64_t max_verts, int64_t max_tris,
                              int64_t* counts_dev, void* stream) {
  if (!S || !origin || !counts_dev || N < 2) return MPL_ERR_INVALID_ARG;
  if (N > kStaticMaxN || mc_work_bytes(N) > (int64_t)sizeof(g_mc_static_ws))
    return MPL_ERR_CAPACITY;
  if (max_verts < 0 || max_tris < 0) return MPL_ERR_INVALID_ARG;
  if ((max_verts > 0 && (!verts || !normals)) || (max_tris > 0 && !faces))
    return MPL_ERR_INVALID_ARG;
  int st = ensure_tables();
  if (st != MPL_OK) return st;
  void* ws = nullptr;
  st = static_ws_address(&ws);
  if (st != MPL_OK) return st;
  // Every workspace entry the kernels read is written earlier in this same
  // call, so the previous call's leftovers need no clearing.
  cudaStream_t s = (cudaStream_t)stream;
  McWork w = mc_work(ws, N);
  const int64_t R = N * N;
  mc_count_kernel<<<(unsigned)((R + 7) / 8), 256, 0, s>>>(S, N, iso, w);
  MPL_LAUNCH_CHECK();
  const int64_t nblk = mc_nblk(N);
  mc_scan_blocks<<<(unsigned)nblk, 256, 0, s>>>(N, w);
  MPL_LAUNCH_CHECK();
  mc_scan_top<<<1, 256, 0, s>>>(nblk, w, counts_dev);
  MPL_LAUNCH_CHECK();
  mc_scan_add<<<(unsigned)((R + 255) / 256), 256, 0, s>>>(N, w);
  MPL_LAUNCH_CHECK();
  mc_emit_kernel<<<(unsigned)R, kEmitThreads, 0, s>>>(S, N, iso, voxel_size, origin[0],
                                                       origin[1], origin[2], w, verts, normals,
                                                       values, faces, max_verts, max_tris);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
