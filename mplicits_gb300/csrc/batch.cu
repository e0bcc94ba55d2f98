// Host side of the batched launch: plan preparation (entry table on the
// device), the launch itself (graph-capturable: one kernel, no host sync),
// and the autotuner that picks the pipeline (one or two tiles per CTA), the
// epilogue unit width and the weight-ring depth by timing the real plan.
#include <string.h>

#include <algorithm>

#include <vector>

#include "batch_launch.h"

namespace mpl {
namespace batch {

static size_t table_bytes(int32_t count) {
  return ((size_t)count * sizeof(Entry) + 255) & ~(size_t)255;
}

// the workspace: the entry table, then the tile prefix [count + 1]
static size_t workspace_bytes(int32_t count) {
  return table_bytes(count) + (((size_t)(count + 1) * 4 + 255) & ~(size_t)255);
}

// Exclusive prefix of the entries' tile counts (device counts applied) into
// a.tiles, for the two-tile batched kernel: one block of 1024 threads.
static_assert(kMaxEntries <= 1024, "one prefix block covers every entry");
__global__ void __launch_bounds__(1024) batch_prefix_kernel(const Args a) {
  __shared__ int32_t warp_sum[32];
  const int e = threadIdx.x, lane = e & 31, w = e >> 5;
  int32_t v = 0;
  if (e < a.count) v = (int32_t)((entry_points(a.entries[e]) + kM - 1) / kM);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) warp_sum[w] = v;
  __syncthreads();
  if (w == 0) {
    int32_t x = warp_sum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += u;
    }
    warp_sum[lane] = x;  // inclusive over warps
  }
  __syncthreads();
  const int32_t incl = v + (w > 0 ? warp_sum[w - 1] : 0);
  if (e < a.count) a.tiles[e + 1] = incl;
  if (e == 0) a.tiles[0] = 0;
}


static int launch_config(const Args& a, int32_t precision, int unit, int stages, int ctas,
                         cudaStream_t s) {
  const bool f16 = precision == MPL_F16;
  if (unit == 16 && stages == 2) return f16 ? launch_u16_s2_f16(a, ctas, s) : launch_u16_s2_bf16(a, ctas, s);
  if (unit == 16 && stages == 3) return f16 ? launch_u16_s3_f16(a, ctas, s) : launch_u16_s3_bf16(a, ctas, s);
  if (unit == 32 && stages == 2) return f16 ? launch_u32_s2_f16(a, ctas, s) : launch_u32_s2_bf16(a, ctas, s);
  if (unit == 32 && stages == 3) return f16 ? launch_u32_s3_f16(a, ctas, s) : launch_u32_s3_bf16(a, ctas, s);
  return MPL_ERR_INVALID_ARG;
}

// Defaults: two tiles per CTA, 32-wide epilogue units (the level kernels'
// default), one CTA per SM; the one-tile pipeline's weight ring 3 stages
// deep (the two-tile pipeline takes the level kernel's ring at each width).
static int resolve(const MplBatchConfig* cfg, int* tiles, int* unit, int* stages, int* ctas) {
  *tiles = cfg && cfg->tiles_in_flight ? cfg->tiles_in_flight : 2;
  *unit = cfg && cfg->epilogue_unit ? cfg->epilogue_unit : 32;
  *stages = cfg && cfg->stages ? cfg->stages : (*tiles == 2 ? 0 : 3);
  *ctas = cfg && cfg->ctas > 0 ? cfg->ctas : sm_count();
  if ((*tiles != 1 && *tiles != 2) || (*unit != 16 && *unit != 32) || *ctas <= 0)
    return MPL_ERR_INVALID_ARG;
  if (*tiles == 1 && *stages != 2 && *stages != 3) return MPL_ERR_INVALID_ARG;
  // two A operands leave shared memory for the level kernel's ring and the
  // 32-wide epilogue's reduction buffers only
  if (*tiles == 2 && (*stages != 0 || *unit != 32)) return MPL_ERR_UNSUPPORTED;
  return MPL_OK;
}

}  // namespace batch
}  // namespace mpl

using namespace mpl;
using namespace mpl::batch;

extern "C" int mpl_batch_workspace_bytes(int32_t count, int64_t* bytes) {
  if (!bytes || count < 0 || count > kMaxEntries) return MPL_ERR_INVALID_ARG;
  *bytes = (int64_t)workspace_bytes(count);
  return MPL_OK;
}

extern "C" int mpl_batch_prepare(const MplBatchEntry* entries, int32_t count, int32_t precision,
                                 void* workspace, int64_t workspace_bytes, MplBatchPlan* plan,
                                 void* stream) {
  if (!plan || count < 0 || count > kMaxEntries || (count > 0 && (!entries || !workspace)))
    return MPL_ERR_INVALID_ARG;
  if (precision != MPL_BF16 && precision != MPL_F16) return MPL_ERR_UNSUPPORTED;
  if ((int64_t)mpl::batch::workspace_bytes(count) > workspace_bytes) return MPL_ERR_CAPACITY;
  if (((uintptr_t)workspace & 255) != 0) return MPL_ERR_INVALID_ARG;
  const bool f16 = precision == MPL_F16;
  std::vector<Entry> tab((size_t)count);
  for (int32_t i = 0; i < count; ++i) {
    const MplBatchEntry& in = entries[i];
    Entry& e = tab[(size_t)i];
    memset(&e, 0, sizeof(e));
    PackLayout lay;
    int st = make_layout(&in.net, &lay);
    if (st != MPL_OK) return st;
    if (lay.nh < 1 || lay.nh > kMaxHidden || lay.WP > kWPMax) return MPL_ERR_UNSUPPORTED;
    if (!in.packed_dev || ((uintptr_t)in.packed_dev & 255) != 0) return MPL_ERR_INVALID_ARG;
    if (in.n < 0 || in.n > INT32_MAX || (!in.S_dev && (in.n > 0 || in.n_dev)))
      return MPL_ERR_INVALID_ARG;
    if (in.store_mode != MPL_STORE && in.store_mode != MPL_ACCUMULATE) return MPL_ERR_INVALID_ARG;
    if (in.points.kind == MPL_POINTS_XYZ) {
      if (!in.points.xyz && in.n > 0) return MPL_ERR_INVALID_ARG;
    } else if (in.points.kind == MPL_POINTS_GRID) {
      const int64_t N = in.points.grid_n;
      if (N < 2) return MPL_ERR_INVALID_ARG;
      if (N * N * N > (int64_t)INT32_MAX + 1) return MPL_ERR_UNSUPPORTED;
    } else {
      return MPL_ERR_INVALID_ARG;
    }
    e.packed = (const char*)in.packed_dev;
    e.xyz = in.points.xyz;
    e.index = in.index_dev;
    e.n_dev = in.n_dev;
    e.S = in.S_dev;
    e.n = in.n;
    e.w0f = lay.w0f;
    e.wout = lay.wout;
    e.bout = lay.bout;
    for (int l = 1; l <= lay.nh; ++l) {
      e.hw[l - 1] = f16 ? lay.hwh[l] : lay.hw[l];
      e.hbx[l - 1] = f16 ? lay.hbxh[l] : lay.hbx[l];
    }
    e.nh = lay.nh;
    e.WP = lay.WP;
    e.kind = in.points.kind;
    e.grid_n = in.points.grid_n;
    e.voxel = in.points.voxel_size;
    e.off0 = in.points.offset[0];
    e.off1 = in.points.offset[1];
    e.off2 = in.points.offset[2];
    e.store_mode = in.store_mode;
  }
  // entries grouped by padded width (64, 128, 256), each group in the
  // caller's order: the two-tile kernel runs one launch per group
  std::stable_sort(tab.begin(), tab.end(),
                   [](const Entry& x, const Entry& y) { return x.WP < y.WP; });
  int32_t widths[3] = {0, 0, 0};
  for (const Entry& e : tab) ++widths[e.WP == 64 ? 0 : (e.WP == 128 ? 1 : 2)];
  cudaStream_t s = (cudaStream_t)stream;
  if (count > 0) {
    MPL_CUDA_TRY(cudaMemcpyAsync(workspace, tab.data(), (size_t)count * sizeof(Entry),
                                 cudaMemcpyHostToDevice, s));
    // the host table is released on return
    MPL_CUDA_TRY(cudaStreamSynchronize(s));
  }
  plan->workspace_dev = workspace;
  plan->count = count;
  plan->precision = precision;
  for (int i = 0; i < 3; ++i) plan->width_count[i] = widths[i];
  plan->reserved = 0;
  return MPL_OK;
}

extern "C" int mpl_batch_run(const MplBatchPlan* plan, const MplBatchConfig* config,
                             void* stream) {
  if (!plan || plan->count < 0 || plan->count > kMaxEntries) return MPL_ERR_INVALID_ARG;
  if (plan->count == 0) return MPL_OK;
  int tiles, unit, stages, ctas;
  int st = resolve(config, &tiles, &unit, &stages, &ctas);
  if (st != MPL_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  Args a;
  a.entries = (const Entry*)plan->workspace_dev;
  a.count = plan->count;
  a.status = device_status_ptr();
  a.tiles = (int32_t*)((char*)plan->workspace_dev + table_bytes(plan->count));
  if (tiles == 1) return launch_config(a, plan->precision, unit, stages, ctas, s);
  // one launch per width group, each after the prefix of its tile counts
  // (stream order keeps a group's prefix until its kernel has run)
  const bool f16 = plan->precision == MPL_F16;
  const int wps[3] = {64, 128, 256};
  int first = 0;
  for (int i = 0; i < 3; ++i) {
    const int n = plan->width_count[i];
    if (n < 0 || first + n > plan->count) return MPL_ERR_INVALID_ARG;
    if (n == 0) continue;
    Args g = a;
    g.entries = a.entries + first;
    g.count = n;
    batch_prefix_kernel<<<1, 1024, 0, s>>>(g);
    MPL_LAUNCH_CHECK();
    st = f16 ? launch_p_u32_f16(g, wps[i], ctas, s) : launch_p_u32_bf16(g, wps[i], ctas, s);
    if (st != MPL_OK) return st;
    first += n;
  }
  return first == plan->count ? MPL_OK : MPL_ERR_INVALID_ARG;
}

extern "C" int mpl_batch_autotune(const MplBatchPlan* plan, int32_t repeats, MplBatchConfig* best,
                                  float* best_ms, void* stream) {
  if (!plan || !best || repeats < 1) return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  // (tiles in flight, epilogue unit, weight stages)
  const int opts[5][3] = {{2, 32, 0}, {1, 16, 3}, {1, 16, 2}, {1, 32, 3}, {1, 32, 2}};
  cudaEvent_t e0, e1;
  MPL_CUDA_TRY(cudaEventCreate(&e0));
  MPL_CUDA_TRY(cudaEventCreate(&e1));
  float best_t = -1.f;
  MplBatchConfig pick;
  memset(&pick, 0, sizeof(pick));
  int st = MPL_OK;
  for (int oi = 0; oi < 5 && st == MPL_OK; ++oi) {
    {
      MplBatchConfig c;
      memset(&c, 0, sizeof(c));
      c.tiles_in_flight = opts[oi][0];
      c.epilogue_unit = opts[oi][1];
      c.stages = opts[oi][2];
      c.ctas = sm_count();
      st = mpl_batch_run(plan, &c, stream);  // warm-up
      if (st != MPL_OK) break;
      float ms_min = -1.f;
      for (int r = 0; r < repeats && st == MPL_OK; ++r) {
        if (cudaEventRecord(e0, s) != cudaSuccess) { st = MPL_ERR_CUDA; break; }
        st = mpl_batch_run(plan, &c, stream);
        if (st != MPL_OK) break;
        if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
          st = MPL_ERR_CUDA;
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms_min < 0.f || ms < ms_min) ms_min = ms;
      }
      if (st == MPL_OK && (best_t < 0.f || ms_min < best_t)) {
        best_t = ms_min;
        pick = c;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != MPL_OK) return st;
  *best = pick;
  if (best_ms) *best_ms = best_t;
  return MPL_OK;
}
