// Host side of the batched launch: plan preparation (entry table on the
// device), the launch itself (graph-capturable: one kernel, no host sync),
// and the autotuner that picks the epilogue unit width and the weight-ring
// depth by timing the real plan.
#include <string.h>

#include <vector>

#include "batch_launch.h"

namespace mpl {
namespace batch {

static size_t table_bytes(int32_t count) {
  return ((size_t)count * sizeof(Entry) + 255) & ~(size_t)255;
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

static int resolve(const MplBatchConfig* cfg, int* unit, int* stages, int* ctas) {
  *unit = cfg && cfg->epilogue_unit ? cfg->epilogue_unit : 16;
  *stages = cfg && cfg->stages ? cfg->stages : 3;
  *ctas = cfg && cfg->ctas > 0 ? cfg->ctas : sm_count();
  if ((*unit != 16 && *unit != 32) || (*stages != 2 && *stages != 3) || *ctas <= 0)
    return MPL_ERR_INVALID_ARG;
  return MPL_OK;
}

}  // namespace batch
}  // namespace mpl

using namespace mpl;
using namespace mpl::batch;

extern "C" int mpl_batch_workspace_bytes(int32_t count, int64_t* bytes) {
  if (!bytes || count < 0 || count > kMaxEntries) return MPL_ERR_INVALID_ARG;
  *bytes = (int64_t)table_bytes(count);
  return MPL_OK;
}

extern "C" int mpl_batch_prepare(const MplBatchEntry* entries, int32_t count, int32_t precision,
                                 void* workspace, int64_t workspace_bytes, MplBatchPlan* plan,
                                 void* stream) {
  if (!plan || count < 0 || count > kMaxEntries || (count > 0 && (!entries || !workspace)))
    return MPL_ERR_INVALID_ARG;
  if (precision != MPL_BF16 && precision != MPL_F16) return MPL_ERR_UNSUPPORTED;
  if ((int64_t)table_bytes(count) > workspace_bytes) return MPL_ERR_CAPACITY;
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
  return MPL_OK;
}

extern "C" int mpl_batch_run(const MplBatchPlan* plan, const MplBatchConfig* config,
                             void* stream) {
  if (!plan || plan->count < 0 || plan->count > kMaxEntries) return MPL_ERR_INVALID_ARG;
  if (plan->count == 0) return MPL_OK;
  int unit, stages, ctas;
  int st = resolve(config, &unit, &stages, &ctas);
  if (st != MPL_OK) return st;
  Args a;
  a.entries = (const Entry*)plan->workspace_dev;
  a.count = plan->count;
  a.status = device_status_ptr();
  return launch_config(a, plan->precision, unit, stages, ctas, (cudaStream_t)stream);
}

extern "C" int mpl_batch_autotune(const MplBatchPlan* plan, int32_t repeats, MplBatchConfig* best,
                                  float* best_ms, void* stream) {
  if (!plan || !best || repeats < 1) return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int units[2] = {16, 32};
  const int stage_opts[2] = {3, 2};
  cudaEvent_t e0, e1;
  MPL_CUDA_TRY(cudaEventCreate(&e0));
  MPL_CUDA_TRY(cudaEventCreate(&e1));
  float best_t = -1.f;
  MplBatchConfig pick;
  memset(&pick, 0, sizeof(pick));
  int st = MPL_OK;
  for (int ui = 0; ui < 2 && st == MPL_OK; ++ui) {
    for (int si = 0; si < 2 && st == MPL_OK; ++si) {
      MplBatchConfig c;
      memset(&c, 0, sizeof(c));
      c.epilogue_unit = units[ui];
      c.stages = stage_opts[si];
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
