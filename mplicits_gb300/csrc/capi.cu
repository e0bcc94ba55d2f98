// extern "C" entry points of libmplicits: argument validation and dispatch.
#include <string.h>

#include <atomic>

#include "level.cuh"

namespace mpl {

__device__ int g_device_status = 0;

int* device_status_ptr() {
  // looked up once per device; concurrent first calls store the same address
  static std::atomic<int*> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  int* p = cached[dev].load(std::memory_order_acquire);
  if (!p) {
    void* q = nullptr;
    if (cudaGetSymbolAddress(&q, g_device_status) != cudaSuccess) return nullptr;
    p = (int*)q;
    cached[dev].store(p, std::memory_order_release);
  }
  return p;
}

static thread_local int t_last_cuda_error = 0;

void set_last_cuda_error(cudaError_t e) { t_last_cuda_error = (int)e; }

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!cached[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 148;
  }
  return cached[dev];
}

static int64_t g_opt_bf16_unit = 32;
static int64_t g_opt_tc_tiles = 2;
static int64_t g_opt_grad_reverse = 1;
static int64_t g_opt_layer0_warps = 8;

int64_t option_value(int32_t option) {
  switch (option) {
    case MPL_OPT_BF16_EPILOGUE_UNIT: return g_opt_bf16_unit;
    case MPL_OPT_TC_TILES_IN_FLIGHT: return g_opt_tc_tiles;
    case MPL_OPT_TC_GRAD_REVERSE: return g_opt_grad_reverse;
    case MPL_OPT_TC_LAYER0_WARPS: return g_opt_layer0_warps;
    default: return 0;
  }
}

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_set_option(int32_t option, int64_t value) {
  switch (option) {
    case MPL_OPT_BF16_EPILOGUE_UNIT:
      if (value != 16 && value != 32) return MPL_ERR_INVALID_ARG;
      g_opt_bf16_unit = value;
      return MPL_OK;
    case MPL_OPT_TC_TILES_IN_FLIGHT:
      if (value != 1 && value != 2) return MPL_ERR_INVALID_ARG;
      g_opt_tc_tiles = value;
      return MPL_OK;
    case MPL_OPT_TC_GRAD_REVERSE:
      if (value != 0 && value != 1) return MPL_ERR_INVALID_ARG;
      g_opt_grad_reverse = value;
      return MPL_OK;
    case MPL_OPT_TC_LAYER0_WARPS:
      if (value != 0 && value != 4 && value != 8) return MPL_ERR_INVALID_ARG;
      g_opt_layer0_warps = value;
      return MPL_OK;
    default:
      return MPL_ERR_INVALID_ARG;
  }
}

extern "C" int mpl_get_option(int32_t option, int64_t* value) {
  if (!value) return MPL_ERR_INVALID_ARG;
  if (option != MPL_OPT_BF16_EPILOGUE_UNIT && option != MPL_OPT_TC_TILES_IN_FLIGHT &&
      option != MPL_OPT_TC_GRAD_REVERSE && option != MPL_OPT_TC_LAYER0_WARPS)
    return MPL_ERR_INVALID_ARG;
  *value = option_value(option);
  return MPL_OK;
}

static int level_call(const MplNet* net, const void* packed, const MplPoints* points,
                      const int32_t* index, const int32_t* n_dev, int64_t n, float* S, float* G,
                      int32_t grad, int32_t store_mode, const MplBand* band, int32_t precision,
                      void* stream) {
  if (!net || !packed || !points || n < 0 || n > INT32_MAX) return MPL_ERR_INVALID_ARG;
  if (!S && (n > 0 || n_dev)) return MPL_ERR_INVALID_ARG;
  if (((uintptr_t)packed & 255) != 0) return MPL_ERR_INVALID_ARG;
  if (store_mode != MPL_STORE && store_mode != MPL_ACCUMULATE) return MPL_ERR_INVALID_ARG;
  if (points->kind == MPL_POINTS_XYZ) {
    if (!points->xyz && n > 0) return MPL_ERR_INVALID_ARG;
  } else if (points->kind == MPL_POINTS_GRID) {
    if (points->grid_n < 2) return MPL_ERR_INVALID_ARG;
    const int64_t N = points->grid_n;
    if (N * N * N > (int64_t)INT32_MAX + 1) return MPL_ERR_UNSUPPORTED;
  } else {
    return MPL_ERR_INVALID_ARG;
  }
  LevelArgs a;
  memset(&a, 0, sizeof(a));
  int st = make_layout(net, &a.lay);
  if (st != MPL_OK) return st;
  a.packed = (const char*)packed;
  for (int l = 0; l < MPL_MAX_LAYERS; ++l) a.omega[l] = net->omega[l];
  a.pts = *points;
  a.index = index;
  a.n_dev = n_dev;
  a.n = n;
  a.S = S;
  a.store_mode = store_mode;
  a.status = device_status_ptr();
  a.grad = grad;
  a.G = G;
  cudaStream_t s = (cudaStream_t)stream;
  if (band) {
    if (!band->out_index || !band->count_dev || band->capacity < 0) return MPL_ERR_INVALID_ARG;
    a.has_band = 1;
    a.band_delta = band->delta;
    a.band_lower = band->lower;
    a.band_out = band->out_index;
    a.band_count = band->count_dev;
    a.band_capacity = band->capacity;
    MPL_CUDA_TRY(cudaMemsetAsync(band->count_dev, 0, sizeof(int32_t), s));
  }
  if (n == 0) return MPL_OK;
  if (precision == MPL_FP32) return launch_level_fp32(a, s);
  if (precision == MPL_BF16) return launch_level_bf16(a, s);
  if (precision == MPL_F16) return launch_level_f16(a, s);
  return MPL_ERR_INVALID_ARG;
}

extern "C" int mpl_level_forward(const MplNet* net, const void* packed, const MplPoints* points,
                                 const int32_t* index, const int32_t* n_dev, int64_t n,
                                 float* S, int32_t store_mode, const MplBand* band,
                                 int32_t precision, void* stream) {
  return level_call(net, packed, points, index, n_dev, n, S, nullptr, 0, store_mode, band,
                    precision, stream);
}

extern "C" int mpl_level_gradient(const MplNet* net, const void* packed,
                                  const MplPoints* points, const int32_t* index,
                                  const int32_t* n_dev, int64_t n, float* S, float* G,
                                  int32_t store_mode, const MplBand* band, int32_t precision,
                                  void* stream) {
  if (!G && (n > 0 || n_dev)) return MPL_ERR_INVALID_ARG;
  return level_call(net, packed, points, index, n_dev, n, S, G, 1, store_mode, band, precision,
                    stream);
}

extern "C" const char* mpl_status_string(int status) {
  switch (status) {
    case MPL_OK: return "ok";
    case MPL_ERR_INVALID_ARG: return "invalid argument";
    case MPL_ERR_UNSUPPORTED: return "unsupported shape or mode";
    case MPL_ERR_CAPACITY: return "output capacity exceeded";
    case MPL_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case MPL_ERR_CUDA: return "CUDA runtime error";
    case MPL_ERR_NO_DEVICE: return "no suitable CUDA device";
    default: return "unknown status";
  }
}

extern "C" int mpl_last_cuda_error(void) { return t_last_cuda_error; }

extern "C" int mpl_abi_version(void) { return MPL_ABI_VERSION; }

// Reads and clears the device status word (synchronises the device).
extern "C" int mpl_device_status(int32_t* status_out) {
  if (!status_out) return MPL_ERR_INVALID_ARG;
  int v = 0;
  MPL_CUDA_TRY(cudaDeviceSynchronize());
  MPL_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_device_status, sizeof(int)));
  const int zero = 0;
  MPL_CUDA_TRY(cudaMemcpyToSymbol(g_device_status, &zero, sizeof(int)));
  *status_out = v;
  return MPL_OK;
}
