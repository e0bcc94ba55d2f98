// Weight packing: nn.Linear tensors -> the device image the level kernels
// read.  Replaces the per-layer CUTLASS tensors of the reference renderer
// (renderer/cuda/gemms.cu:5-100, loaded by tools.cu:81-111).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace mpl {

int make_layout(const MplNet* net, PackLayout* lay) {
  if (!net || !lay) return MPL_ERR_INVALID_ARG;
  const int L = net->n_layers;
  if (L < 2 || L > MPL_MAX_LAYERS) return MPL_ERR_UNSUPPORTED;
  if (net->dims[0] != 3 || net->dims[L] != 1) return MPL_ERR_UNSUPPORTED;
  int wmax = 0;
  for (int l = 1; l < L; ++l) {
    if (net->dims[l] < 1 || net->dims[l] > 256) return MPL_ERR_UNSUPPORTED;
    wmax = net->dims[l] > wmax ? net->dims[l] : wmax;
  }
  const int WP = wmax <= 64 ? 64 : (wmax <= 128 ? 128 : 256);
  lay->L = L;
  lay->WP = WP;
  lay->nh = L - 2;
  int64_t o = 0;
  auto take = [&](int64_t bytes) {
    int64_t at = o;
    o = align256(o + bytes);
    return at;
  };
  lay->w0t = take(3 * WP * 4);
  lay->b0 = take(WP * 4);
  for (int l = 0; l < MPL_MAX_LAYERS; ++l) {
    lay->wht[l] = lay->bh[l] = lay->hb[l] = lay->hw[l] = lay->hwT[l] = lay->hbx[l] = -1;
    lay->hwh[l] = lay->hbxh[l] = lay->whn[l] = lay->hwTh[l] = -1;
  }
  for (int l = 1; l <= L - 2; ++l) {
    lay->wht[l] = take((int64_t)WP * WP * 4);
    lay->bh[l] = take(WP * 4);
  }
  lay->wout = take(WP * 4);
  lay->bout = take(16);
  lay->w0f = take(WP * 16);
  for (int l = 1; l <= L - 2; ++l) {
    lay->hb[l] = take(WP * 4);
    lay->hw[l] = take((int64_t)WP * WP * 2);
    lay->hwT[l] = take((int64_t)WP * WP * 2);
    lay->hbx[l] = take((int64_t)WP * 16 * 2);
    lay->hwh[l] = take((int64_t)WP * WP * 2);
    lay->hbxh[l] = take((int64_t)WP * 16 * 2);
    lay->whn[l] = take((int64_t)WP * WP * 4);
    lay->hwTh[l] = take((int64_t)WP * WP * 2);
  }
  lay->total = o;
  return MPL_OK;
}

// offset (in elements) of (row n, col k) in the K-chunked core-matrix tiling
__device__ __forceinline__ int64_t umma_tile_offset(int n, int k, int WP) {
  const int c = k >> 6, kk = k & 63;
  return (int64_t)c * WP * 64 + ((int64_t)(n >> 3) * 8 + (kk >> 3)) * 64 + (n & 7) * 8 + (k & 7);
}

__global__ void pack_layer0(const float* __restrict__ W, const float* __restrict__ b, int out,
                            int WP, float omega, float* w0t, float* b0, float* w0f) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= WP) return;
  const bool v = j < out;
  for (int c = 0; c < 3; ++c) {
    float w = v ? W[j * 3 + c] : 0.f;
    w0t[c * WP + j] = w;
    w0f[c * WP + j] = omega * w;
  }
  float bb = v ? b[j] : 0.f;
  b0[j] = bb;
  w0f[3 * WP + j] = omega * bb;
}

__global__ void pack_hidden(const float* __restrict__ W, const float* __restrict__ b, int out,
                            int in, int WP, float omega, float* wt, float* bh, float* hb,
                            __nv_bfloat16* hw, __nv_bfloat16* hwT, __half* hwh, float* whn,
                            __half* hwTh) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)WP * WP) return;
  const int n = (int)(e / WP), k = (int)(e % WP);  // n: output row, k: input col
  const float w = (n < out && k < in) ? W[(int64_t)n * in + k] : 0.f;
  wt[(int64_t)k * WP + n] = w;
  whn[(int64_t)n * WP + k] = w;
  hw[umma_tile_offset(n, k, WP)] = __float2bfloat16_rn(omega * w);
  hwT[umma_tile_offset(k, n, WP)] = __float2bfloat16_rn(omega * w);
  hwh[umma_tile_offset(n, k, WP)] = __float2half_rn(omega * w);
  hwTh[umma_tile_offset(k, n, WP)] = __float2half_rn(omega * w);
  if (k == 0) {
    const float bb = n < out ? b[n] : 0.f;
    bh[n] = bb;
    hb[n] = omega * bb;
  }
}

// bias tile of the MMA (see PackLayout::hbx): row n, K columns 0 and 1
__global__ void pack_bias_tile(const float* __restrict__ b, int out, int WP, float omega,
                               __nv_bfloat16* hbx, __half* hbxh) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= WP) return;
  const float v = n < out ? omega * b[n] : 0.f;
  const int base = ((n >> 3) * 2) * 64 + (n & 7) * 8;  // elements; K group 0
  for (int k = 0; k < 8; ++k) {
    hbx[base + k] = hbx[base + 64 + k] = __float2bfloat16_rn(0.f);
    hbxh[base + k] = hbxh[base + 64 + k] = __float2half_rn(0.f);
  }
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  hbx[base + 0] = hi;
  hbx[base + 1] = __float2bfloat16_rn(v - __bfloat162float(hi));
  const __half hh = __float2half_rn(v);
  hbxh[base + 0] = hh;
  hbxh[base + 1] = __float2half_rn(v - __half2float(hh));
}

__global__ void pack_output(const float* __restrict__ W, const float* __restrict__ b, int in,
                            int WP, float* wout, float* bout) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < WP) wout[j] = j < in ? W[j] : 0.f;
  if (j == 0) {
    bout[0] = b[0];
    bout[1] = bout[2] = bout[3] = 0.f;
  }
}

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_net_packed_bytes(const MplNet* net, int64_t* bytes) {
  if (!bytes) return MPL_ERR_INVALID_ARG;
  PackLayout lay;
  int st = make_layout(net, &lay);
  if (st != MPL_OK) return st;
  *bytes = lay.total;
  return MPL_OK;
}

extern "C" int mpl_net_pack(const MplNet* net, const float* const* weights,
                            const float* const* biases, void* packed, void* stream) {
  PackLayout lay;
  int st = make_layout(net, &lay);
  if (st != MPL_OK) return st;
  if (!weights || !biases || !packed) return MPL_ERR_INVALID_ARG;
  if (((uintptr_t)packed & 255) != 0) return MPL_ERR_INVALID_ARG;
  for (int l = 0; l < lay.L; ++l)
    if (!weights[l] || !biases[l]) return MPL_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  char* base = (char*)packed;
  MPL_CUDA_TRY(cudaMemsetAsync(packed, 0, lay.total, s));
  const int WP = lay.WP;
  pack_layer0<<<(WP + 127) / 128, 128, 0, s>>>(weights[0], biases[0], net->dims[1], WP,
                                                net->omega[0], (float*)(base + lay.w0t),
                                                (float*)(base + lay.b0), (float*)(base + lay.w0f));
  MPL_LAUNCH_CHECK();
  for (int l = 1; l <= lay.L - 2; ++l) {
    const int64_t n = (int64_t)WP * WP;
    pack_hidden<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        weights[l], biases[l], net->dims[l + 1], net->dims[l], WP, net->omega[l],
        (float*)(base + lay.wht[l]), (float*)(base + lay.bh[l]), (float*)(base + lay.hb[l]),
        (__nv_bfloat16*)(base + lay.hw[l]), (__nv_bfloat16*)(base + lay.hwT[l]),
        (__half*)(base + lay.hwh[l]), (float*)(base + lay.whn[l]),
        (__half*)(base + lay.hwTh[l]));
    MPL_LAUNCH_CHECK();
    pack_bias_tile<<<(WP + 127) / 128, 128, 0, s>>>(biases[l], net->dims[l + 1], WP,
                                                    net->omega[l],
                                                    (__nv_bfloat16*)(base + lay.hbx[l]),
                                                    (__half*)(base + lay.hbxh[l]));
    MPL_LAUNCH_CHECK();
  }
  pack_output<<<(WP + 127) / 128, 128, 0, s>>>(weights[lay.L - 1], biases[lay.L - 1],
                                                net->dims[lay.L - 1], WP,
                                                (float*)(base + lay.wout),
                                                (float*)(base + lay.bout));
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
