// BF16 fused level evaluator on the 5th-generation tensor cores (sm_103a):
// the kernel template, instantiated for two epilogue unit widths by
// level_bf16_u16.cu and level_bf16_u32.cu.
//
// One persistent CTA per SM walks 128-point tiles.  Per tile:
//   layer 0      FP32 SIMT: z = omega0*(W0 x + b0) stays in FP32 (omega0
//                amplifies phase error), sin, BF16 -> A operand in smem;
//   hidden l     tcgen05.mma (kind::f16, BF16 in, FP32 accumulate) of
//                A[128 x WP] by omega_l*W_l^T into a TMEM accumulator;
//                the epilogue reads TMEM (tcgen05.ld), adds omega_l*b_l,
//                takes sin in FP32 and writes the next A operand;
//   output       FP32 dot product with W_L of the FP32 sines + b_L, then the
//                store/accumulate into S and the fused band compaction.
// The A operand is produced in 64-feature chunks and each chunk is handed to
// the MMA issuer through its own mbarrier, so the GEMM of layer l+1 starts
// while the epilogue of layer l is still running; two TMEM accumulators
// alternate between consecutive GEMMs.  Hidden-layer weights stream from L2
// in 64-row K chunks through a ring of shared-memory stages filled by the
// TMA engine (cp.async.bulk).  Roles:
//   epilogue   4*Q warps (Q = 64/U): warp w owns TMEM lanes 32*(w%4)..
//              (its 32 rows) and features h*U..h*U+U-1 (h = w/4) of every
//              64-feature chunk;
//   MMA warp   TMEM allocation and the single MMA-issuing thread;
//   TMA warp   the single TMA-issuing thread.
// GRAD mode returns df/dx as well, by forward-mode differentiation: the 128
// rows of a tile are 32 points x (value, d/dx, d/dy, d/dz); TMEM lane m holds
// row m, the four rows of a point sit in four adjacent lanes of one warp, the
// value row's pre-activation z reaches the tangent lanes by a shuffle and a
// tangent row becomes cos(z) * (omega W t) = sin(z + pi/2) * (omega W t).
// Every wait is bounded (mbar_wait_abort); a wait that gives up records
// MPL_ERR_DEVICE_TIMEOUT, raises the CTA's abort flag, and every role leaves
// its loop, drains its outstanding copies/MMAs and frees TMEM.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "level.cuh"
#include "tc.cuh"

namespace mpl {
namespace bf16 {

constexpr int kM = 128;  // points per tile = MMA M = TMEM lanes
constexpr int kKC = 64;  // K per weight stage and per A chunk
constexpr int kMaxNC = 4;

// Epilogue geometry for a unit width U (features a warp handles per 64-wide
// chunk): Q = 64/U warps share each TMEM lane quadrant, 4*Q epilogue warps
// in all, then one MMA-issuing warp and one TMA warp.
template <int U>
struct Epi {
  static constexpr int kQ = 64 / U;
  static constexpr int kWarps = 4 * kQ;
  static constexpr int kMmaWarp = kWarps;
  static constexpr int kTmaWarp = kWarps + 1;
  static constexpr int kThreads = (kWarps + 2) * 32;
};

template <int WP, int STAGES, int U>
struct Bf16Cfg {
  static constexpr int NC = WP / kKC;  // K chunks per GEMM
  static constexpr int kStages = STAGES;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t kTmemCols = WP == 64 ? 128 : (WP == 128 ? 256 : 512);
  // shared-memory offsets (bytes)
  static constexpr uint32_t oA = 0;
  static constexpr uint32_t oW = kABytes;
  static constexpr uint32_t oW0 = oW + kStages * kStageBytes;  // float4 [WP]
  static constexpr uint32_t oWout = oW0 + WP * 16;             // float [WP]
  static constexpr uint32_t oRed = oWout + WP * 4;             // float [2][Q-1][128]
  static constexpr uint32_t oBar = oRed + 2 * (64 / U - 1) * kM * 4;  // barriers
  static constexpr uint32_t kNumBars = 2 * kStages + kMaxNC + 2 + 2 + 4 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;       // tmem slot, abort flag
  // MMA operand tiles start on 1 KiB boundaries (descriptors drop 4 address bits)
  static constexpr uint32_t oAx = (oMisc + 16 + 1023) & ~1023u;  // bf16 [128][16] ones tile
  static constexpr uint32_t oBx = oAx + kM * 16 * 2;             // bf16 [nh][WP][16] bias tiles
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  static size_t bytes(int nh) { return oBx + (size_t)nh * kBxBytes; }
};

// sin through the hardware approximation.  The unit reduces its argument
// itself after a float32 multiply by 1/(2 pi), so for the phases of these
// networks (|z| <~ 60) the absolute error stays near 1e-6, three orders below
// the BF16 rounding of the activations it feeds.  The two-argument form adds
// `phase` first (pi/2 for a cosine); the one-argument form has no add, since
// z + 0.f cannot be folded away (it turns -0 into +0).
__device__ __forceinline__ float sin_fast(float z) { return __sinf(z); }
__device__ __forceinline__ float sin_fast(float z, float phase) { return __sinf(z + phase); }

// Bounded wait: the thread sleeps in hardware between polls (up to 20 us a
// poll), leaves early when another role raised the abort flag, and gives up
// after limit_ns of wall time (kWaitLimitNs in the kernels; the wait
// self-test passes a shorter one), recording MPL_ERR_DEVICE_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, int* status,
                                                volatile int* abort_flag,
                                                uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
    if ((i & 7) == 0) {
      if (*abort_flag) return false;
      if (global_timer_ns() - t0 > limit_ns) break;
    }
  }
  report_device_error(status, MPL_ERR_DEVICE_TIMEOUT);
  *abort_flag = 1;
  return false;
}

// OR of `fail` over the epilogue warps at named barrier 1 (every epilogue
// thread calls it the same number of times); orders their memory accesses
// like a CTA barrier, so all of them leave a loop together.
__device__ __forceinline__ bool epi_any(bool fail, int nthreads) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)fail), "r"(nthreads)
      : "memory");
  return r != 0;
}

// warp-uniform bounded wait (all lanes poll; any failure fails the warp)
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* status,
                                          volatile int* abort_flag) {
  const bool ok = mbar_wait_abort(bar, parity, status, abort_flag);
  return __all_sync(0xffffffffu, ok);
}

// A operand tile [128 x WP] bf16, K-major core matrices, layout
// [k/8][m/8][m%8][k%8]: LBO (next 8 K) = 2048 B, SBO (next 8 rows) = 128 B.
// The two 16-bit operand types of kind::f16 (A and B always share one).
template <typename T>
struct Operand;
template <>
struct Operand<__nv_bfloat16> {
  static constexpr uint32_t kFormat = 1;
  __device__ static uint32_t pack(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
  }
  __device__ static __nv_bfloat16 value(float f) { return __float2bfloat16_rn(f); }
};
template <>
struct Operand<__half> {
  static constexpr uint32_t kFormat = 0;
  __device__ static uint32_t pack(float lo, float hi) {
    __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
  }
  __device__ static __half value(float f) { return __float2half_rn(f); }
};

template <typename T, int U>
__device__ __forceinline__ void store_a_unit(uint8_t* sA, int m, int j0, const float (&v)[U]) {
#pragma unroll
  for (int g = 0; g < U / 8; ++g) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = Operand<T>::pack(v[g * 8 + 2 * i], v[g * 8 + 2 * i + 1]);
    const int k8 = (j0 >> 3) + g;
    const uint32_t off = (uint32_t)((k8 * 16 + (m >> 3)) * 128 + (m & 7) * 16);
    *reinterpret_cast<uint4*>(sA + off) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Paired FP32 arithmetic (sm_100 family): two IEEE fma.rn in one
// instruction, so results equal the scalar form bit for bit.
__device__ __forceinline__ uint64_t f2pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// Four consecutive weights of the first-layer image: from shared memory, or
// (GW) through the read-only path of global memory.
template <bool GW>
__device__ __forceinline__ float4 w0_load4(const float* p) {
  if (GW) return __ldg(reinterpret_cast<const float4*>(p));
  return *reinterpret_cast<const float4*>(p);
}

// First-layer phases z_j = omega0 (W0 x + b0)_j of features j..j+3 for one
// point, evaluated as fma(x, wx, fma(y, wy, fma(z, wz, wb))) two features at
// a time.  w0s is the [4][stride] image (rows: omega0 W0[:, 0..2], omega0 b0)
// in shared memory, or in global memory when GW; the x, y, z weights are
// returned for the tangent rows.
template <bool GW = false>
__device__ __forceinline__ void phase4(const float* w0s, int stride, int j, float x, float y,
                                       float z, float (&zz)[4], float4& wx, float4& wy,
                                       float4& wz) {
  wx = w0_load4<GW>(w0s + j);
  wy = w0_load4<GW>(w0s + stride + j);
  wz = w0_load4<GW>(w0s + 2 * stride + j);
  const float4 wb = w0_load4<GW>(w0s + 3 * stride + j);
  const uint64_t X = f2pack(x, x), Y = f2pack(y, y), Z = f2pack(z, z);
  const uint64_t a = ffma2(X, f2pack(wx.x, wx.y),
                           ffma2(Y, f2pack(wy.x, wy.y), ffma2(Z, f2pack(wz.x, wz.y),
                                                              f2pack(wb.x, wb.y))));
  const uint64_t b = ffma2(X, f2pack(wx.z, wx.w),
                           ffma2(Y, f2pack(wy.z, wy.w), ffma2(Z, f2pack(wz.z, wz.w),
                                                              f2pack(wb.z, wb.w))));
  f2unpack(a, zz[0], zz[1]);
  f2unpack(b, zz[2], zz[3]);
}

// Layer 0 of one U-feature unit (features j0..j0+U-1) for this thread's row:
// FP32 phase omega0*(W0 x + b0) (omega folded into w0s), sine, 16-bit into
// the A operand.  GRAD: tangent row ch gets cos(z) * omega0*W0[:, ch-1].
// GW: w0s lives in global memory.
template <typename T, bool GRAD, int U, bool GW = false>
__device__ __forceinline__ void layer0_unit(uint8_t* sA, const float* w0s, int stride, int m,
                                            int j0, int ch, float phase, float x, float y,
                                            float z) {
  float v[U];
#pragma unroll
  for (int j4 = 0; j4 < U / 4; ++j4) {
    float zz[4];
    float4 wx, wy, wz;
    phase4<GW>(w0s, stride, j0 + 4 * j4, x, y, z, zz, wx, wy, wz);
    const float ax[4] = {wx.x, wx.y, wx.z, wx.w};
    const float ay[4] = {wy.x, wy.y, wy.z, wy.w};
    const float az[4] = {wz.x, wz.y, wz.z, wz.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (GRAD) {
        const float dz = ch == 1 ? ax[i] : (ch == 2 ? ay[i] : az[i]);
        const float sc = sin_fast(zz[i], phase);
        v[4 * j4 + i] = ch ? __fmul_rn(sc, dz) : sc;
      } else {
        v[4 * j4 + i] = sin_fast(zz[i]);
      }
    }
  }
  store_a_unit<T, U>(sA, m, j0, v);
}

template <int WP, bool GRAD, int STAGES, int U, typename T>
__global__ void __launch_bounds__(Epi<U>::kThreads, 1) level_bf16_kernel(const LevelArgs a) {
  using C = Bf16Cfg<WP, STAGES, U>;
  using E = Epi<U>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int PT = GRAD ? kM / 4 : kM;  // points per tile
  constexpr int NC = C::NC;
  constexpr int S = C::kStages;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Operand<T>::kFormat);
  constexpr bool kF16 = Operand<T>::kFormat == 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  float* w0s = reinterpret_cast<float*>(smem + C::oW0);  // [4][WP]
  float* wout = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;            // [S]   TMA -> MMA
  uint64_t* wempty = bars + S;       // [S]   MMA -> TMA
  uint64_t* achunk = bars + 2 * S;   // [NC]  epilogue -> MMA (count: epilogue warps)
  uint64_t* dfull = achunk + kMaxNC; // [2]   MMA -> epilogue
  uint64_t* dempty = dfull + 2;      // [2]   epilogue -> MMA (count: epilogue warps)
  uint64_t* redfull = dempty + 2;    // [2]   h > 0 warps -> h = 0 warps (count 4(Q-1))
  uint64_t* redfree = redfull + 2;   // [2]   h = 0 warps -> h > 0 warps (count 4)
  uint64_t* finalb = redfree + 2;    // [1]   last MMA commit
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  uint8_t* sAx = smem + C::oAx;  // ones tile: K columns 0, 1 of bias-carrying rows
  uint8_t* sBx = smem + C::oBx;  // per hidden layer: bias tile

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nh = a.lay.nh;
  const int64_t n = level_point_count(a);
  const int64_t ntiles = (n + PT - 1) / PT;
  if ((int64_t)blockIdx.x >= ntiles) return;

  // ---- set-up: barriers, TMEM, constants
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    for (int c = 0; c < kMaxNC; ++c) mbar_init(&achunk[c], kEpiWarps);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&dfull[b], 1);
      mbar_init(&dempty[b], kEpiWarps);
      mbar_init(&redfull[b], 4 * (Q - 1));
      mbar_init(&redfree[b], 4);
    }
    mbar_init(finalb, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tmem_slot, C::kTmemCols);
  const char* pk = a.packed;
  {
    const float4* g0 = reinterpret_cast<const float4*>(pk + a.lay.w0f);
    for (int i = threadIdx.x; i < WP; i += kThreads) {
      reinterpret_cast<float4*>(w0s)[i] = g0[i];
      wout[i] = reinterpret_cast<const float*>(pk + a.lay.wout)[i];
    }
    for (int l = 1; l <= nh; ++l) {
      const uint4* gb = reinterpret_cast<const uint4*>(pk + (kF16 ? a.lay.hbxh[l] : a.lay.hbx[l]));
      uint4* db = reinterpret_cast<uint4*>(sBx + (l - 1) * C::kBxBytes);
      for (int i = threadIdx.x; i < (int)(C::kBxBytes / 16); i += kThreads) db[i] = gb[i];
    }
    // ones tile, layout of the A operand ([k/8][m/8][m%8][k%8]); in GRAD mode
    // only value rows (m % 4 == 0) carry the bias
    for (int i = threadIdx.x; i < kM * 16; i += kThreads) {
      const int m = i >> 4, k = i & 15;
      const bool one = k < 2 && (!GRAD || (m & 3) == 0);
      const uint32_t off = (uint32_t)(((k >> 3) * 16 + (m >> 3)) * 128 + (m & 7) * 16 + (k & 7) * 2);
      *reinterpret_cast<T*>(sAx + off) = Operand<T>::value(one ? 1.f : 0.f);
    }
    fence_proxy_async_smem();
  }
  const float bout = reinterpret_cast<const float*>(pk + a.lay.bout)[0];
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == kTmaWarp) {
    // ================= TMA producer: hidden-layer weight K chunks =========
    if (lane == 0) {
      int64_t w = 0;
      for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        for (int l = 1; l <= nh && !*abort_flag; ++l) {
          const char* src = pk + (kF16 ? a.lay.hwh[l] : a.lay.hw[l]);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            const int64_t u = w / S;
            if (u > 0 && !mbar_wait_abort(&wempty[s], (uint32_t)((u - 1) & 1), a.status,
                                          abort_flag))
              break;
            mbar_arrive_expect_tx(&wfull[s], C::kStageBytes);
            tma_bulk_g2s(sW + s * C::kStageBytes, src + (size_t)c * C::kStageBytes,
                         C::kStageBytes, &wfull[s]);
          }
        }
      }
      // copies still in flight must land before the CTA can exit: the last
      // S issued chunks are the only ones that can be outstanding
      const int64_t first = w > S ? w - S : 0;
      for (int64_t v = first; v < w; ++v)
        mbar_wait(&wfull[v % S], (uint32_t)((v / S) & 1), a.status);
    }
  } else if (warp == kMmaWarp) {
    // ================= MMA issuer ==========================================
    if (lane == 0) {
      // descriptor bases; an operand at byte offset o adds o >> 4 (the start
      // address field, which stays below 2^14 inside shared memory)
      const uint64_t aDesc = tc::smem_desc(smem_u32(sA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      int64_t w = 0, g = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int l = 1; l <= nh && ok; ++l, ++g) {
          // GEMM g uses accumulator g & 1, whose earlier uses number g >> 1
          const int b = (int)(g & 1);
          if (g >= 2 &&
              !mbar_wait_abort(&dempty[b], (uint32_t)(((g >> 1) - 1) & 1), a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(b * WP);
          // D = bias (ones tile x bias tile), then D += A * W^T chunk by chunk
          tc::mma_bf16(d_tmem, xDesc,
                       tc::smem_desc(smem_u32(sBx) + (uint32_t)(l - 1) * C::kBxBytes, 128u, 256u),
                       IDESC, false);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            if (!mbar_wait_abort(&achunk[c], (uint32_t)(g & 1), a.status, abort_flag) ||
                !mbar_wait_abort(&wfull[s], (uint32_t)((w / S) & 1), a.status, abort_flag)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const uint64_t aC = aDesc + (uint64_t)((c * 8 * 2048) >> 4);
            const uint64_t wC = wDesc + (uint64_t)((s * C::kStageBytes) >> 4);
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks)
              tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                           wC + (uint64_t)((ks * 256) >> 4), IDESC, true);
            tc::commit(&wempty[s]);
          }
          if (!ok) break;
          tc::commit(&dfull[b]);
        }
      }
      // every MMA issued so far must complete before TMEM is released
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else {
    // ================= epilogue warps =====================================
    const int q = warp & 3, h = warp >> 2;
    const int m = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    // GRAD: row m is channel ch of point m/4 (ch 0: value, 1..3: d/dx_(ch-1))
    const int ch = GRAD ? (m & 3) : 0;
    const int vlane = lane & ~3;
    const float phase = ch ? 1.57079632679489662f : 0.f;
    int64_t g = 0, tloc = 0;
    bool ok = true;
    // Software pipeline over tiles: layer 0 of tile t+1 is computed chunk by
    // chunk inside the last drain of tile t (the A operand is free once the
    // last GEMM of t has completed), so GEMM 1 of t+1 runs on the tensor
    // cores while the output layer of t is still being reduced.
    const int prow = GRAD ? (m >> 2) : m;  // this row's point within the tile
    int64_t p = -1;
    float x = 0.f, y = 0.f, z = 0.f;
    {
      const int64_t qi = (int64_t)blockIdx.x * PT + prow;
      if (qi < n) load_point(a, qi, p, x, y, z);
    }
#pragma unroll 1
    for (int c = 0; c < NC; ++c) {
      layer0_unit<T, GRAD, U>(sA, w0s, WP, m, c * kKC + h * U, ch, phase, x, y, z);
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&achunk[c]);
    }
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tloc) {
      const int64_t tn = t + gridDim.x;  // next tile of this CTA
      const bool has_next = tn < ntiles;
      int64_t pn = -1;
      float xn = 0.f, yn = 0.f, zn = 0.f;

      float part = 0.f;
      for (int l = 1; l <= nh; ++l, ++g) {
        const int b = (int)(g & 1);
        if (!warp_wait(&dfull[b], (uint32_t)((g >> 1) & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        if (l == nh && has_next) {
          // point of the next tile, first needed by its layer 0 inside this
          // last drain
          const int64_t qn = tn * PT + prow;
          if (qn < n) load_point(a, qn, pn, xn, yn, zn);
        }
        const uint32_t taddr = tl + (uint32_t)(b * WP);
        // two TMEM loads in flight per wait
#pragma unroll 1
        for (int c0 = 0; c0 < NC; c0 += 2) {
          uint32_t r2[2][U];
          tc::ld_32x32b<U>(taddr + (uint32_t)(c0 * kKC + h * U), r2[0]);
          if (c0 + 1 < NC) tc::ld_32x32b<U>(taddr + (uint32_t)((c0 + 1) * kKC + h * U), r2[1]);
          tc::wait_ld();
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int c = c0 + u;
            if (c >= NC) break;
            const int j0 = c * kKC + h * U;
            uint32_t (&r)[U] = r2[u];
            if (GRAD) {
              // value pre-activation of this point to its tangent lanes
#pragma unroll
              for (int jj = 0; jj < U; ++jj) {
                const float acc = __uint_as_float(r[jj]);
                const float zz = __shfl_sync(0xffffffffu, acc, vlane);
                const float sc = sin_fast(zz, phase);
                r[jj] = __float_as_uint(ch ? __fmul_rn(sc, acc) : sc);
              }
            }
            if (l < nh) {
              float v[U];
#pragma unroll
              for (int jj = 0; jj < U; ++jj)
                v[jj] = GRAD ? __uint_as_float(r[jj]) : sin_fast(__uint_as_float(r[jj]));
              store_a_unit<T, U>(sA, m, j0, v);
              fence_proxy_async_smem();
              __syncwarp();
              if (lane == 0) mbar_arrive(&achunk[c]);
            } else {
              const float4* wo4 = reinterpret_cast<const float4*>(wout + j0);
#pragma unroll
              for (int j4 = 0; j4 < U / 4; ++j4) {
                const float4 wv = wo4[j4];
                const float wa[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const float acc = __uint_as_float(r[4 * j4 + i]);
                  const float sv = GRAD ? acc : sin_fast(acc);
                  part = __fmaf_rn(sv, wa[i], part);
                }
              }
              if (has_next) {
                layer0_unit<T, GRAD, U>(sA, w0s, WP, m, j0, ch, phase, xn, yn, zn);
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&achunk[c]);
              }
            }
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&dempty[b]);
      }
      if (!ok) break;

      // combine the feature splits, store, band
      const int rb = (int)(tloc & 1);
      if (h > 0) {
        if (tloc >= 2 && !warp_wait(&redfree[rb], (uint32_t)(((tloc >> 1) - 1) & 1), a.status,
                                    abort_flag)) {
          ok = false;
          break;
        }
        red[(rb * (Q - 1) + (h - 1)) * kM + m] = part;
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfull[rb]);
      } else {
        if (!warp_wait(&redfull[rb], (uint32_t)((tloc >> 1) & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        float sum = part;
#pragma unroll
        for (int hh = 0; hh < Q - 1; ++hh) sum = __fadd_rn(sum, red[(rb * (Q - 1) + hh) * kM + m]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfree[rb]);
        if (GRAD) {
          if (ch && p >= 0 && a.G) {
            float* gp = a.G + 3 * p + (ch - 1);
            *gp = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(*gp, sum) : sum;
          }
          store_and_band(a, p >= 0 && ch == 0, p, __fadd_rn(sum, bout));
        } else {
          store_and_band(a, p >= 0, p, __fadd_rn(sum, bout));
        }
      }
      p = pn;
    }
  }

  // ---- teardown: all roles have left their loops; release TMEM
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, bool GRAD, int STAGES, int U, typename T>
int launch_cfg(const LevelArgs& a, cudaStream_t s) {
  using C = Bf16Cfg<WP, STAGES, U>;
  constexpr int PT = GRAD ? kM / 4 : kM;
  const size_t smem = C::bytes(a.lay.nh);
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_bf16_kernel<WP, GRAD, STAGES, U, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + PT - 1) / PT;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_bf16_kernel<WP, GRAD, STAGES, U, T><<<(unsigned)grid, Epi<U>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// the deepest weight ring that fits the shared memory next to this level's
// bias tiles
template <int WP, bool GRAD, int U, typename T>
int launch_wp(const LevelArgs& a, cudaStream_t s) {
  constexpr size_t kLimit = 227 * 1024;
  constexpr int SHI = WP == 256 ? 4 : 6;
  if (Bf16Cfg<WP, SHI, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, SHI, U, T>(a, s);
  if (Bf16Cfg<WP, 3, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 3, U, T>(a, s);
  if (Bf16Cfg<WP, 2, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 2, U, T>(a, s);
  return MPL_ERR_UNSUPPORTED;
}

template <int U, typename T>
int launch_unit(const LevelArgs& a, cudaStream_t s) {
  switch (a.lay.WP) {
    case 64: return a.grad ? launch_wp<64, true, U, T>(a, s) : launch_wp<64, false, U, T>(a, s);
    case 128: return a.grad ? launch_wp<128, true, U, T>(a, s) : launch_wp<128, false, U, T>(a, s);
    case 256: return a.grad ? launch_wp<256, true, U, T>(a, s) : launch_wp<256, false, U, T>(a, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace bf16
}  // namespace mpl
