// BF16 fused level evaluator on the 5th-generation tensor cores (sm_103a).
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
//   warps 0-7  epilogue: warp w owns TMEM lanes 32*(w%4).. (its 32 points)
//              and the feature half w/4 of every 64-feature chunk;
//   warp 8     TMEM allocation and the single MMA-issuing thread;
//   warp 9     the single TMA-issuing thread.
// GRAD mode returns df/dx as well, by forward-mode differentiation: the 128
// rows of a tile are 32 points x (value, d/dx, d/dy, d/dz); TMEM lane m holds
// row m, the four rows of a point sit in four adjacent lanes of one warp, the
// value row's pre-activation z reaches the tangent lanes by a shuffle and a
// tangent row becomes cos(z) * (omega W t) = sin(z + pi/2) * (omega W t).
// Every wait is bounded (mbar_wait_abort); a wait that gives up records
// MPL_ERR_DEVICE_TIMEOUT, raises the CTA's abort flag, and every role leaves
// its loop, drains its outstanding copies/MMAs and frees TMEM.
#include <cuda_bf16.h>

#include "level.cuh"
#include "tc.cuh"

namespace mpl {

namespace {

constexpr int kM = 128;  // points per tile = MMA M = TMEM lanes
constexpr int kKC = 64;  // K per weight stage and per A chunk
constexpr int kEpiWarps = 8;
constexpr int kMmaWarp = 8;
constexpr int kTmaWarp = 9;
constexpr int kThreads = 320;
constexpr int kMaxNC = 4;

template <int WP>
struct Bf16Cfg {
  static constexpr int NC = WP / kKC;  // K chunks per GEMM
  static constexpr int kStages = WP == 256 ? 4 : 6;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t kTmemCols = WP == 64 ? 128 : (WP == 128 ? 256 : 512);
  // shared-memory offsets (bytes)
  static constexpr uint32_t oA = 0;
  static constexpr uint32_t oW = kABytes;
  static constexpr uint32_t oW0 = oW + kStages * kStageBytes;  // float4 [WP]
  static constexpr uint32_t oWout = oW0 + WP * 16;             // float [WP]
  static constexpr uint32_t oRed = oWout + WP * 4;             // float [2][128]
  static constexpr uint32_t oBar = oRed + 2 * kM * 4;          // barriers
  static constexpr uint32_t kNumBars = 2 * kStages + kMaxNC + 2 + 2 + 4 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;       // tmem slot, abort flag
  static constexpr uint32_t oHb = oMisc + 16;                  // float [nh][WP]
  static size_t bytes(int nh) { return oHb + (size_t)nh * WP * 4; }
};

// Cody-Waite reduction to [-pi, pi] with 2*pi split in two floats.
__device__ __forceinline__ float reduce_2pi(float z) {
  const float n = rintf(z * 0.15915494309189535f);
  const float r = __fmaf_rn(-n, 6.28318548202514648f, z);
  return __fmaf_rn(-n, -1.7484555314695172e-07f, r);
}

// sin through the hardware approximation (abs. error ~2^-21 on [-pi, pi]);
// `phase` is 0 or pi/2 (cosine) and keeps the argument within [-pi, 3pi/2].
__device__ __forceinline__ float sin_fast(float z, float phase = 0.f) {
  return __sinf(reduce_2pi(z) + phase);
}

__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, int* status,
                                                volatile int* abort_flag) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  report_device_error(status, MPL_ERR_DEVICE_TIMEOUT);
  *abort_flag = 1;
  return false;
}

// warp-uniform bounded wait (all lanes poll; any failure fails the warp)
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* status,
                                          volatile int* abort_flag) {
  const bool ok = mbar_wait_abort(bar, parity, status, abort_flag);
  return __all_sync(0xffffffffu, ok);
}

// A operand tile [128 x WP] bf16, K-major core matrices, layout
// [k/8][m/8][m%8][k%8]: LBO (next 8 K) = 2048 B, SBO (next 8 rows) = 128 B.
__device__ __forceinline__ void store_a_unit(uint8_t* sA, int m, int j0, const float (&v)[32]) {
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      __nv_bfloat162 b2 = __floats2bfloat162_rn(v[g * 8 + 2 * i], v[g * 8 + 2 * i + 1]);
      w[i] = *reinterpret_cast<uint32_t*>(&b2);
    }
    const int k8 = (j0 >> 3) + g;
    const uint32_t off = (uint32_t)((k8 * 16 + (m >> 3)) * 128 + (m & 7) * 16);
    *reinterpret_cast<uint4*>(sA + off) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

template <int WP, bool GRAD>
__global__ void __launch_bounds__(kThreads, 1) level_bf16_kernel(const LevelArgs a) {
  using C = Bf16Cfg<WP>;
  constexpr int PT = GRAD ? kM / 4 : kM;  // points per tile
  constexpr int NC = C::NC;
  constexpr int S = C::kStages;
  constexpr uint32_t IDESC = tc::idesc_bf16_f32(kM, WP);
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  float4* w0f = reinterpret_cast<float4*>(smem + C::oW0);
  float* wout = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;            // [S]   TMA -> MMA
  uint64_t* wempty = bars + S;       // [S]   MMA -> TMA
  uint64_t* achunk = bars + 2 * S;   // [NC]  epilogue -> MMA (count 8 warps)
  uint64_t* dfull = achunk + kMaxNC; // [2]   MMA -> epilogue
  uint64_t* dempty = dfull + 2;      // [2]   epilogue -> MMA (count 8 warps)
  uint64_t* redfull = dempty + 2;    // [2]   half-1 warps -> half-0 warps (count 4)
  uint64_t* redfree = redfull + 2;   // [2]   half-0 warps -> half-1 warps (count 4)
  uint64_t* finalb = redfree + 2;    // [1]   last MMA commit
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  float* hb = reinterpret_cast<float*>(smem + C::oHb);

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
      mbar_init(&redfull[b], 4);
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
      w0f[i] = g0[i];
      wout[i] = reinterpret_cast<const float*>(pk + a.lay.wout)[i];
    }
    for (int l = 1; l <= nh; ++l) {
      const float* gb = reinterpret_cast<const float*>(pk + a.lay.hb[l]);
      for (int i = threadIdx.x; i < WP; i += kThreads) hb[(l - 1) * WP + i] = gb[i];
    }
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
          const char* src = pk + a.lay.hw[l];
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
      const uint32_t aBase = smem_u32(sA);
      const uint32_t wBase = smem_u32(sW);
      int64_t w = 0, g = 0;
      int64_t duse[2] = {0, 0};
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int l = 1; l <= nh && ok; ++l, ++g) {
          const int b = (int)(g & 1);
          if (duse[b] > 0 &&
              !mbar_wait_abort(&dempty[b], (uint32_t)((duse[b] - 1) & 1), a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(b * WP);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            if (!mbar_wait_abort(&achunk[c], (uint32_t)(g & 1), a.status, abort_flag) ||
                !mbar_wait_abort(&wfull[s], (uint32_t)((w / S) & 1), a.status, abort_flag)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks) {
              const uint64_t ad = tc::smem_desc(aBase + (uint32_t)(c * 8 + ks * 2) * 2048u,
                                                2048u, 128u);
              const uint64_t bd = tc::smem_desc(wBase + (uint32_t)s * C::kStageBytes +
                                                    (uint32_t)ks * 256u,
                                                128u, 1024u);
              tc::mma_bf16(d_tmem, ad, bd, IDESC, (c | ks) != 0);
            }
            tc::commit(&wempty[s]);
          }
          if (!ok) break;
          tc::commit(&dfull[b]);
          ++duse[b];
        }
      }
      // every MMA issued so far must complete before TMEM is released
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else {
    // ================= epilogue warps (0-7) ================================
    const int q = warp & 3, h = warp >> 2;
    const int m = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    // GRAD: row m is channel ch of point m/4 (ch 0: value, 1..3: d/dx_(ch-1))
    const int ch = GRAD ? (m & 3) : 0;
    const int vlane = lane & ~3;
    const float phase = ch ? 1.57079632679489662f : 0.f;
    int64_t g = 0, tloc = 0;
    int64_t dcnt[2] = {0, 0};
    bool ok = true;
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tloc) {
      const int64_t qi = t * PT + (GRAD ? (m >> 2) : m);
      int64_t p = -1;
      float x = 0.f, y = 0.f, z = 0.f;
      if (qi < n) load_point(a, qi, p, x, y, z);

      // layer 0 (FP32) -> A chunks of the first hidden GEMM
#pragma unroll 1
      for (int c = 0; c < NC; ++c) {
        const int j0 = c * kKC + h * 32;
        float v[32];
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const float4 wv = w0f[j0 + jj];
          const float zz = __fmaf_rn(x, wv.x, __fmaf_rn(y, wv.y, __fmaf_rn(z, wv.z, wv.w)));
          if (GRAD) {
            const float dz = ch == 1 ? wv.x : (ch == 2 ? wv.y : wv.z);
            const float sc = sin_fast(zz, phase);
            v[jj] = ch ? __fmul_rn(sc, dz) : sc;
          } else {
            v[jj] = sin_fast(zz);
          }
        }
        store_a_unit(sA, m, j0, v);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&achunk[c]);
      }

      float part = 0.f;
      for (int l = 1; l <= nh; ++l, ++g) {
        const int b = (int)(g & 1);
        if (!warp_wait(&dfull[b], (uint32_t)(dcnt[b] & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t taddr = tl + (uint32_t)(b * WP);
        const float* bias = hb + (l - 1) * WP;
#pragma unroll 1
        for (int c = 0; c < NC; ++c) {
          const int j0 = c * kKC + h * 32;
          uint32_t r[32];
          tc::ld_32x32b_x32(taddr + (uint32_t)j0, r);
          tc::wait_ld();
          if (GRAD) {
            // value pre-activation of this point to its tangent lanes
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
              const float acc = __uint_as_float(r[jj]);
              const float zz = __fadd_rn(__shfl_sync(0xffffffffu, acc, vlane), bias[j0 + jj]);
              const float sc = sin_fast(zz, phase);
              r[jj] = __float_as_uint(ch ? __fmul_rn(sc, acc) : sc);
            }
          }
          if (l < nh) {
            float v[32];
#pragma unroll
            for (int jj = 0; jj < 32; ++jj)
              v[jj] = GRAD ? __uint_as_float(r[jj])
                           : sin_fast(__fadd_rn(__uint_as_float(r[jj]), bias[j0 + jj]));
            store_a_unit(sA, m, j0, v);
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&achunk[c]);
          } else {
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
              const float sv = GRAD ? __uint_as_float(r[jj])
                                    : sin_fast(__fadd_rn(__uint_as_float(r[jj]), bias[j0 + jj]));
              part = __fmaf_rn(sv, wout[j0 + jj], part);
            }
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&dempty[b]);
        ++dcnt[b];
      }
      if (!ok) break;

      // combine the two feature halves, store, band
      const int rb = (int)(tloc & 1);
      if (h == 1) {
        if (tloc >= 2 && !warp_wait(&redfree[rb], (uint32_t)(((tloc >> 1) - 1) & 1), a.status,
                                    abort_flag)) {
          ok = false;
          break;
        }
        red[rb * kM + m] = part;
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfull[rb]);
      } else {
        if (!warp_wait(&redfull[rb], (uint32_t)((tloc >> 1) & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        const float sum = __fadd_rn(part, red[rb * kM + m]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfree[rb]);
        if (GRAD) {
          if (ch && qi < n && a.G) {
            float* gp = a.G + 3 * p + (ch - 1);
            *gp = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(*gp, sum) : sum;
          }
          store_and_band(a, qi < n && ch == 0, p, __fadd_rn(sum, bout));
        } else {
          store_and_band(a, qi < n, p, __fadd_rn(sum, bout));
        }
      }
    }
  }

  // ---- teardown: all roles have left their loops; release TMEM
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, bool GRAD>
int launch_bf16_wp(const LevelArgs& a, cudaStream_t s) {
  using C = Bf16Cfg<WP>;
  constexpr int PT = GRAD ? kM / 4 : kM;
  const size_t smem = C::bytes(a.lay.nh);
  if (smem > 227 * 1024) return MPL_ERR_UNSUPPORTED;
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_bf16_kernel<WP, GRAD>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + PT - 1) / PT;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_bf16_kernel<WP, GRAD><<<(unsigned)grid, kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

template <bool GRAD>
int launch_bf16_mode(const LevelArgs& a, cudaStream_t s) {
  switch (a.lay.WP) {
    case 64: return launch_bf16_wp<64, GRAD>(a, s);
    case 128: return launch_bf16_wp<128, GRAD>(a, s);
    case 256: return launch_bf16_wp<256, GRAD>(a, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace

int launch_level_bf16(const LevelArgs& a, cudaStream_t s) {
  if (a.lay.nh == 0) return launch_level_fp32(a, s);  // no hidden GEMM to run in BF16
  return a.grad ? launch_bf16_mode<true>(a, s) : launch_bf16_mode<false>(a, s);
}

}  // namespace mpl
