// Two-tile ("ping-pong") form of the tensor-core level kernel (sm_103a).
//
// The single-tile kernel of level_bf16.cuh keeps one 128-row tile in flight
// per CTA: the tensor cores wait while the epilogue warps turn an
// accumulator into the next A operand, and the epilogue waits while a GEMM
// runs.  Here every CTA holds two tiles, X and Y, each with its own A
// operand buffer and its own TMEM accumulator, and the work is interleaved
//   epilogue:  E1(X) E1(Y) E2(X)+L0(X') E2(Y)+L0(Y') E1(X') ...
//   MMA:         G2(X) G2(Y)  G1(X')     G1(Y')        G2(X') ...
// so each GEMM of one tile runs while the epilogue drains the other tile.
// L0 is the FP32 first layer of the slot's next tile, computed inside the
// last drain as in the single-tile kernel; E_l turns the accumulator of GEMM l
// into the A operand of GEMM l+1 (sin, 16-bit), and the last drain adds the
// output layer, the store and the fused band list.  Per element the
// arithmetic is the single-tile kernel's, so both kernels give identical
// results.
//
// Barriers (per slot s): achunk[s][c] (epilogue -> MMA, A chunk c written),
// dfull[s] (MMA commit -> epilogue), dempty[s] (epilogue -> MMA, accumulator
// drained; the next GEMM of the slot overwrites it), redfull[s]/redfree[s]
// (feature-split partial sums of the output layer).  Weights stream through
// one ring in the MMA's GEMM order.  Every wait is bounded (the abort
// protocol of level_bf16.cuh).
#pragma once

#include "level_bf16.cuh"

namespace mpl {
namespace pp {

using bf16::kKC;
using bf16::kM;
using bf16::kMaxNC;

template <int WP, int STAGES, int U>
struct Cfg {
  static constexpr int NC = WP / kKC;
  static constexpr int Q = 64 / U;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t kTmemCols = WP == 64 ? 128 : (WP == 128 ? 256 : 512);
  static constexpr uint32_t oA = 0;                                  // [2] A operands
  static constexpr uint32_t oW = 2 * kABytes;                        // [S] weight chunks
  static constexpr uint32_t oW0 = oW + STAGES * kStageBytes;         // float [4][WP]
  static constexpr uint32_t oWout = oW0 + WP * 16;                   // float [WP]
  static constexpr uint32_t oRed = oWout + WP * 4;                   // float [2][Q-1][128]
  static constexpr uint32_t oBar = oRed + 2 * (Q > 1 ? Q - 1 : 1) * kM * 4;
  static constexpr uint32_t kNumBars = 2 * STAGES + 2 * kMaxNC + 2 + 2 + 2 + 2 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr uint32_t oAx = (oMisc + 16 + 1023) & ~1023u;     // ones tile
  static constexpr uint32_t oBx = oAx + kM * 16 * 2;                 // [nh] bias tiles
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  static size_t bytes(int nh) { return oBx + (size_t)nh * kBxBytes; }
};

template <int WP, bool GRAD, int STAGES, int U, typename T>
__global__ void __launch_bounds__(bf16::Epi<U>::kThreads, 1) level_pp_kernel(const LevelArgs a) {
  using C = Cfg<WP, STAGES, U>;
  using E = bf16::Epi<U>;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int PT = GRAD ? kM / 4 : kM;  // points per tile
  constexpr int NC = C::NC;
  constexpr int S = STAGES;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
  constexpr bool kF16 = Op::kFormat == 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem + C::oW;
  float* w0s = reinterpret_cast<float*>(smem + C::oW0);
  float* wout = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;                  // [S]
  uint64_t* wempty = bars + S;             // [S]
  uint64_t* achunk = bars + 2 * S;         // [2][kMaxNC]
  uint64_t* dfull = achunk + 2 * kMaxNC;   // [2]
  uint64_t* dempty = dfull + 2;            // [2]
  uint64_t* redfull = dempty + 2;          // [2]
  uint64_t* redfree = redfull + 2;         // [2]
  uint64_t* finalb = redfree + 2;          // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  uint8_t* sAx = smem + C::oAx;
  uint8_t* sBx = smem + C::oBx;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nh = a.lay.nh;
  const int64_t n = level_point_count(a);
  const int64_t ntiles = (n + PT - 1) / PT;
  if ((int64_t)blockIdx.x >= ntiles) return;
  const int64_t G = gridDim.x;
  // tile of slot s in round r
  auto tile_of = [&](int64_t r, int s) { return (int64_t)blockIdx.x + (2 * r + s) * G; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    for (int c = 0; c < 2 * kMaxNC; ++c) mbar_init(&achunk[c], kEpiWarps);
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
    for (int i = threadIdx.x; i < kM * 16; i += kThreads) {
      const int m = i >> 4, k = i & 15;
      const bool one = k < 2 && (!GRAD || (m & 3) == 0);
      const uint32_t off =
          (uint32_t)(((k >> 3) * 16 + (m >> 3)) * 128 + (m & 7) * 16 + (k & 7) * 2);
      *reinterpret_cast<T*>(sAx + off) = Op::value(one ? 1.f : 0.f);
    }
    fence_proxy_async_smem();
  }
  const float bout = reinterpret_cast<const float*>(pk + a.lay.bout)[0];
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const int64_t nrounds = (ntiles - blockIdx.x + 2 * G - 1) / (2 * G);

  if (warp == kTmaWarp) {
    // ================= TMA: weight K chunks in the MMA's GEMM order ========
    if (lane == 0) {
      int64_t w = 0;
      bool ok = true;
      for (int64_t r = 0; r < nrounds && ok && !*abort_flag; ++r) {
        for (int l = 1; l <= nh && ok; ++l) {
          for (int s = 0; s < 2 && ok; ++s) {
            if (tile_of(r, s) >= ntiles) continue;
            const char* src = pk + (kF16 ? a.lay.hwh[l] : a.lay.hw[l]);
            for (int c = 0; c < NC; ++c, ++w) {
              const int st = (int)(w % S);
              const int64_t u = w / S;
              if (u > 0 && !bf16::mbar_wait_abort(&wempty[st], (uint32_t)((u - 1) & 1), a.status,
                                                  abort_flag)) {
                ok = false;
                break;
              }
              mbar_arrive_expect_tx(&wfull[st], C::kStageBytes);
              tma_bulk_g2s(sW + st * C::kStageBytes, src + (size_t)c * C::kStageBytes,
                           C::kStageBytes, &wfull[st]);
            }
          }
        }
      }
      const int64_t first = w > S ? w - S : 0;
      for (int64_t v = first; v < w; ++v)
        mbar_wait(&wfull[v % S], (uint32_t)((v / S) & 1), a.status);
    }
  } else if (warp == kMmaWarp) {
    // ================= MMA issuer ==========================================
    if (lane == 0) {
      // descriptor bases; an operand at byte offset o adds o >> 4 (the start
      // address field, which stays below 2^14 inside shared memory)
      const uint64_t aDesc = tc::smem_desc(smem_u32(smem + C::oA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      const uint64_t bxDesc = tc::smem_desc(smem_u32(sBx), 128u, 256u);
      int64_t w = 0;
      bool ok = true;
      for (int64_t r = 0; r < nrounds && ok; ++r) {
        for (int l = 1; l <= nh && ok; ++l) {
          for (int s = 0; s < 2 && ok; ++s) {
            if (tile_of(r, s) >= ntiles) continue;
            // GEMMs the slot issued before: a slot has a tile in every round
            // up to its last, so the count follows from (r, l)
            const int64_t k = r * nh + (l - 1);
            if (k > 0 && !bf16::mbar_wait_abort(&dempty[s], (uint32_t)((k - 1) & 1), a.status,
                                                abort_flag)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const uint32_t d_tmem = tmem + (uint32_t)(s * WP);
            const uint64_t aS = aDesc + (uint64_t)((s * C::kABytes) >> 4);
            tc::mma_bf16(d_tmem, xDesc, bxDesc + (uint64_t)(((l - 1) * C::kBxBytes) >> 4), IDESC,
                         false);
            for (int c = 0; c < NC; ++c, ++w) {
              const int st = (int)(w % S);
              if (!bf16::mbar_wait_abort(&achunk[s * kMaxNC + c], (uint32_t)(k & 1), a.status,
                                         abort_flag) ||
                  !bf16::mbar_wait_abort(&wfull[st], (uint32_t)((w / S) & 1), a.status,
                                         abort_flag)) {
                ok = false;
                break;
              }
              tc::fence_after_sync();
              const uint64_t aC = aS + (uint64_t)((c * 8 * 2048) >> 4);
              const uint64_t wC = wDesc + (uint64_t)((st * C::kStageBytes) >> 4);
#pragma unroll
              for (int ks = 0; ks < kKC / 16; ++ks)
                tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                             wC + (uint64_t)((ks * 256) >> 4), IDESC, true);
              tc::commit(&wempty[st]);
            }
            if (!ok) break;
            tc::commit(&dfull[s]);
          }
        }
      }
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else {
    // ================= epilogue warps =====================================
    const int q = warp & 3, h = warp >> 2;
    const int m = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    const int ch = GRAD ? (m & 3) : 0;
    const int vlane = lane & ~3;
    const float phase = ch ? 1.57079632679489662f : 0.f;
    const int prow = GRAD ? (m >> 2) : m;
    // point index of each slot's current row (two scalars rather than an
    // array indexed by the slot, which would live in local memory)
    int64_t p0 = -1, p1 = -1;
    bool ok = true;
    // layer 0 of the first tile of each slot
    for (int s = 0; s < 2; ++s) {
      const int64_t t = tile_of(0, s);
      if (t >= ntiles) continue;
      float x = 0.f, y = 0.f, z = 0.f;
      const int64_t qi = t * PT + prow;
      int64_t pq = -1;
      if (qi < n) load_point(a, qi, pq, x, y, z);
      if (s)
        p1 = pq;
      else
        p0 = pq;
      uint8_t* sA = smem + C::oA + s * C::kABytes;
#pragma unroll 1
      for (int c = 0; c < NC; ++c) {
        bf16::layer0_unit<T, GRAD, U>(sA, w0s, WP, m, c * kKC + h * U, ch, phase, x, y, z);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&achunk[s * kMaxNC + c]);
      }
    }
    for (int64_t r = 0; r < nrounds && ok; ++r) {
      for (int l = 1; l <= nh && ok; ++l) {
        for (int s = 0; s < 2 && ok; ++s) {
          const int64_t t = tile_of(r, s);
          if (t >= ntiles) continue;
          // drains of the slot before this one (as the MMA's GEMM count)
          const int64_t dn = r * nh + (l - 1);
          if (!bf16::warp_wait(&dfull[s], (uint32_t)(dn & 1), a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          uint8_t* sA = smem + C::oA + s * C::kABytes;
          const int64_t tn = t + 2 * G;  // the slot's next tile
          const bool has_next = l == nh && tn < ntiles;
          int64_t pn = -1;
          float xn = 0.f, yn = 0.f, zn = 0.f;
          if (has_next) {
            const int64_t qn = tn * PT + prow;
            if (qn < n) load_point(a, qn, pn, xn, yn, zn);
          }
          float part = 0.f;  // this lane's share of the output dot (last drain)
          const uint32_t taddr = tl + (uint32_t)(s * WP);
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
              uint32_t (&rr)[U] = r2[u];
              if (GRAD) {
#pragma unroll
                for (int jj = 0; jj < U; ++jj) {
                  const float acc = __uint_as_float(rr[jj]);
                  const float zz = __shfl_sync(0xffffffffu, acc, vlane);
                  const float sc = bf16::sin_fast(zz, phase);
                  rr[jj] = __float_as_uint(ch ? __fmul_rn(sc, acc) : sc);
                }
              }
              if (l < nh) {
                float v[U];
#pragma unroll
                for (int jj = 0; jj < U; ++jj)
                  v[jj] = GRAD ? __uint_as_float(rr[jj]) : bf16::sin_fast(__uint_as_float(rr[jj]));
                bf16::store_a_unit<T, U>(sA, m, j0, v);
              } else {
                const float4* wo4 = reinterpret_cast<const float4*>(wout + j0);
                float pt = part;
#pragma unroll
                for (int j4 = 0; j4 < U / 4; ++j4) {
                  const float4 wv = wo4[j4];
                  const float wa[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
                  for (int i = 0; i < 4; ++i) {
                    const float acc = __uint_as_float(rr[4 * j4 + i]);
                    const float sv = GRAD ? acc : bf16::sin_fast(acc);
                    pt = __fmaf_rn(sv, wa[i], pt);
                  }
                }
                part = pt;
                if (has_next) bf16::layer0_unit<T, GRAD, U>(sA, w0s, WP, m, j0, ch, phase, xn, yn, zn);
              }
            }
          }
          // the slot's next GEMM waits for the whole drain (it overwrites the
          // accumulator), so the A chunks written here are handed over at once
          if (l < nh || has_next) fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) {
            if (l < nh || has_next)
              for (int c = 0; c < NC; ++c) mbar_arrive(&achunk[s * kMaxNC + c]);
            mbar_arrive(&dempty[s]);
          }
          if (l < nh) continue;

          // output layer: combine the feature splits, store, band
          const int64_t u = r;  // output reductions of the slot before this one
          float* rs = red + s * (Q > 1 ? Q - 1 : 1) * kM;
          if (h > 0) {
            if (u >= 1 && !bf16::warp_wait(&redfree[s], (uint32_t)((u - 1) & 1), a.status,
                                           abort_flag)) {
              ok = false;
              break;
            }
            rs[(h - 1) * kM + m] = part;
            __syncwarp();
            if (lane == 0) mbar_arrive(&redfull[s]);
          } else {
            if (!bf16::warp_wait(&redfull[s], (uint32_t)(u & 1), a.status, abort_flag)) {
              ok = false;
              break;
            }
            float sum = part;
#pragma unroll
            for (int hh = 0; hh < Q - 1; ++hh) sum = __fadd_rn(sum, rs[hh * kM + m]);
            __syncwarp();
            if (lane == 0) mbar_arrive(&redfree[s]);
            const int64_t ps = s ? p1 : p0;
            if (GRAD) {
              if (ch && ps >= 0 && a.G) {
                float* gp = a.G + 3 * ps + (ch - 1);
                *gp = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(*gp, sum) : sum;
              }
              store_and_band(a, ps >= 0 && ch == 0, ps, __fadd_rn(sum, bout));
            } else {
              store_and_band(a, ps >= 0, ps, __fadd_rn(sum, bout));
            }
          }
          if (s)
            p1 = pn;
          else
            p0 = pn;
        }
      }
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, bool GRAD, int STAGES, int U, typename T>
int launch_cfg(const LevelArgs& a, cudaStream_t s) {
  using C = Cfg<WP, STAGES, U>;
  constexpr int PT = GRAD ? kM / 4 : kM;
  const size_t smem = C::bytes(a.lay.nh);
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_pp_kernel<WP, GRAD, STAGES, U, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + PT - 1) / PT;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_pp_kernel<WP, GRAD, STAGES, U, T><<<(unsigned)grid, bf16::Epi<U>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// the two-tile kernel with the deepest weight ring that fits next to the
// level's bias tiles; MPL_ERR_UNSUPPORTED when none does (the caller falls
// back to the single-tile kernel)
template <int WP, bool GRAD, int U, typename T>
int launch_wp(const LevelArgs& a, cudaStream_t s) {
  constexpr size_t kLimit = 227 * 1024;
  if (Cfg<WP, 4, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 4, U, T>(a, s);
  if (Cfg<WP, 3, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 3, U, T>(a, s);
  if (Cfg<WP, 2, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 2, U, T>(a, s);
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

}  // namespace pp
}  // namespace mpl
