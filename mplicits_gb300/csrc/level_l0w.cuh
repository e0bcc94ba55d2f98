// Two-tile tensor-core level kernel with dedicated first-layer warps (sm_103a).
//
// The two-tile kernel of level_pp.cuh computes the next tile's FP32 first
// layer (phase omega0 (W0 x + b0), sine, 16-bit A operand) inside the last
// drain of the current tile: about a third of the epilogue's instructions,
// on the epilogue's critical chain, and the grid coordinates of every row
// are computed by all four warps that share the row.  Here four more warps
// own the first layer: warp i computes rows 32i..32i+31 of a slot's next
// tile (each row's point once) and hands the A operand to the MMA issuer in
// 64-feature chunks, so the first GEMM of a tile starts on chunk 0 while
// the later chunks are still being written, and the epilogue warps only
// drain accumulators.  Per element the arithmetic is the other kernels', so
// the results are identical bit for bit.
//
// Barriers (per slot s), next to level_pp.cuh's: l0chunk[s][c] (first-layer
// warps -> MMA, A chunk c of the slot's tile written; one phase per tile),
// afree[s] (MMA commit after the tile's last GEMM -> first-layer warps, the
// slot's A operand may be overwritten; one phase per tile).  achunk[s][c]
// now carries only the A operands that drains write (GEMMs 2..nh).  A slot's
// barriers cannot run more than one phase ahead of a waiter: each of their
// next phases needs the waiter's own hand-off first.  Every wait is bounded
// (the abort protocol of level_bf16.cuh).
#pragma once

#include "level_pp.cuh"

namespace mpl {
namespace l0w {

using bf16::kKC;
using bf16::kM;
using bf16::kMaxNC;

// Warp roles for an epilogue unit width U and NL first-layer warps (4 or 8):
// 4 (64 / U) epilogue warps, the first-layer warps (warp w of them owns rows
// 32 (w % 4) .. + 31 and, with 8, half of every 64-feature chunk), the
// MMA-issuing warp and the TMA warp.
template <int U, int NL>
struct Roles {
  static_assert(NL == 4 || NL == 8, "first-layer warps");
  static constexpr int kQ = 64 / U;
  static constexpr int kEpiWarps = 4 * kQ;
  static constexpr int kL0Warps = NL;
  static constexpr int kL0First = kEpiWarps;
  static constexpr int kMmaWarp = kEpiWarps + NL;
  static constexpr int kTmaWarp = kMmaWarp + 1;
  static constexpr int kThreads = (kTmaWarp + 1) * 32;
};

template <int WP, int STAGES, int U>
struct Cfg {
  using P = pp::Cfg<WP, STAGES, U>;
  static constexpr int NC = P::NC;
  static constexpr uint32_t kStageBytes = P::kStageBytes;
  static constexpr uint32_t kABytes = P::kABytes;
  static constexpr uint32_t kTmemCols = P::kTmemCols;
  static constexpr uint32_t oA = P::oA;
  static constexpr uint32_t oW = P::oW;
  static constexpr uint32_t oW0 = P::oW0;
  static constexpr uint32_t oWout = P::oWout;
  static constexpr uint32_t oRed = P::oRed;
  static constexpr uint32_t oBar = P::oBar;
  // wfull/wempty [S], achunk/l0chunk [2][kMaxNC], dfull, dempty, redfull,
  // redfree, afree [2], final
  static constexpr uint32_t kNumBars = 2 * STAGES + 4 * kMaxNC + 5 * 2 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr uint32_t oAx = (oMisc + 16 + 1023) & ~1023u;  // ones tile
  static constexpr uint32_t oBx = oAx + kM * 16 * 2;             // [nh] bias tiles
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  static size_t bytes(int nh) { return oBx + (size_t)nh * kBxBytes; }
};

template <int WP, bool GRAD, int STAGES, int U, int NL, typename T>
__global__ void __launch_bounds__(Roles<U, NL>::kThreads, 1) level_l0w_kernel(const LevelArgs a) {
  using C = Cfg<WP, STAGES, U>;
  using R = Roles<U, NL>;
  constexpr int kL0Warps = NL;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = R::kEpiWarps;
  constexpr int kL0First = R::kL0First;
  constexpr int kMmaWarp = R::kMmaWarp;
  constexpr int kTmaWarp = R::kTmaWarp;
  constexpr int kThreads = R::kThreads;
  constexpr int Q = R::kQ;
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
  uint64_t* wfull = bars;                   // [S]
  uint64_t* wempty = bars + S;              // [S]
  uint64_t* achunk = bars + 2 * S;          // [2][kMaxNC] drains -> MMA
  uint64_t* l0chunk = achunk + 2 * kMaxNC;  // [2][kMaxNC] first layer -> MMA
  uint64_t* dfull = l0chunk + 2 * kMaxNC;   // [2]
  uint64_t* dempty = dfull + 2;             // [2]
  uint64_t* redfull = dempty + 2;           // [2]
  uint64_t* redfree = redfull + 2;          // [2]
  uint64_t* afree = redfree + 2;            // [2]
  uint64_t* finalb = afree + 2;             // [1]
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
    for (int c = 0; c < 2 * kMaxNC; ++c) {
      mbar_init(&achunk[c], kEpiWarps);
      mbar_init(&l0chunk[c], kL0Warps);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&dfull[b], 1);
      mbar_init(&dempty[b], kEpiWarps);
      mbar_init(&redfull[b], 4 * (Q - 1));
      mbar_init(&redfree[b], 4);
      mbar_init(&afree[b], 1);
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
            // the A operand of GEMM 1 comes from the first-layer warps (one
            // phase per tile), that of GEMM l > 1 from drain l - 1 (nh - 1
            // phases per tile)
            uint64_t* abar = l == 1 ? l0chunk + s * kMaxNC : achunk + s * kMaxNC;
            const uint32_t apar = l == 1 ? (uint32_t)(r & 1)
                                         : (uint32_t)((r * (nh - 1) + (l - 2)) & 1);
            const uint32_t d_tmem = tmem + (uint32_t)(s * WP);
            const uint64_t aS = aDesc + (uint64_t)((s * C::kABytes) >> 4);
            tc::mma_bf16(d_tmem, xDesc, bxDesc + (uint64_t)(((l - 1) * C::kBxBytes) >> 4), IDESC,
                         false);
            for (int c = 0; c < NC; ++c, ++w) {
              const int st = (int)(w % S);
              if (!bf16::mbar_wait_abort(&abar[c], apar, a.status, abort_flag) ||
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
            if (l == nh) tc::commit(&afree[s]);  // the slot's A operand is free
          }
        }
      }
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else if (warp >= kL0First) {
    // ================= first-layer warps ==================================
    const int m = 32 * ((warp - kL0First) & 3) + lane;  // row of the tile
    constexpr int kF = kKC * 4 / NL;                      // features per chunk
    const int f0 = ((warp - kL0First) >> 2) * kF;         // first of them
    const int ch = GRAD ? (m & 3) : 0;
    const float phase = ch ? 1.57079632679489662f : 0.f;
    const int prow = GRAD ? (m >> 2) : m;
    // The warp's tiles in order k = 2 r + s (tile blockIdx.x + k gridDim.x);
    // a row's point id is read one tile ahead, so that the gather from an
    // index list (band lists) lands while the previous tile is computed.
    auto point_id = [&](int64_t t) -> int64_t {
      const int64_t qi = t * PT + prow;
      return qi < n ? (a.index ? (int64_t)a.index[qi] : qi) : -1;
    };
    const int64_t nt = (ntiles - blockIdx.x + G - 1) / G;
    int64_t pn = point_id(blockIdx.x);
    bool ok = true;
#pragma unroll 1
    for (int64_t k = 0; k < nt && ok; ++k) {
      const int64_t t = (int64_t)blockIdx.x + k * G;
      const int64_t r = k >> 1;
      const int s = (int)(k & 1);
      const int64_t p = pn;
      if (k + 1 < nt) pn = point_id(t + G);
      float x = 0.f, y = 0.f, z = 0.f;
      if (p >= 0) point_coords(a, p, x, y, z);
      // the slot's previous tile has finished its last GEMM (the reader of
      // the A operand written here)
      if (r > 0 &&
          !bf16::warp_wait(&afree[s], (uint32_t)((r - 1) & 1), a.status, abort_flag)) {
        ok = false;
        break;
      }
      uint8_t* sA = smem + C::oA + s * C::kABytes;
#pragma unroll 1
      for (int c = 0; c < NC; ++c) {
#pragma unroll
        for (int u = 0; u < kF / 16; ++u)
          bf16::layer0_unit<T, GRAD, 16>(sA, w0s, WP, m, c * kKC + f0 + u * 16, ch, phase, x,
                                          y, z);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&l0chunk[s * kMaxNC + c]);
      }
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
    bool ok = true;
    for (int64_t r = 0; r < nrounds && ok; ++r) {
      for (int l = 1; l <= nh && ok; ++l) {
        for (int s = 0; s < 2 && ok; ++s) {
          const int64_t t = tile_of(r, s);
          if (t >= ntiles) continue;
          // drains of the slot before this one (as the MMA's GEMM count)
          const int64_t dn = r * nh + (l - 1);
          int64_t ps = -1;  // point of this row (last drain: the store)
          if (l == nh && h == 0) {
            const int64_t qi = t * PT + prow;
            if (qi < n) ps = a.index ? (int64_t)a.index[qi] : qi;
          }
          if (!bf16::warp_wait(&dfull[s], (uint32_t)(dn & 1), a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          uint8_t* sA = smem + C::oA + s * C::kABytes;
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
              }
            }
          }
          // the value this level adds to, read while the reduction below waits
          // (the point id has arrived during the drain)
          float sold = 0.f;
          if (!GRAD && ps >= 0 && a.store_mode == MPL_ACCUMULATE) sold = a.S[ps];
          // the slot's next GEMM waits for the whole drain (it overwrites the
          // accumulator), so the A chunks written here are handed over at once
          if (l < nh) fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) {
            if (l < nh)
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
            if (GRAD) {
              if (ch && ps >= 0 && a.G) {
                float* gp = a.G + 3 * ps + (ch - 1);
                *gp = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(*gp, sum) : sum;
              }
              store_and_band(a, ps >= 0 && ch == 0, ps, __fadd_rn(sum, bout));
            } else {
              store_and_band_old(a, ps >= 0, ps, __fadd_rn(sum, bout), sold);
            }
          }
        }
      }
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, bool GRAD, int STAGES, int U, int NL, typename T>
int launch_cfg(const LevelArgs& a, cudaStream_t s) {
  using C = Cfg<WP, STAGES, U>;
  constexpr int PT = GRAD ? kM / 4 : kM;
  const size_t smem = C::bytes(a.lay.nh);
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_l0w_kernel<WP, GRAD, STAGES, U, NL, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + PT - 1) / PT;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_l0w_kernel<WP, GRAD, STAGES, U, NL, T>
      <<<(unsigned)grid, Roles<U, NL>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// the deepest weight ring that fits next to the level's bias tiles;
// MPL_ERR_UNSUPPORTED when none does (the caller falls back)
template <int WP, bool GRAD, int U, int NL, typename T>
int launch_wp(const LevelArgs& a, cudaStream_t s) {
  constexpr size_t kLimit = 227 * 1024;
  if (Cfg<WP, 4, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 4, U, NL, T>(a, s);
  if (Cfg<WP, 3, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 3, U, NL, T>(a, s);
  if (Cfg<WP, 2, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, GRAD, 2, U, NL, T>(a, s);
  return MPL_ERR_UNSUPPORTED;
}

template <int U, int NL, typename T>
int launch_unit(const LevelArgs& a, cudaStream_t s) {
  switch (a.lay.WP) {
    case 64:
      return a.grad ? launch_wp<64, true, U, NL, T>(a, s) : launch_wp<64, false, U, NL, T>(a, s);
    case 128:
      return a.grad ? launch_wp<128, true, U, NL, T>(a, s) : launch_wp<128, false, U, NL, T>(a, s);
    case 256:
      return a.grad ? launch_wp<256, true, U, NL, T>(a, s) : launch_wp<256, false, U, NL, T>(a, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace l0w
}  // namespace mpl
