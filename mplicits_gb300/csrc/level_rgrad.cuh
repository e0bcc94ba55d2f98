// Reverse-mode input gradient of one level on the tensor cores (sm_103a):
// f(x) and df/dx for 128 points per tile.
//
// The forward-mode gradient of the level kernels carries three tangent rows
// per point through every GEMM (four rows per point, 32 points per tile).
// Here a tile holds 128 points and the gradient comes from a backward sweep
// over the same tile, two GEMMs per hidden layer instead of four times the
// forward GEMMs:
//   forward   z_0 = w0 (W0 x + b0) (FP32), s_l = sin z_l,
//             z_l = w_l (W_l s_(l-1) + b_l)            GEMM G_l, l = 1..nh
//             f   = W_L s_nh + b_L                      (FP32 dot)
//   backward  dz_nh = cos(z_nh) W_L                     (last forward drain)
//             ds_(l-1) = (w_l W_l)^T dz_l               GEMM B_l, l = nh..1
//             dz_(l-1) = cos(z_(l-1)) ds_(l-1)
//             df/dx = (w0 W0)^T dz_0                    (FP32, z_0 recomputed)
// The adjoints dz_l enter the backward GEMMs as 16-bit A operands against
// the transposed weight tiles (omega folded in), as the activations enter
// the forward ones.  One tile in flight per CTA; the GEMMs of a tile run in
// sequence G_1 .. G_nh, B_nh .. B_1 into two TMEM accumulators (G_l and B_l
// into accumulator (l - 1) & 1), so z_1 stays in accumulator 0 until B_2's
// drain reads it (nh <= 2).  The next tile's first layer is written inside
// the last drain.  Roles, waits and abort handling as in level_bf16.cuh.
#pragma once

#include "level_bf16.cuh"

namespace mpl {
namespace rgrad {

using bf16::kKC;
using bf16::kM;

template <int WP, int STAGES, int U>
struct Cfg {
  static constexpr int NC = WP / kKC;
  static constexpr int Q = 64 / U;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t kTmemCols = WP == 64 ? 128 : (WP == 128 ? 256 : 512);
  static constexpr uint32_t oA = 0;
  static constexpr uint32_t oW = kABytes;                          // [S] weight chunks
  static constexpr uint32_t oW0 = oW + STAGES * kStageBytes;     // float [4][WP]
  static constexpr uint32_t oWout = oW0 + WP * 16;               // float [WP]
  static constexpr uint32_t oRed = oWout + WP * 4;               // float [Q-1][4][128]
  static constexpr uint32_t oBar = oRed + (Q > 1 ? Q - 1 : 1) * 4 * kM * 4;
  static constexpr uint32_t kNumBars = 2 * STAGES + 1 + 1 + 2 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr uint32_t oAx = (oMisc + 16 + 1023) & ~1023u;  // ones tile
  static constexpr uint32_t oBx = oAx + kM * 16 * 2;             // [nh] bias tiles
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  static size_t bytes(int nh) { return oBx + (size_t)nh * kBxBytes; }
};

template <int WP, int STAGES, int U, typename T>
__global__ void __launch_bounds__(bf16::Epi<U>::kThreads, 1) level_rgrad_kernel(const LevelArgs a) {
  using C = Cfg<WP, STAGES, U>;
  using E = bf16::Epi<U>;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int NC = C::NC;
  constexpr int S = STAGES;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
  constexpr bool kF16 = Op::kFormat == 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  float* w0s = reinterpret_cast<float*>(smem + C::oW0);
  float* wout = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;             // [S]  TMA -> MMA
  uint64_t* wempty = bars + S;        // [S]  MMA -> TMA
  uint64_t* afull = bars + 2 * S;     // A operand written (count: epilogue warps)
  uint64_t* dfull = afull + 1;        // GEMM done
  uint64_t* redfull = dfull + 1;      // h > 0 partials written (count 4 (Q-1))
  uint64_t* redfree = redfull + 1;    // h = 0 has read them (count 4)
  uint64_t* finalb = redfree + 1;     // last MMA commit
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  uint8_t* sAx = smem + C::oAx;
  uint8_t* sBx = smem + C::oBx;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nh = a.lay.nh;  // 1 or 2
  const int G2 = 2 * nh;    // GEMMs per tile
  const int64_t n = level_point_count(a);
  const int64_t ntiles = (n + kM - 1) / kM;
  if ((int64_t)blockIdx.x >= ntiles) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    mbar_init(afull, kEpiWarps);
    mbar_init(dfull, 1);
    mbar_init(redfull, 4 * (Q - 1));
    mbar_init(redfree, 4);
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
      const uint32_t off =
          (uint32_t)(((k >> 3) * 16 + (m >> 3)) * 128 + (m & 7) * 16 + (k & 7) * 2);
      *reinterpret_cast<T*>(sAx + off) = Op::value(k < 2 ? 1.f : 0.f);
    }
    fence_proxy_async_smem();
  }
  const float bout = reinterpret_cast<const float*>(pk + a.lay.bout)[0];
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  // GEMM g of a tile: forward G_(g+1) for g < nh, backward B_(2nh-g) after
  auto layer_of = [&](int g) { return g < nh ? g + 1 : G2 - g; };

  if (warp == kTmaWarp) {
    // ================= TMA: weight K chunks in the MMA's GEMM order ========
    if (lane == 0) {
      int64_t w = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok && !*abort_flag; t += gridDim.x)
        for (int g = 0; g < G2 && ok; ++g) {
          const int l = layer_of(g);
          const int64_t off = g < nh ? (kF16 ? a.lay.hwh[l] : a.lay.hw[l])
                                     : (kF16 ? a.lay.hwTh[l] : a.lay.hwT[l]);
          const char* src = pk + off;
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            const int64_t u = w / S;
            if (u > 0 && !bf16::mbar_wait_abort(&wempty[s], (uint32_t)((u - 1) & 1), a.status,
                                                abort_flag)) {
              ok = false;
              break;
            }
            mbar_arrive_expect_tx(&wfull[s], C::kStageBytes);
            tma_bulk_g2s(sW + s * C::kStageBytes, src + (size_t)c * C::kStageBytes,
                         C::kStageBytes, &wfull[s]);
          }
        }
      const int64_t first = w > S ? w - S : 0;
      for (int64_t v = first; v < w; ++v)
        mbar_wait(&wfull[v % S], (uint32_t)((v / S) & 1), a.status);
    }
  } else if (warp == kMmaWarp) {
    // ================= MMA issuer: one GEMM after the other ================
    if (lane == 0) {
      const uint64_t aDesc = tc::smem_desc(smem_u32(sA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      const uint64_t bxDesc = tc::smem_desc(smem_u32(sBx), 128u, 256u);
      int64_t w = 0, k = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x)
        for (int g = 0; g < G2 && ok; ++g, ++k) {
          // GEMM k's A operand is written by drain k - 1 (or by the first
          // layer), which has also finished with both accumulators
          if (!bf16::mbar_wait_abort(afull, (uint32_t)(k & 1), a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const int l = layer_of(g);
          const uint32_t d_tmem = tmem + (uint32_t)(((l - 1) & 1) * WP);
          const bool fwd = g < nh;
          if (fwd)
            tc::mma_bf16(d_tmem, xDesc, bxDesc + (uint64_t)(((l - 1) * C::kBxBytes) >> 4), IDESC,
                         false);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            if (!bf16::mbar_wait_abort(&wfull[s], (uint32_t)((w / S) & 1), a.status,
                                       abort_flag)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const uint64_t aC = aDesc + (uint64_t)((c * 8 * 2048) >> 4);
            const uint64_t wC = wDesc + (uint64_t)((s * C::kStageBytes) >> 4);
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks)
              tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                           wC + (uint64_t)((ks * 256) >> 4), IDESC, fwd || c > 0 || ks > 0);
            tc::commit(&wempty[s]);
          }
          if (!ok) break;
          tc::commit(dfull);
        }
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else {
    // ================= epilogue warps =====================================
    const int q = warp & 3, h = warp >> 2;
    const int m = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    int64_t k = 0, tloc = 0;
    bool ok = true;
    int64_t p = -1;
    float x = 0.f, y = 0.f, z = 0.f;
    {
      const int64_t qi = (int64_t)blockIdx.x * kM + m;
      if (qi < n) load_point(a, qi, p, x, y, z);
    }
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      bf16::layer0_unit<T, false, U>(sA, w0s, WP, m, c * kKC + h * U, 0, 0.f, x, y, z);
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(afull);
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tloc) {
      const int64_t tn = t + gridDim.x;
      const bool has_next = tn < ntiles;
      int64_t pn = -1;
      float xn = 0.f, yn = 0.f, zn = 0.f;
      float fpart = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f;
      for (int g = 0; g < G2; ++g, ++k) {
        if (!bf16::warp_wait(dfull, (uint32_t)(k & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const int l = layer_of(g);
        const uint32_t acc = tl + (uint32_t)(((l - 1) & 1) * WP);
        const bool last = g == G2 - 1;
        if (last && has_next) {
          const int64_t qn = tn * kM + m;
          if (qn < n) load_point(a, qn, pn, xn, yn, zn);
        }
#pragma unroll 1
        for (int c = 0; c < NC; ++c) {
          const int j0 = c * kKC + h * U;
          uint32_t r[U];
          tc::ld_32x32b<U>(acc + (uint32_t)j0, r);
          if (g < nh - 1) {
            // hidden forward drain: s_l = sin z_l (z_l stays in its accumulator)
            tc::wait_ld();
            float v[U];
#pragma unroll
            for (int jj = 0; jj < U; ++jj) v[jj] = bf16::sin_fast(__uint_as_float(r[jj]));
            bf16::store_a_unit<T, U>(sA, m, j0, v);
          } else if (g == nh - 1) {
            // last forward drain: the output dot and dz_nh = cos(z_nh) W_L
            tc::wait_ld();
            const float4* wo4 = reinterpret_cast<const float4*>(wout + j0);
            float v[U];
#pragma unroll
            for (int j4 = 0; j4 < U / 4; ++j4) {
              const float4 wv = wo4[j4];
              const float wa[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const float zz = __uint_as_float(r[4 * j4 + i]);
                fpart = __fmaf_rn(bf16::sin_fast(zz), wa[i], fpart);
                v[4 * j4 + i] = __fmul_rn(__cosf(zz), wa[i]);
              }
            }
            bf16::store_a_unit<T, U>(sA, m, j0, v);
          } else if (!last) {
            // backward drain of B_l, l >= 2: dz_(l-1) = cos(z_(l-1)) ds_(l-1),
            // z_(l-1) from the accumulator of G_(l-1)
            uint32_t rz[U];
            tc::ld_32x32b<U>(tl + (uint32_t)(((l - 2) & 1) * WP) + (uint32_t)j0, rz);
            tc::wait_ld();
            float v[U];
#pragma unroll
            for (int jj = 0; jj < U; ++jj)
              v[jj] = __fmul_rn(__cosf(__uint_as_float(rz[jj])), __uint_as_float(r[jj]));
            bf16::store_a_unit<T, U>(sA, m, j0, v);
          } else {
            // drain of B_1: dz_0 = cos(z_0) ds_0 with z_0 recomputed in FP32,
            // df/dx = (w0 W0)^T dz_0
            tc::wait_ld();
#pragma unroll
            for (int j4 = 0; j4 < U / 4; ++j4) {
              float zz[4];
              float4 wx, wy, wz;
              bf16::phase4(w0s, WP, j0 + 4 * j4, x, y, z, zz, wx, wy, wz);
              const float ax[4] = {wx.x, wx.y, wx.z, wx.w};
              const float ay[4] = {wy.x, wy.y, wy.z, wy.w};
              const float az[4] = {wz.x, wz.y, wz.z, wz.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const float dz = __fmul_rn(__cosf(zz[i]), __uint_as_float(r[4 * j4 + i]));
                g0 = __fmaf_rn(dz, ax[i], g0);
                g1 = __fmaf_rn(dz, ay[i], g1);
                g2 = __fmaf_rn(dz, az[i], g2);
              }
            }
            if (has_next)
              bf16::layer0_unit<T, false, U>(sA, w0s, WP, m, j0, 0, 0.f, xn, yn, zn);
          }
        }
        // this drain wrote the A operand of the next GEMM (of this tile, or
        // the next tile's first); the accumulators are free for it
        const bool hand_over = !last || has_next;
        if (hand_over) fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0 && hand_over) mbar_arrive(afull);
      }
      if (!ok) break;

      // combine the feature splits: f, df/dx, df/dy, df/dz of each point
      if (h > 0) {
        if (tloc >= 1 && !bf16::warp_wait(redfree, (uint32_t)((tloc - 1) & 1), a.status,
                                          abort_flag)) {
          ok = false;
          break;
        }
        float* rs = red + (h - 1) * 4 * kM;
        rs[m] = fpart;
        rs[kM + m] = g0;
        rs[2 * kM + m] = g1;
        rs[3 * kM + m] = g2;
        __syncwarp();
        if (lane == 0) mbar_arrive(redfull);
      } else {
        if (!bf16::warp_wait(redfull, (uint32_t)(tloc & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
#pragma unroll
        for (int hh = 0; hh < Q - 1; ++hh) {
          const float* rs = red + hh * 4 * kM;
          fpart = __fadd_rn(fpart, rs[m]);
          g0 = __fadd_rn(g0, rs[kM + m]);
          g1 = __fadd_rn(g1, rs[2 * kM + m]);
          g2 = __fadd_rn(g2, rs[3 * kM + m]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(redfree);
        if (p >= 0 && a.G) {
          const float gv[3] = {g0, g1, g2};
          for (int c = 0; c < 3; ++c) {
            float* gp = a.G + 3 * p + c;
            *gp = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(*gp, gv[c]) : gv[c];
          }
        }
        store_and_band(a, p >= 0, p, __fadd_rn(fpart, bout));
      }
      p = pn;
      x = xn;
      y = yn;
      z = zn;
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, int STAGES, int U, typename T>
int launch_cfg(const LevelArgs& a, cudaStream_t s) {
  using C = Cfg<WP, STAGES, U>;
  const size_t smem = C::bytes(a.lay.nh);
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_rgrad_kernel<WP, STAGES, U, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + kM - 1) / kM;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_rgrad_kernel<WP, STAGES, U, T><<<(unsigned)grid, bf16::Epi<U>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// the deepest weight ring that fits; MPL_ERR_UNSUPPORTED when the level has
// more than two hidden GEMMs or its constants do not fit (the caller falls
// back to the forward-mode gradient)
template <int WP, int U, typename T>
int launch_wp(const LevelArgs& a, cudaStream_t s) {
  constexpr size_t kLimit = 227 * 1024;
  if (a.lay.nh < 1 || a.lay.nh > 2) return MPL_ERR_UNSUPPORTED;
  if (Cfg<WP, 4, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, 4, U, T>(a, s);
  if (Cfg<WP, 3, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, 3, U, T>(a, s);
  if (Cfg<WP, 2, U>::bytes(a.lay.nh) <= kLimit) return launch_cfg<WP, 2, U, T>(a, s);
  return MPL_ERR_UNSUPPORTED;
}

// U: the epilogue unit width of the forward kernels (MPL_OPT_BF16_EPILOGUE_UNIT),
// whose output-dot partial sums S must equal bit for bit
template <int U, typename T>
int launch(const LevelArgs& a, cudaStream_t s) {
  switch (a.lay.WP) {
    case 64: return launch_wp<64, U, T>(a, s);
    case 128: return launch_wp<128, U, T>(a, s);
    case 256: return launch_wp<256, U, T>(a, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace rgrad
}  // namespace mpl
