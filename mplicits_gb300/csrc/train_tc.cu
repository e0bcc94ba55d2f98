// BF16 tensor-core training step of one level (sm_103a): the residual
// trainer's forward, loss (i3d/loss_functions.py:347-394), double backward
// and weight gradients, in three launches.
//
// 1. train_tc_kernel: one persistent CTA per SM walks 32-point tiles
//    (128 rows: value, d/dx, d/dy, d/dz of each point).  Per tile:
//      forward    layer 0 (FP32 SIMT) -> GEMM_1 -> ... -> GEMM_nh on tcgen05
//                 (BF16 operands, FP32 accumulators in TMEM) -> output dot;
//      loss       per point from f, df/dx, the frozen levels' sums and the
//                 targets; its seeds dL/df, dL/d(df/dx) start the backward;
//      backward   dz_l from ds_l and the layer's accumulators z_l, which stay
//                 in TMEM from the forward (the sines are recomputed from z,
//                 not stored), then ds_(l-1) = dz_l (omega_l W_l) on tcgen05
//                 against the transposed weight tiles; layer 0 last.
//    The BF16 A operands of the forward GEMMs (activations s_l) and of the
//    backward GEMMs (adjoints dz_l) are also written to HBM, tiled for the
//    weight-gradient GEMM.
// 2. train_tc_wgrad_kernel: dW_l = omega_l * sum_rows dz_l (x) s_(l-1), a
//    GEMM over rows (K = rows) on tcgen05 with both operands MN-major, split
//    over row blocks, partial sums added atomically.
// 3. train_tc_ends_kernel: biases, layer 0 and the output layer (SIMT).
//
// With z = omega (W s + b) the pre-activation (omega folded), value row
// s = sin z_v, tangent rows s = cos(z_v) zt.  Backward, given ds:
//   dzt = cos(z_v) ds_t,  dz_v = cos(z_v) ds_v - sin(z_v) sum_k ds_tk zt_k,
//   d(omega W) += dz (x) s_prev,  d(omega b) += dz_v,  ds_prev = dz (omega W).
// Every device wait is bounded; a wait that gives up records
// MPL_ERR_DEVICE_TIMEOUT and all roles leave their loops.
#include <string.h>

#include <mutex>

#include "level_bf16.cuh"
#include "train_loss.cuh"

namespace mpl {
namespace ttc {

using bf16::kKC;
using bf16::kM;
constexpr int kPts = kM / 4;

// Element offset of (row, feature f) in a tile buffer of the weight-gradient
// layout: 64-row blocks, inside a block [f/8][(row%64)/8][row%8][f%8], i.e.
// MN-major core matrices (8 rows x 16 bytes of 8 features) for K = rows.
__device__ __forceinline__ int64_t wg_offset(int64_t row, int f, int WP) {
  return (row >> 6) * (int64_t)(64 * WP) + (int64_t)(f >> 3) * 512 + ((row & 63) >> 3) * 64 +
         (row & 7) * 8 + (f & 7);
}

struct Args {
  const char* packed;
  PackLayout lay;
  int64_t n;
  const float* xyz;
  const float* Ff;     // nullable [n]
  const float* Gf;     // nullable [n][3]
  const float* gt_sdf;
  const float* gt_n;
  LossParams L;
  __nv_bfloat16* s_tiles;   // [nh + 1][rows_pad * WP]
  __nv_bfloat16* dz_tiles;  // [nh + 1][rows_pad * WP]
  float* seeds;             // [n][4]
  float* loss;              // [4]
  int64_t rows_pad;
  int* status;
};

template <int WP, int STAGES, int U>
struct Cfg {
  static constexpr int NC = WP / kKC;
  static constexpr int Q = 64 / U;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t oA = 0;
  static constexpr uint32_t oW = kM * WP * 2;
  static constexpr uint32_t oW0 = oW + STAGES * kStageBytes;
  static constexpr uint32_t oWout = oW0 + WP * 16;
  static constexpr uint32_t oRed = oWout + WP * 4;
  static constexpr uint32_t oSeed = oRed + (Q > 1 ? Q - 1 : 1) * kM * 4;
  static constexpr uint32_t oBar = oSeed + kM * 4;
  static constexpr uint32_t kNumBars = 2 * STAGES + bf16::kMaxNC + 1 + 2 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr uint32_t oAx = (oMisc + 16 + 1023) & ~1023u;
  static constexpr uint32_t oBx = oAx + kM * 16 * 2;
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  static size_t bytes(int nh) { return oBx + (size_t)nh * kBxBytes; }
};

__host__ __device__ inline uint32_t tmem_cols_for(int cols) {
  uint32_t c = 32;
  while (c < (uint32_t)cols) c <<= 1;
  return c;
}

// U values of row m, features j0.. -> BF16 A operand chunk in smem and the
// same 16-byte words into a weight-gradient tile in HBM.
template <int U>
__device__ __forceinline__ void store_unit(uint8_t* sA, __nv_bfloat16* g, int64_t grow, int m,
                                           int j0, int WP, const float (&v)[U]) {
#pragma unroll
  for (int gq = 0; gq < U / 8; ++gq) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      w[i] = bf16::Operand<__nv_bfloat16>::pack(v[gq * 8 + 2 * i], v[gq * 8 + 2 * i + 1]);
    const uint4 word = make_uint4(w[0], w[1], w[2], w[3]);
    const int k8 = (j0 >> 3) + gq;
    if (sA) {
      const uint32_t off = (uint32_t)((k8 * 16 + (m >> 3)) * 128 + (m & 7) * 16);
      *reinterpret_cast<uint4*>(sA + off) = word;
    }
    *reinterpret_cast<uint4*>(g + wg_offset(grow, k8 * 8, WP)) = word;
  }
}

template <int WP, int STAGES, int U>
__global__ void __launch_bounds__(bf16::Epi<U>::kThreads, 1) train_tc_kernel(const Args a) {
  using C = Cfg<WP, STAGES, U>;
  using E = bf16::Epi<U>;
  using T = __nv_bfloat16;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kEpiThreads = kEpiWarps * 32;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int NC = C::NC;
  constexpr int S = STAGES;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
  constexpr float kHalfPi = 1.57079632679489662f;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  float* w0s = reinterpret_cast<float*>(smem + C::oW0);  // [4][WP]
  float* wout = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  float* seedbuf = reinterpret_cast<float*>(smem + C::oSeed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;
  uint64_t* wempty = bars + S;
  uint64_t* achunk = bars + 2 * S;
  uint64_t* dfull = achunk + bf16::kMaxNC;
  uint64_t* freeacc = dfull + 1;  // [2]
  uint64_t* finalb = freeacc + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  uint8_t* sAx = smem + C::oAx;
  uint8_t* sBx = smem + C::oBx;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nh = a.lay.nh;
  const int ngemm = 2 * nh;
  const int64_t ntiles = (a.n + kPts - 1) / kPts;
  if ((int64_t)blockIdx.x >= ntiles) return;
  const uint32_t tcols = tmem_cols_for(nh * WP);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    for (int c = 0; c < bf16::kMaxNC; ++c) mbar_init(&achunk[c], kEpiWarps);
    mbar_init(dfull, 1);
    mbar_init(&freeacc[0], kEpiWarps);
    mbar_init(&freeacc[1], kEpiWarps);
    mbar_init(finalb, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tmem_slot, tcols);
  const char* pk = a.packed;
  {
    const float4* g0 = reinterpret_cast<const float4*>(pk + a.lay.w0f);
    for (int i = threadIdx.x; i < WP; i += kThreads) {
      reinterpret_cast<float4*>(w0s)[i] = g0[i];
      wout[i] = reinterpret_cast<const float*>(pk + a.lay.wout)[i];
    }
    for (int l = 1; l <= nh; ++l) {
      const uint4* gb = reinterpret_cast<const uint4*>(pk + a.lay.hbx[l]);
      uint4* db = reinterpret_cast<uint4*>(sBx + (l - 1) * C::kBxBytes);
      for (int i = threadIdx.x; i < (int)(C::kBxBytes / 16); i += kThreads) db[i] = gb[i];
    }
    // ones tile: only value rows (m % 4 == 0) carry the bias
    for (int i = threadIdx.x; i < kM * 16; i += kThreads) {
      const int m = i >> 4, k = i & 15;
      const bool one = k < 2 && (m & 3) == 0;
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

  if (warp == kTmaWarp) {
    // ================= TMA: forward then transposed weights, per tile ======
    if (lane == 0) {
      int64_t w = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok && !*abort_flag; t += gridDim.x) {
        for (int gi = 0; gi < ngemm && ok; ++gi) {
          const char* src = gi < nh ? pk + a.lay.hw[gi + 1] : pk + a.lay.hwT[2 * nh - gi];
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
      const uint64_t aDesc = tc::smem_desc(smem_u32(sA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      const uint64_t bxDesc = tc::smem_desc(smem_u32(sBx), 128u, 256u);
      int64_t w = 0, g = 0;
      int64_t uses0 = 0, uses1 = 0;  // GEMMs issued into each accumulator
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int gi = 0; gi < ngemm && ok; ++gi, ++g) {
          const int acc = gi < nh ? gi : nh - 1;
          const int64_t used = acc ? uses1 : uses0;
          if (used > 0 &&
              !bf16::mbar_wait_abort(&freeacc[acc], (uint32_t)((used - 1) & 1), a.status,
                                     abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(acc * WP);
          bool acc_on = false;
          if (gi < nh) {
            tc::mma_bf16(d_tmem, xDesc, bxDesc + (uint64_t)((gi * C::kBxBytes) >> 4), IDESC, false);
            acc_on = true;
          }
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            if (!bf16::mbar_wait_abort(&achunk[c], (uint32_t)(g & 1), a.status, abort_flag) ||
                !bf16::mbar_wait_abort(&wfull[s], (uint32_t)((w / S) & 1), a.status,
                                       abort_flag)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const uint64_t aC = aDesc + (uint64_t)((c * 8 * 2048) >> 4);
            const uint64_t wC = wDesc + (uint64_t)((s * C::kStageBytes) >> 4);
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks) {
              tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                           wC + (uint64_t)((ks * 256) >> 4), IDESC, acc_on);
              acc_on = true;
            }
            tc::commit(&wempty[s]);
          }
          if (!ok) break;
          tc::commit(dfull);
          if (acc)
            ++uses1;
          else
            ++uses0;
        }
      }
      tc::commit(finalb);
      mbar_wait(finalb, 0u, a.status);
    }
  } else {
    // ================= epilogue warps =====================================
    const int q = warp & 3, h = warp >> 2;
    const int m = 32 * q + lane;
    const int ch = m & 3;
    const int vlane = lane & ~3;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    const int64_t lstride = a.rows_pad * WP;  // elements per layer in the tile buffers
    int64_t g = 0;
    float lsum[4] = {0.f, 0.f, 0.f, 0.f};
    bool fail = false;
    float x = 0.f, y = 0.f, z = 0.f;
    bool valid = false;

    // layer 0 of tile t: A operand chunks and the s_0 tile
    auto layer0 = [&](int64_t t) {
      const int64_t qp = t * kPts + (m >> 2);
      valid = qp < a.n;
      x = y = z = 0.f;
      if (valid) {
        x = a.xyz[3 * qp + 0];
        y = a.xyz[3 * qp + 1];
        z = a.xyz[3 * qp + 2];
      }
      const int64_t grow = t * kM + m;
      for (int c = 0; c < NC; ++c) {
        const int j0 = c * kKC + h * U;
        float v[U];
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
            const float dz0 = ch == 1 ? ax[i] : (ch == 2 ? ay[i] : az[i]);
            const float sc = bf16::sin_fast(zz[i], ch ? kHalfPi : 0.f);
            v[4 * j4 + i] = ch ? __fmul_rn(sc, dz0) : sc;
          }
        }
        store_unit<U>(sA, a.s_tiles, grow, m, j0, WP, v);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&achunk[c]);
      }
    };

    layer0(blockIdx.x);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int64_t qp = t * kPts + (m >> 2);
      const int64_t grow = t * kM + m;
      float part = 0.f;
      // ---- forward GEMMs
      for (int l = 1; l <= nh && !fail; ++l, ++g) {
        if (!bf16::warp_wait(dfull, (uint32_t)(g & 1), a.status, abort_flag)) {
          fail = true;
          break;
        }
        tc::fence_after_sync();
        const uint32_t taddr = tl + (uint32_t)((l - 1) * WP);
        __nv_bfloat16* sg = a.s_tiles + (int64_t)l * lstride;
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
            float v[U];
#pragma unroll
            for (int jj = 0; jj < U; ++jj) {
              const float acc = __uint_as_float(r2[u][jj]);
              const float zv = __shfl_sync(0xffffffffu, acc, vlane);
              const float sc = bf16::sin_fast(zv, ch ? kHalfPi : 0.f);
              v[jj] = ch ? __fmul_rn(sc, acc) : sc;
            }
            if (l < nh) {
              store_unit<U>(sA, sg, grow, m, j0, WP, v);
              fence_proxy_async_smem();
              __syncwarp();
              if (lane == 0) mbar_arrive(&achunk[c]);
            } else {
              store_unit<U>(nullptr, sg, grow, m, j0, WP, v);
#pragma unroll
              for (int jj = 0; jj < U; ++jj) part = __fmaf_rn(v[jj], wout[j0 + jj], part);
            }
          }
        }
      }
      // ---- output dot over the feature splits, loss and seeds
      if (h > 0 && !fail) red[(h - 1) * kM + m] = part;
      if (bf16::epi_any(fail, kEpiThreads)) break;
      if (h == 0) {
        float tot = part;
#pragma unroll
        for (int hh = 0; hh < Q - 1; ++hh) tot = __fadd_rn(tot, red[hh * kM + m]);
        if (ch == 0) tot = __fadd_rn(tot, bout);
        const float f = __shfl_sync(0xffffffffu, tot, vlane);
        const float gx = __shfl_sync(0xffffffffu, tot, vlane + 1);
        const float gy = __shfl_sync(0xffffffffu, tot, vlane + 2);
        const float gz = __shfl_sync(0xffffffffu, tot, vlane + 3);
        float phi = 0.f, gam0 = 0.f, gam1 = 0.f, gam2 = 0.f;
        if (valid && ch == 0) {
          const float Sv = __fadd_rn(f, a.Ff ? a.Ff[qp] : 0.f);
          const float G[3] = {__fadd_rn(gx, a.Gf ? a.Gf[3 * qp + 0] : 0.f),
                              __fadd_rn(gy, a.Gf ? a.Gf[3 * qp + 1] : 0.f),
                              __fadd_rn(gz, a.Gf ? a.Gf[3 * qp + 2] : 0.f)};
          const float N[3] = {a.gt_n[3 * qp + 0], a.gt_n[3 * qp + 1], a.gt_n[3 * qp + 2]};
          float gam[3], term[4];
          point_loss(a.L, Sv, G, a.gt_sdf[qp], N, phi, gam, term);
          gam0 = gam[0];
          gam1 = gam[1];
          gam2 = gam[2];
#pragma unroll
          for (int k = 0; k < 4; ++k) lsum[k] += term[k];
          *reinterpret_cast<float4*>(a.seeds + 4 * qp) = make_float4(phi, gam0, gam1, gam2);
        }
        const float s_phi = __shfl_sync(0xffffffffu, phi, vlane);
        const float s_g0 = __shfl_sync(0xffffffffu, gam0, vlane);
        const float s_g1 = __shfl_sync(0xffffffffu, gam1, vlane);
        const float s_g2 = __shfl_sync(0xffffffffu, gam2, vlane);
        const float mine = ch == 0 ? s_phi : (ch == 1 ? s_g0 : (ch == 2 ? s_g1 : s_g2));
        seedbuf[m] = valid ? mine : 0.f;
      }
      if (bf16::epi_any(false, kEpiThreads)) break;
      const float seed = seedbuf[m];

      // ---- backward: dz_l from ds_l and z_l, then GEMM ds_(l-1) = dz_l (omega W_l)
      for (int l = nh; l >= 1 && !fail; --l) {
        if (l < nh) {
          if (!bf16::warp_wait(dfull, (uint32_t)(g & 1), a.status, abort_flag)) {
            fail = true;
            break;
          }
          ++g;
          tc::fence_after_sync();
        }
        const uint32_t zaddr = tl + (uint32_t)((l - 1) * WP);
        const uint32_t daddr = tl + (uint32_t)((nh - 1) * WP);
        __nv_bfloat16* dg = a.dz_tiles + (int64_t)l * lstride;
#pragma unroll 1
        for (int c = 0; c < NC; ++c) {
          const int j0 = c * kKC + h * U;
          uint32_t zr[U], dr[U];
          tc::ld_32x32b<U>(zaddr + (uint32_t)j0, zr);
          if (l < nh) tc::ld_32x32b<U>(daddr + (uint32_t)j0, dr);
          tc::wait_ld();
          float v[U];
#pragma unroll
          for (int jj = 0; jj < U; ++jj) {
            const float zo = __uint_as_float(zr[jj]);
            const float zv = __shfl_sync(0xffffffffu, zo, vlane);
            const float ds = l < nh ? __uint_as_float(dr[jj]) : __fmul_rn(seed, wout[j0 + jj]);
            float tt = ch ? __fmul_rn(ds, zo) : 0.f;
            tt = __fadd_rn(tt, __shfl_xor_sync(0xffffffffu, tt, 1));
            tt = __fadd_rn(tt, __shfl_xor_sync(0xffffffffu, tt, 2));
            const float cv = bf16::sin_fast(zv, kHalfPi);
            const float sv = bf16::sin_fast(zv);
            const float dz = ch ? __fmul_rn(cv, ds) : __fsub_rn(__fmul_rn(cv, ds), __fmul_rn(sv, tt));
            v[jj] = valid ? dz : 0.f;
          }
          store_unit<U>(sA, dg, grow, m, j0, WP, v);
          fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) mbar_arrive(&achunk[c]);
        }
        // z_l (and ds_l) have been read for the last time
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&freeacc[l - 1]);
          if (l < nh && l - 1 != nh - 1) mbar_arrive(&freeacc[nh - 1]);
        }
      }
      // ---- layer 0: dz_0 from ds_0 and the recomputed first-layer phase
      if (!fail) {
        if (!bf16::warp_wait(dfull, (uint32_t)(g & 1), a.status, abort_flag)) {
          fail = true;
        } else {
          ++g;
          tc::fence_after_sync();
          const uint32_t daddr = tl + (uint32_t)((nh - 1) * WP);
          __nv_bfloat16* dg = a.dz_tiles;
#pragma unroll 1
          for (int c = 0; c < NC; ++c) {
            const int j0 = c * kKC + h * U;
            uint32_t dr[U];
            tc::ld_32x32b<U>(daddr + (uint32_t)j0, dr);
            tc::wait_ld();
            float v[U];
#pragma unroll
            for (int j4 = 0; j4 < U / 4; ++j4) {
              float zq[4];
              float4 wx, wy, wz;
              bf16::phase4(w0s, WP, j0 + 4 * j4, x, y, z, zq, wx, wy, wz);
              const float ax[4] = {wx.x, wx.y, wx.z, wx.w};
              const float ay[4] = {wy.x, wy.y, wy.z, wy.w};
              const float az[4] = {wz.x, wz.y, wz.z, wz.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const int jj = 4 * j4 + i;
                const float zv = zq[i];
                const float zt = ch == 1 ? ax[i] : (ch == 2 ? ay[i] : az[i]);
                const float ds = __uint_as_float(dr[jj]);
                float tt = ch ? __fmul_rn(ds, zt) : 0.f;
                tt = __fadd_rn(tt, __shfl_xor_sync(0xffffffffu, tt, 1));
                tt = __fadd_rn(tt, __shfl_xor_sync(0xffffffffu, tt, 2));
                const float cv = bf16::sin_fast(zv, kHalfPi);
                const float sv = bf16::sin_fast(zv);
                const float dz =
                    ch ? __fmul_rn(cv, ds) : __fsub_rn(__fmul_rn(cv, ds), __fmul_rn(sv, tt));
                v[jj] = valid ? dz : 0.f;
              }
            }
            store_unit<U>(nullptr, dg, grow, m, j0, WP, v);
          }
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) mbar_arrive(&freeacc[nh - 1]);
        }
      }
      // ---- next tile's layer 0 (the A operand is free: its last GEMM completed)
      const int64_t tn = t + gridDim.x;
      if (!fail && tn < ntiles) layer0(tn);
    }
    // loss sums of this CTA
    if (h == 0) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float v = lsum[k];
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.f) atomicAdd(&a.loss[k], v);
      }
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, tcols);
}

// ---------------------------------------------------------------------------
// Weight gradients of the hidden layers: for job l, dW_l[j][k] +=
// omega_l * sum_rows dz_l[row][j] * s_(l-1)[row][k].  M = j (one or two
// 128-row halves, one TMEM accumulator each), N = k, K = rows in 64-row
// blocks.  Warps 0-3 read the accumulators out, warp 4 issues the MMAs,
// warp 5 the bulk copies.
// ---------------------------------------------------------------------------
constexpr int kWgStages = 3;

struct WgArgs {
  const __nv_bfloat16* A[MPL_MAX_LAYERS];  // dz_l tiles per job
  const __nv_bfloat16* B[MPL_MAX_LAYERS];  // s_(l-1) tiles per job
  float* dW[MPL_MAX_LAYERS];
  float omega[MPL_MAX_LAYERS];
  int64_t nblocks;  // 64-row blocks
  int* status;
};

template <int WP>
__global__ void __launch_bounds__(192, 1) train_tc_wgrad_kernel(const WgArgs w) {
  constexpr int H = WP / 128;                   // M halves
  constexpr uint32_t kOpBytes = 64 * WP * 2;    // one operand block
  constexpr uint32_t kStage = 2 * kOpBytes;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32_major(128, WP, 1u, true, true);
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kWgStages * kStage);
  uint64_t* full = bars;
  uint64_t* empty = bars + kWgStages;
  uint64_t* done = bars + 2 * kWgStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int job = blockIdx.y;
  const int64_t per = (w.nblocks + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * per;
  const int64_t b1 = b0 + per < w.nblocks ? b0 + per : w.nblocks;
  if (b0 >= b1) return;
  constexpr uint32_t kCols = H * WP;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kWgStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 4) tc::tmem_alloc(tmem_slot, kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint8_t* gA = reinterpret_cast<const uint8_t*>(w.A[job]);
  const uint8_t* gB = reinterpret_cast<const uint8_t*>(w.B[job]);

  if (warp == 5) {
    if (lane == 0) {
      int64_t i = 0;
      for (int64_t b = b0; b < b1; ++b, ++i) {
        const int s = (int)(i % kWgStages);
        const int64_t u = i / kWgStages;
        if (u > 0 && !bf16::mbar_wait_abort(&empty[s], (uint32_t)((u - 1) & 1), w.status,
                                            abort_flag))
          break;
        mbar_arrive_expect_tx(&full[s], kStage);
        tma_bulk_g2s(smem + s * kStage, gA + b * kOpBytes, kOpBytes, &full[s]);
        tma_bulk_g2s(smem + s * kStage + kOpBytes, gB + b * kOpBytes, kOpBytes, &full[s]);
      }
      const int64_t first = i > kWgStages ? i - kWgStages : 0;
      for (int64_t v = first; v < i; ++v)
        mbar_wait(&full[v % kWgStages], (uint32_t)((v / kWgStages) & 1), w.status);
    }
  } else if (warp == 4) {
    if (lane == 0) {
      const uint32_t base = smem_u32(smem);
      int64_t i = 0;
      bool acc_on = false;
      for (int64_t b = b0; b < b1; ++b, ++i) {
        const int s = (int)(i % kWgStages);
        if (!bf16::mbar_wait_abort(&full[s], (uint32_t)((i / kWgStages) & 1), w.status,
                                   abort_flag))
          break;
        tc::fence_after_sync();
        const uint32_t sa = base + (uint32_t)s * kStage;
        const uint32_t sb = sa + kOpBytes;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
          for (int hh = 0; hh < H; ++hh) {
            const uint64_t ad = tc::smem_desc(sa + (uint32_t)hh * 16u * 1024u + (uint32_t)ks * 256u,
                                              128u, 1024u);
            const uint64_t bd = tc::smem_desc(sb + (uint32_t)ks * 256u, 128u, 1024u);
            tc::mma_bf16(tmem + (uint32_t)(hh * WP), ad, bd, IDESC, acc_on);
          }
          acc_on = true;
        }
        tc::commit(&empty[s]);
      }
      tc::commit(done);
    }
  } else {
    // read-out: warp q owns TMEM lanes 32q..32q+31, i.e. j = 128 hh + 32 q + lane
    const bool ok = bf16::warp_wait(done, 0u, w.status, abort_flag);
    if (ok) {
      tc::fence_after_sync();
      float* dW = w.dW[job];
      const float om = w.omega[job];
      for (int hh = 0; hh < H; ++hh) {
        const int j = 128 * hh + 32 * warp + lane;
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(hh * WP);
#pragma unroll 1
        for (int k0 = 0; k0 < WP; k0 += 32) {
          uint32_t r[32];
          tc::ld_32x32b_x32(taddr + (uint32_t)k0, r);
          tc::wait_ld();
#pragma unroll
          for (int kk = 0; kk < 32; kk += 4)
            atomicAdd(reinterpret_cast<float4*>(dW + (int64_t)j * WP + k0 + kk),
                      make_float4(__fmul_rn(om, __uint_as_float(r[kk])),
                                  __fmul_rn(om, __uint_as_float(r[kk + 1])),
                                  __fmul_rn(om, __uint_as_float(r[kk + 2])),
                                  __fmul_rn(om, __uint_as_float(r[kk + 3]))));
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 4) tc::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------------------
// Biases, layer 0 and the output layer from the tiles:
//   db_l[j]  += omega_l * sum_points dz_l[value row][j]        (l = 0..nh)
//   dW0[j][c] += omega_0 * sum_points (dz_0[v][j] x_c + dz_0[t_c][j])
//   dWL[j]   += sum_rows seed_row * s_nh[row][j],  dbL += sum_points seed_v.
// Block (f8, split): features 8 f8 .. 8 f8 + 7.  Each warp walks 64-row
// blocks, lane l taking rows l and l + 32, so a warp reads 512 contiguous
// bytes per operand (one 8-feature column of a block is 1 KiB contiguous).
// Lanes keep their partial sums across blocks; one warp reduction and one
// atomic per value at the end.
// ---------------------------------------------------------------------------
struct EndsArgs {
  const __nv_bfloat16* dz;  // layer 0 of the dz tiles; layer l at + l * lstride
  const __nv_bfloat16* s_last;
  const float* seeds;
  const float* xyz;
  int64_t n, nblocks, lstride;
  int WP, nh;
  float omega[MPL_MAX_LAYERS];
  float* dW0;
  float* db[MPL_MAX_LAYERS];
  float* dWL;
  float* dbL;
};

__device__ __forceinline__ void add8(float (&acc)[8], const uint4& v) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    acc[2 * i] += f.x;
    acc[2 * i + 1] += f.y;
  }
}

__device__ __forceinline__ void fma8(float (&acc)[8], const uint4& v, float s) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    acc[2 * i] = __fmaf_rn(s, f.x, acc[2 * i]);
    acc[2 * i + 1] = __fmaf_rn(s, f.y, acc[2 * i + 1]);
  }
}

constexpr int kEndsWarps = 8;
constexpr int kEndsQ = 3 + 3 + 1;  // db_0..db_2, dW0 x/y/z, dWL

__global__ void __launch_bounds__(kEndsWarps * 32, 2) train_tc_ends_kernel(const EndsArgs e) {
  __shared__ float part[kEndsWarps][kEndsQ * 8 + 1];
  const int WP = e.WP, nh = e.nh;
  const int f8 = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[kEndsQ][8];
  float dbl = 0.f;
#pragma unroll
  for (int qq = 0; qq < kEndsQ; ++qq)
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[qq][i] = 0.f;
  // one 64-row block per iteration, two rows per lane: every load of an
  // iteration is issued before the arithmetic that uses it, and two CTAs
  // fit on an SM (128 registers a thread)
  const int64_t stride = (int64_t)gridDim.y * kEndsWarps;
  for (int64_t b0 = (int64_t)blockIdx.y * kEndsWarps + warp; b0 < e.nblocks; b0 += stride) {
    uint4 sv[2], dv[2], d1[2], d2[2];
    float sd[2], cx[2], cy[2], cz[2];
    int64_t rowv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t b = b0 + (u >> 1) * stride;
      const int64_t row = b * 64 + lane + 32 * (u & 1);
      rowv[u] = (b < e.nblocks && (row >> 2) < e.n) ? row : -1;
      if (rowv[u] < 0) continue;
      const int64_t p = row >> 2;
      const int ch = (int)(row & 3);
      const int64_t off = wg_offset(row, f8 * 8, WP);
      sd[u] = e.seeds[4 * p + ch];
      sv[u] = *reinterpret_cast<const uint4*>(e.s_last + off);
      dv[u] = *reinterpret_cast<const uint4*>(e.dz + off);
      if (ch == 0) {
        d1[u] = *reinterpret_cast<const uint4*>(e.dz + e.lstride + off);
        if (nh > 1) d2[u] = *reinterpret_cast<const uint4*>(e.dz + 2 * e.lstride + off);
        cx[u] = e.xyz[3 * p + 0];
        cy[u] = e.xyz[3 * p + 1];
        cz[u] = e.xyz[3 * p + 2];
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (rowv[u] < 0) continue;
      const int ch = (int)(rowv[u] & 3);
      fma8(acc[6], sv[u], sd[u]);
      if (ch == 0) {
        dbl += sd[u];
        add8(acc[0], dv[u]);
        fma8(acc[3], dv[u], cx[u]);
        fma8(acc[4], dv[u], cy[u]);
        fma8(acc[5], dv[u], cz[u]);
        add8(acc[1], d1[u]);
        if (nh > 1) add8(acc[2], d2[u]);
      } else if (ch == 1) {
        add8(acc[3], dv[u]);
      } else if (ch == 2) {
        add8(acc[4], dv[u]);
      } else {
        add8(acc[5], dv[u]);
      }
    }
  }
#pragma unroll
  for (int qq = 0; qq < kEndsQ; ++qq)
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float v = acc[qq][i];
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) part[warp][qq * 8 + i] = v;
    }
  for (int o = 16; o >= 1; o >>= 1) dbl += __shfl_xor_sync(0xffffffffu, dbl, o);
  if (lane == 0) part[warp][kEndsQ * 8] = dbl;
  __syncthreads();
  for (int t = threadIdx.x; t < kEndsQ * 8 + 1; t += blockDim.x) {
    float v = 0.f;
    for (int w = 0; w < kEndsWarps; ++w) v += part[w][t];
    if (t == kEndsQ * 8) {
      if (f8 == 0) atomicAdd(e.dbL, v);
      continue;
    }
    const int qq = t >> 3, j = f8 * 8 + (t & 7);
    if (qq <= 2) {
      if (qq <= nh) atomicAdd(&e.db[qq][j], __fmul_rn(e.omega[qq], v));
    } else if (qq <= 5) {
      atomicAdd(&e.dW0[j * 3 + (qq - 3)], __fmul_rn(e.omega[0], v));
    } else {
      atomicAdd(&e.dWL[j], v);
    }
  }
}

template <int WP, int STAGES, int U>
int launch_fused(const Args& a, cudaStream_t s) {
  using C = Cfg<WP, STAGES, U>;
  const size_t smem = C::bytes(a.lay.nh);
  if (smem > 227 * 1024) return MPL_ERR_UNSUPPORTED;
  MPL_CUDA_TRY(cudaFuncSetAttribute(train_tc_kernel<WP, STAGES, U>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t ntiles = (a.n + kPts - 1) / kPts;
  int64_t grid = sm_count();
  grid = ntiles < grid ? ntiles : grid;
  train_tc_kernel<WP, STAGES, U><<<(unsigned)grid, bf16::Epi<U>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

template <int WP>
int launch_wgrad(const WgArgs& w, int jobs, cudaStream_t s) {
  const size_t smem = (size_t)kWgStages * 2 * 64 * WP * 2 + 64;
  MPL_CUDA_TRY(cudaFuncSetAttribute(train_tc_wgrad_kernel<WP>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t splits = sm_count() / (jobs > 0 ? jobs : 1);
  if (splits < 1) splits = 1;
  if (splits > w.nblocks) splits = w.nblocks;
  dim3 grid((unsigned)splits, (unsigned)jobs);
  train_tc_wgrad_kernel<WP><<<grid, 192, smem, s>>>(w);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

}  // namespace ttc
}  // namespace mpl

using namespace mpl;
using namespace mpl::ttc;

static int64_t tc_rows_pad(int64_t n) { return ((n + kPts - 1) / kPts) * kM; }

// A second stream per device (created once) on which the end-layer
// reductions run next to the weight-gradient GEMM: both read the tiles the
// fused kernel wrote, the GEMM at most of the DRAM bandwidth and the
// reductions latency-bound, and both fit on an SM together.  Fork and join
// are events, so the pair also works inside a captured CUDA graph.
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

static int side_stream(SideStream** out) {
  static SideStream per_device[64];
  static std::mutex mu;
  int dev = 0;
  MPL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return MPL_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> guard(mu);
  SideStream& ss = per_device[dev];
  if (!ss.s) {
    MPL_CUDA_TRY(cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking));
    MPL_CUDA_TRY(cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming));
    MPL_CUDA_TRY(cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming));
  }
  *out = &ss;
  return MPL_OK;
}

extern "C" int mpl_train_tc_scratch_bytes(const MplNet* net, int64_t n, int64_t* bytes) {
  PackLayout lay;
  int st = make_layout(net, &lay);
  if (st != MPL_OK) return st;
  if (!bytes || n < 0) return MPL_ERR_INVALID_ARG;
  *bytes = 2 * (int64_t)(lay.nh + 1) * tc_rows_pad(n) * lay.WP * 2;
  return MPL_OK;
}

extern "C" int mpl_train_tc_step(const MplNet* net, const void* packed, const float* xyz,
                                 int64_t n, const float* f_frozen, const float* g_frozen,
                                 const float* gt_sdf, const float* gt_normals,
                                 const MplLoss* loss, void* scratch,
                                 int64_t scratch_bytes, float* seeds, float* loss_sums,
                                 float* const* dW, float* const* db, void* stream) {
  if (!net || !packed || !gt_sdf || !gt_normals || !seeds || !loss_sums || !dW || !db || n < 0 ||
      n > INT32_MAX / 4 || (n > 0 && (!xyz || !scratch)))
    return MPL_ERR_INVALID_ARG;
  if (((uintptr_t)packed & 255) != 0 || ((uintptr_t)scratch & 255) != 0 ||
      ((uintptr_t)seeds & 15) != 0)
    return MPL_ERR_INVALID_ARG;
  Args a;
  memset(&a, 0, sizeof(a));
  int st = make_layout(net, &a.lay);
  if (st != MPL_OK) return st;
  st = loss_params(loss, n, &a.L);
  if (st != MPL_OK) return st;
  const int nh = a.lay.nh, WP = a.lay.WP, L = a.lay.L;
  if (nh < 1 || nh > 2 || (WP != 128 && WP != 256)) return MPL_ERR_UNSUPPORTED;
  for (int l = 0; l < L; ++l)
    if (!dW[l] || !db[l]) return MPL_ERR_INVALID_ARG;
  int64_t need = 0;
  mpl_train_tc_scratch_bytes(net, n, &need);
  if (scratch_bytes < need) return MPL_ERR_CAPACITY;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(loss_sums, 0, 4 * sizeof(float), s));
  if (n == 0) return MPL_OK;
  const int64_t rows_pad = tc_rows_pad(n);
  const int64_t lstride = rows_pad * WP;
  a.packed = (const char*)packed;
  a.n = n;
  a.xyz = xyz;
  a.Ff = f_frozen;
  a.Gf = g_frozen;
  a.gt_sdf = gt_sdf;
  a.gt_n = gt_normals;
  a.s_tiles = (__nv_bfloat16*)scratch;
  a.dz_tiles = a.s_tiles + (int64_t)(nh + 1) * lstride;
  a.seeds = seeds;
  a.loss = loss_sums;
  a.rows_pad = rows_pad;
  a.status = device_status_ptr();
  // 16-wide epilogue units: twice the epilogue warps of the 32-wide form for
  // this latency-bound kernel (2.24 against 2.51 ms for the 196,608-row step)
  st = WP == 256 ? launch_fused<256, 4, 16>(a, s) : launch_fused<128, 6, 16>(a, s);
  if (st != MPL_OK) return st;
  // hidden-layer weight gradients
  WgArgs w;
  memset(&w, 0, sizeof(w));
  for (int l = 1; l <= nh; ++l) {
    w.A[l - 1] = a.dz_tiles + (int64_t)l * lstride;
    w.B[l - 1] = a.s_tiles + (int64_t)(l - 1) * lstride;
    w.dW[l - 1] = dW[l];
    w.omega[l - 1] = net->omega[l];
  }
  w.nblocks = rows_pad / 64;
  w.status = a.status;
  SideStream* side = nullptr;
  st = side_stream(&side);
  if (st != MPL_OK) return st;
  MPL_CUDA_TRY(cudaEventRecord(side->fork, s));
  MPL_CUDA_TRY(cudaStreamWaitEvent(side->s, side->fork, 0));
  st = WP == 256 ? launch_wgrad<256>(w, nh, s) : launch_wgrad<128>(w, nh, s);
  if (st != MPL_OK) return st;
  // biases, layer 0, output layer
  EndsArgs e;
  memset(&e, 0, sizeof(e));
  e.dz = a.dz_tiles;
  e.s_last = a.s_tiles + (int64_t)nh * lstride;
  e.seeds = seeds;
  e.xyz = xyz;
  e.n = n;
  e.nblocks = rows_pad / 64;
  e.lstride = lstride;
  e.WP = WP;
  e.nh = nh;
  for (int l = 0; l <= nh; ++l) {
    e.omega[l] = net->omega[l];
    e.db[l] = db[l];
  }
  e.dW0 = dW[0];
  e.dWL = dW[L - 1];
  e.dbL = db[L - 1];
  int64_t splits = (4 * (int64_t)sm_count()) / (WP / 8);
  const int64_t wmax = (e.nblocks + kEndsWarps - 1) / kEndsWarps;
  if (splits > wmax) splits = wmax;
  if (splits < 1) splits = 1;
  train_tc_ends_kernel<<<dim3((unsigned)(WP / 8), (unsigned)splits), kEndsWarps * 32, 0,
                         side->s>>>(e);
  MPL_LAUNCH_CHECK();
  MPL_CUDA_TRY(cudaEventRecord(side->join, side->s));
  MPL_CUDA_TRY(cudaStreamWaitEvent(s, side->join, 0));
  return MPL_OK;
}
