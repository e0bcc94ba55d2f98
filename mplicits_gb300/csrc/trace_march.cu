// Persistent sphere-tracing kernel on the tensor cores (sm_103a): all
// remaining steps of the marching rays in one launch.
//
// Late in a frame few rays are still marching, and each step of the
// launch-per-level loop of trace.cu then costs the fixed latency of one-tile
// passes through the level kernels and of their launches.  Here one CTA keeps
// a tile of 128 active rays for every remaining step.  Per step it evaluates
// the levels at the rays' positions -- level l > 0 accumulated only for rays
// whose partial sum lies inside band l - 1, as the band lists of the
// launch-per-level loop select them -- then advances, stops or records each
// ray with march_ray.  Per ray the arithmetic is that of the two-tile level
// kernel (FP32 first layer and sines, 16-bit GEMM operands, the same output
// reduction) and of trace_step_kernel, so a frame gives the same image.
//
// Roles (as the level kernels): 4*Q epilogue warps, one MMA-issuing warp,
// one TMA warp.  One accumulator and one A operand: GEMM k waits for its A
// operand (afull, written by the first layer or by the previous drain) and
// for the previous accumulator to be drained (dempty); the epilogue waits for
// dfull.  The weights of every level stream through one ring in the MMA's
// GEMM order (tile, step, level, layer).  The first layer of level l + 1 is
// written inside the last drain of level l (the rays have not moved).  The
// epilogue warps meet at a named barrier twice per step, once with every
// level's feature-split partial sums written and once after the marching
// step; its reduction carries the abort decision, so all of them leave
// together.
// Every mbarrier wait is bounded (the abort protocol of level_bf16.cuh).
#include <string.h>

#include "level_bf16.cuh"
#include "trace.cuh"

namespace mpl {
namespace march {

using bf16::kKC;
using bf16::kM;

constexpr int kMaxLevels = 3;
constexpr int kStages = 3;
constexpr int kMaxBiasLayers = 8;  // hidden layers whose biases share one K = 16 tile

struct Args {
  const char* packed[kMaxLevels];
  PackLayout lay[kMaxLevels];
  int32_t levels;
  float delta[kMaxLevels];  // band of level l + 1 around the partial sum of levels 0..l
  const int32_t* active;
  const int32_t* count;
  int64_t n_max;
  float* org;
  const float* dir;
  int32_t* state;
  float* S;
  float eps, R;
  int32_t steps;
  int32_t last_final;  // the last of these steps ends the step budget
  int32_t* hit_out;
  int32_t* hit_count;
  int64_t capacity;
  int* status;
};

template <int WP, int U>
struct Cfg {
  static constexpr int NC = WP / kKC;
  static constexpr int Q = 64 / U;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t oA = 0;
  static constexpr uint32_t oW = kABytes;                                // [S] weight chunks
  static constexpr uint32_t oW0 = oW + kStages * kStageBytes;          // float [levels][4][WP]
  static constexpr uint32_t oWout = oW0 + kMaxLevels * WP * 16;        // float [levels][WP]
  static constexpr uint32_t oRed = oWout + kMaxLevels * WP * 4;        // float [levels][Q][128]
  static constexpr uint32_t oPos = oRed + kMaxLevels * Q * kM * 4;    // float4 [128] x, y, z, alive
  static constexpr uint32_t oBar = oPos + kM * 16;
  static constexpr uint32_t kNumBars = 2 * kStages + 4;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;              // tmem slot, abort, bout[3]
  // the biases of every hidden layer j = level * nh + layer - 1 share one
  // bias tile (K columns 2j, 2j + 1: the two 16-bit pieces of omega*b); the
  // bias MMA of layer j multiplies it by ones tile j, which is 1 in those
  // two columns only
  static constexpr uint32_t oAx = (oMisc + 32 + 1023) & ~1023u;        // [levels*nh] ones tiles
  static constexpr uint32_t kOnesBytes = kM * 16 * 2;
  static constexpr uint32_t kBxBytes = WP * 16 * 2;
  __host__ __device__ static uint32_t oBx(int layers) { return oAx + (uint32_t)layers * kOnesBytes; }
  static size_t bytes(int levels, int nh) { return oBx(levels * nh) + kBxBytes; }
};

template <int WP, int U, typename T>
__global__ void __launch_bounds__(bf16::Epi<U>::kThreads, 1) trace_march_kernel(const Args a) {
  using C = Cfg<WP, U>;
  using E = bf16::Epi<U>;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int NC = C::NC;
  constexpr int S = kStages;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
  constexpr bool kF16 = Op::kFormat == 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  float* w0s = reinterpret_cast<float*>(smem + C::oW0);
  float* wouts = reinterpret_cast<float*>(smem + C::oWout);
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  float4* spos = reinterpret_cast<float4*>(smem + C::oPos);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;           // [S]  TMA -> MMA
  uint64_t* wempty = bars + S;      // [S]  MMA -> TMA
  uint64_t* afull = bars + 2 * S;   // A operand written (count: epilogue warps)
  uint64_t* dfull = afull + 1;      // accumulator ready
  uint64_t* dempty = dfull + 1;     // accumulator drained (count: epilogue warps)
  uint64_t* finalb = dempty + 1;    // last MMA commit
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  float* bouts = reinterpret_cast<float*>(smem + C::oMisc + 8);  // [levels] output biases
  uint8_t* sAx = smem + C::oAx;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int L = a.levels;
  const int nh = a.lay[0].nh;
  int64_t n = *a.count;
  n = n < a.n_max ? n : a.n_max;
  n = n < 0 ? 0 : n;
  const int64_t ntiles = (n + kM - 1) / kM;
  if ((int64_t)blockIdx.x >= ntiles) return;
  const int64_t G = gridDim.x;
  uint8_t* sBx = smem + C::oBx(L * nh);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    mbar_init(afull, kEpiWarps);
    mbar_init(dfull, 1);
    mbar_init(dempty, kEpiWarps);
    mbar_init(finalb, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tmem_slot, WP);
  for (int lev = 0; lev < L; ++lev) {
    const char* pk = a.packed[lev];
    const PackLayout& lay = a.lay[lev];
    const float4* g0 = reinterpret_cast<const float4*>(pk + lay.w0f);
    for (int i = threadIdx.x; i < WP; i += kThreads) {
      reinterpret_cast<float4*>(w0s + lev * 4 * WP)[i] = g0[i];
      wouts[lev * WP + i] = reinterpret_cast<const float*>(pk + lay.wout)[i];
    }
    if (threadIdx.x == 0) bouts[lev] = reinterpret_cast<const float*>(pk + lay.bout)[0];
  }
  // the shared bias tile: element (n, k) of a [WP rows][16 K] tile at
  // ((n/8)*2 + k/8)*128 + (n%8)*16 + (k%8)*2 bytes; layer j's pieces (its
  // own tile's K columns 0, 1) go to K columns 2j, 2j + 1
  for (int i = threadIdx.x; i < WP * 16; i += kThreads) {
    const int nn = i >> 4, kk = i & 15, j = kk >> 1;
    T v = Op::value(0.f);
    if (j < L * nh) {
      const int lev = j / nh, l = j % nh + 1;
      const T* src = reinterpret_cast<const T*>(
          a.packed[lev] + (kF16 ? a.lay[lev].hbxh[l] : a.lay[lev].hbx[l]));
      v = src[(((nn >> 3) * 2) * 128 + (nn & 7) * 16 + (kk & 1) * 2) / 2];
    }
    *reinterpret_cast<T*>(sBx + ((nn >> 3) * 2 + (kk >> 3)) * 128 + (nn & 7) * 16 + (kk & 7) * 2) = v;
  }
  for (int i = threadIdx.x; i < L * nh * kM * 16; i += kThreads) {
    const int j = i / (kM * 16), m = (i >> 4) & (kM - 1), k = i & 15;
    const uint32_t off = (uint32_t)(j * C::kOnesBytes + ((k >> 3) * 16 + (m >> 3)) * 128 +
                                    (m & 7) * 16 + (k & 7) * 2);
    *reinterpret_cast<T*>(sAx + off) = Op::value((k >> 1) == j ? 1.f : 0.f);
  }
  fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == kTmaWarp) {
    // ================= TMA: weight K chunks in the MMA's GEMM order ========
    if (lane == 0) {
      int64_t w = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok && !*abort_flag; t += G)
        for (int st = 0; st < a.steps && ok; ++st)
          for (int lev = 0; lev < L && ok; ++lev)
            for (int l = 1; l <= nh && ok; ++l) {
              const char* src = a.packed[lev] + (kF16 ? a.lay[lev].hwh[l] : a.lay[lev].hw[l]);
              for (int c = 0; c < NC; ++c, ++w) {
                const int s = (int)(w % S);
                const int64_t u = w / S;
                if (u > 0 && !bf16::mbar_wait_abort(&wempty[s], (uint32_t)((u - 1) & 1),
                                                    a.status, abort_flag)) {
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
    // ================= MMA issuer ==========================================
    if (lane == 0) {
      const uint64_t aDesc = tc::smem_desc(smem_u32(sA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      const uint64_t bxDesc = tc::smem_desc(smem_u32(sBx), 128u, 256u);
      int64_t w = 0, k = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += G)
        for (int st = 0; st < a.steps && ok; ++st)
          for (int lev = 0; lev < L && ok; ++lev)
            for (int l = 1; l <= nh && ok; ++l, ++k) {
              if ((k > 0 && !bf16::mbar_wait_abort(dempty, (uint32_t)((k - 1) & 1), a.status,
                                                   abort_flag)) ||
                  !bf16::mbar_wait_abort(afull, (uint32_t)(k & 1), a.status, abort_flag)) {
                ok = false;
                break;
              }
              tc::fence_after_sync();
              tc::mma_bf16(tmem, xDesc + (uint64_t)(((lev * nh + l - 1) * C::kOnesBytes) >> 4),
                           bxDesc, IDESC, false);
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
                  tc::mma_bf16(tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                               wC + (uint64_t)((ks * 256) >> 4), IDESC, true);
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
    constexpr int kEpiThreads = kEpiWarps * 32;
    int64_t k = 0;  // GEMMs drained
    bool fail = false;
    for (int64_t t = blockIdx.x; t < ntiles && !fail; t += G) {
      const int64_t qi = t * kM + m;
      const int64_t r = qi < n ? (int64_t)a.active[qi] : -1;
      // the h = 0 warps own the tile's rays: position, direction and state in
      // registers, the position shared with the other warps through smem;
      // the frame's arrays are written when a ray stops
      float o[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f};
      int ray_state = 2;
      if (h == 0) {
        if (r >= 0) {
          ray_state = a.state[r];
          for (int c = 0; c < 3; ++c) {
            o[c] = a.org[3 * r + c];
            d[c] = a.dir[3 * r + c];
          }
        }
        spos[m] = make_float4(o[0], o[1], o[2], ray_state == 0 ? 1.f : 0.f);
      }
      fail = bf16::epi_any(fail, kEpiThreads);
      for (int st = 0; st < a.steps && !fail; ++st) {
        // this step's position; rays that have stopped are evaluated where
        // they are and left alone
        const float4 pv = spos[m];
        const float x = pv.x, y = pv.y, z = pv.z;
        const bool alive = pv.w != 0.f;
        // layer 0 of level 0 (the A operand is free: the last GEMM that read
        // it has been drained)
#pragma unroll 1
        for (int c = 0; c < NC; ++c)
          bf16::layer0_unit<T, false, U>(sA, w0s, WP, m, c * kKC + h * U, 0, 0.f, x, y, z);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(afull);
        for (int lev = 0; lev < L; ++lev) {
          const float* wout = wouts + lev * WP;
          const bool next = lev + 1 < L;  // layer 0 of the next level in the last drain
          const float* w0n = w0s + (lev + 1) * 4 * WP;
          float part = 0.f;
          for (int l = 1; l <= nh; ++l, ++k) {
            if (!fail && !bf16::warp_wait(dfull, (uint32_t)(k & 1), a.status, abort_flag))
              fail = true;
            tc::fence_after_sync();
            if (!fail) {
#pragma unroll 1
              for (int c0 = 0; c0 < NC; c0 += 2) {
                uint32_t r2[2][U];
                tc::ld_32x32b<U>(tl + (uint32_t)(c0 * kKC + h * U), r2[0]);
                if (c0 + 1 < NC) tc::ld_32x32b<U>(tl + (uint32_t)((c0 + 1) * kKC + h * U), r2[1]);
                tc::wait_ld();
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                  const int c = c0 + u;
                  if (c >= NC) break;
                  const int j0 = c * kKC + h * U;
                  if (l < nh) {
                    float v[U];
#pragma unroll
                    for (int jj = 0; jj < U; ++jj) v[jj] = bf16::sin_fast(__uint_as_float(r2[u][jj]));
                    bf16::store_a_unit<T, U>(sA, m, j0, v);
                  } else {
                    const float4* wo4 = reinterpret_cast<const float4*>(wout + j0);
#pragma unroll
                    for (int j4 = 0; j4 < U / 4; ++j4) {
                      const float4 wv = wo4[j4];
                      const float wa[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
                      for (int i = 0; i < 4; ++i)
                        part = __fmaf_rn(bf16::sin_fast(__uint_as_float(r2[u][4 * j4 + i])), wa[i],
                                         part);
                    }
                    if (next) bf16::layer0_unit<T, false, U>(sA, w0n, WP, m, j0, 0, 0.f, x, y, z);
                  }
                }
              }
            }
            const bool hand_over = l < nh || next;  // this drain wrote the next A operand
            if (hand_over) fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) {
              if (hand_over) mbar_arrive(afull);
              mbar_arrive(dempty);
            }
          }
          red[(lev * Q + h) * kM + m] = part;
        }
        // every level's partial sums written: the h = 0 warps combine the
        // feature splits, gate the levels by band and take the marching step
        fail = bf16::epi_any(fail, kEpiThreads);
        if (fail) break;
        if (h == 0) {
          float sacc = 0.f;
          bool gate = alive;
          for (int lev = 0; lev < L; ++lev) {
            float sum = red[(lev * Q) * kM + m];
#pragma unroll
            for (int hh = 1; hh < Q; ++hh) sum = __fadd_rn(sum, red[(lev * Q + hh) * kM + m]);
            const float f = __fadd_rn(sum, bouts[lev]);
            if (lev == 0) {
              sacc = f;
            } else {
              gate = gate && fabsf(sacc) < a.delta[lev - 1];
              if (gate) sacc = __fadd_rn(sacc, f);
            }
          }
          bool hit = false;
          if (alive) {
            const bool last = st == a.steps - 1;
            ray_state = march_step(sacc, o, d, a.eps, a.R, a.last_final && last);
            hit = ray_state == 1;
            if (ray_state != 0 || last) {
              a.S[r] = sacc;
              for (int c = 0; c < 3; ++c) a.org[3 * r + c] = o[c];
              if (ray_state != 0) a.state[r] = ray_state;
            }
            spos[m] = make_float4(o[0], o[1], o[2], ray_state == 0 ? 1.f : 0.f);
          }
          warp_append(hit, (int32_t)r, a.hit_out, a.hit_count, a.capacity);
        }
        __threadfence_block();
        fail = bf16::epi_any(fail, kEpiThreads);
      }
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, WP);
}

template <int WP, int U, typename T>
int launch_u(const Args& a, cudaStream_t s) {
  using C = Cfg<WP, U>;
  const size_t smem = C::bytes(a.levels, a.lay[0].nh);
  if (smem > 227 * 1024) return MPL_ERR_UNSUPPORTED;
  MPL_CUDA_TRY(cudaFuncSetAttribute(trace_march_kernel<WP, U, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = (a.n_max + kM - 1) / kM;
  const int64_t sms = sm_count();
  grid = grid < sms ? grid : sms;
  if (grid <= 0) return MPL_OK;
  trace_march_kernel<WP, U, T><<<(unsigned)grid, bf16::Epi<U>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// the epilogue unit width of the level launches (MPL_OPT_BF16_EPILOGUE_UNIT),
// so that every ray gets the arithmetic of the launch-per-level loop
template <int WP, typename T>
int launch(const Args& a, cudaStream_t s) {
  return option_value(MPL_OPT_BF16_EPILOGUE_UNIT) == 32 ? launch_u<WP, 32, T>(a, s)
                                                         : launch_u<WP, 16, T>(a, s);
}

}  // namespace march
}  // namespace mpl

using namespace mpl;

extern "C" int mpl_trace_march(const MplNet* nets, const void* const* packed, int32_t levels,
                               const float* deltas, const int32_t* active, const int32_t* count,
                               int64_t n_max, float* origins, const float* dirs, int32_t* state,
                               float* S, float eps, float radius, int32_t steps,
                               int32_t last_is_final, int32_t* hit_out, int32_t* hit_count,
                               int64_t capacity, int32_t precision, void* stream) {
  if (!nets || !packed || levels < 1 || levels > march::kMaxLevels || (levels > 1 && !deltas) ||
      !active || !count || n_max < 0 || !origins || !dirs || !state || !S || steps < 0 ||
      !hit_out || !hit_count || capacity < 0)
    return MPL_ERR_INVALID_ARG;
  if (precision != MPL_BF16 && precision != MPL_F16) return MPL_ERR_UNSUPPORTED;
  march::Args a;
  memset(&a, 0, sizeof(a));
  for (int lev = 0; lev < levels; ++lev) {
    if (!packed[lev] || ((uintptr_t)packed[lev] & 255) != 0) return MPL_ERR_INVALID_ARG;
    const int st = make_layout(&nets[lev], &a.lay[lev]);
    if (st != MPL_OK) return st;
    if (a.lay[lev].WP != a.lay[0].WP || a.lay[lev].nh != a.lay[0].nh || nets[lev].dims[0] != 3 ||
        nets[lev].dims[nets[lev].n_layers] != 1)
      return MPL_ERR_UNSUPPORTED;
    a.packed[lev] = (const char*)packed[lev];
  }
  if (a.lay[0].nh < 1 || (a.lay[0].WP != 128 && a.lay[0].WP != 256) ||
      levels * a.lay[0].nh > march::kMaxBiasLayers)
    return MPL_ERR_UNSUPPORTED;
  for (int lev = 0; lev + 1 < levels; ++lev) a.delta[lev] = deltas[lev];
  a.levels = levels;
  a.active = active;
  a.count = count;
  a.n_max = n_max;
  a.org = origins;
  a.dir = dirs;
  a.state = state;
  a.S = S;
  a.eps = eps;
  a.R = radius;
  a.steps = steps;
  a.last_final = last_is_final;
  a.hit_out = hit_out;
  a.hit_count = hit_count;
  a.capacity = capacity;
  a.status = device_status_ptr();
  if (steps == 0 || n_max == 0) return MPL_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const bool f16 = precision == MPL_F16;
  switch (a.lay[0].WP) {
    case 128:
      return f16 ? march::launch<128, __half>(a, s) : march::launch<128, __nv_bfloat16>(a, s);
    case 256:
      return f16 ? march::launch<256, __half>(a, s) : march::launch<256, __nv_bfloat16>(a, s);
    default:
      return MPL_ERR_UNSUPPORTED;
  }
}
