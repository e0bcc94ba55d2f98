// Batched evaluation of many levels of many models in ONE persistent launch
// on the tensor cores (sm_103a): the serving form of the fused level kernel
// of level_bf16.cuh.
//
// The launch walks the concatenated 128-point tiles of all entries (an entry
// = one level of one model on its own point list).  Every CTA builds the
// exclusive prefix of the entries' tile counts in shared memory at start-up
// (point counts may live on the device, e.g. band lists written by earlier
// kernels), takes tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... and finds
// the entry of a tile by binary search in that prefix.  Entries may differ in
// width (64, 128 or 256) and depth (1 or 2 hidden GEMMs): the MMA shape
// (N = width), the K-chunk count and the weight copy sizes are per tile.
//
// Per-entry constants (omega0-scaled first layer, output row, bias tiles of
// the hidden layers) live in two shared-memory slots, one per tile parity,
// filled by the TMA warp and handed over through mbarriers: cfull[slot]
// (TMA -> MMA and epilogue), cfree[slot] (epilogue -> TMA, after the tile's
// last drain, which also proves the tile's MMAs, the readers of the bias
// tiles, have completed).  A slot is re-filled only when its tile belongs to
// another entry than the slot holds.  Everything else (warp roles, chunked
// A-operand hand-off, double TMEM accumulators, weight ring, cross-tile
// pipelining of layer 0, bounded waits with abort) is the single-level
// kernel's.  Only the TMA thread reads the global entry table (when its tile
// leaves the current entry); it publishes the entry's scalars in the slot, so
// the MMA and epilogue warps read shared memory only.
#pragma once

#include "level_bf16.cuh"

namespace mpl {
namespace batch {

using bf16::kKC;
using bf16::kM;

constexpr int kMaxHidden = 2;     // hidden GEMMs per level (3 hidden layers)
constexpr int kMaxEntries = 1024;
constexpr int kWPMax = 256;
constexpr uint32_t kStageMax = kWPMax * kKC * 2;             // one weight K chunk
constexpr uint32_t kBiasTile = kWPMax * 16 * 2;              // one bias tile
// Scalars of the entry a slot holds, written by the TMA thread next to the
// constants so that the MMA and epilogue warps never touch the global entry
// table on their critical paths.
struct SlotInfo {
  const float* xyz;
  const int32_t* index;
  float* S;
  int64_t n;           // points (device count applied)
  int64_t first_tile;  // first global tile of the entry
  float bout;
  int32_t WP, nh, kind, grid_n, store_mode;
  float voxel, off0, off1, off2;
};
constexpr uint32_t kInfoBytes = 128;
static_assert(sizeof(SlotInfo) <= kInfoBytes, "slot info size");
constexpr uint32_t kSlotBytes = kMaxHidden * kBiasTile + kWPMax * 16 + kWPMax * 4 + kInfoBytes;

// One entry as the kernel reads it (built on the host from MplBatchEntry).
struct Entry {
  const char* packed;
  const float* xyz;
  const int32_t* index;
  const int32_t* n_dev;
  float* S;
  int64_t n;
  int64_t w0f, wout, bout;
  int64_t hw[kMaxHidden];   // hidden layer l = 1..nh at [l - 1]: weight K chunks
  int64_t hbx[kMaxHidden];  // bias tiles
  int32_t nh, WP, kind, grid_n;
  float voxel, off0, off1, off2;
  int32_t store_mode, pad;
};

struct Args {
  const Entry* entries;
  int32_t count;
  int* status;
  int32_t* tiles;  // [count + 1] tile prefix in the workspace (two-tile kernel)
};


template <int STAGES, int U>
struct Cfg {
  static constexpr int kStages = STAGES;
  static constexpr uint32_t oA = 0;                                // bf16 [128][256]
  static constexpr uint32_t oW = kM * kWPMax * 2;                  // [S] weight chunks
  static constexpr uint32_t oSlot = oW + STAGES * kStageMax;       // [2] constants
  // within a slot: bias tiles, then w0f ([4][WP] floats), then wout (float [WP])
  static constexpr uint32_t sBx = 0;
  static constexpr uint32_t sW0 = kMaxHidden * kBiasTile;
  static constexpr uint32_t sWout = sW0 + kWPMax * 16;
  static constexpr uint32_t sInfo = sWout + kWPMax * 4;
  static constexpr uint32_t oAx = (oSlot + 2 * kSlotBytes + 1023) & ~1023u;  // ones tile
  static constexpr uint32_t oRed = oAx + kM * 16 * 2;
  static constexpr uint32_t oBar = oRed + 2 * (64 / U - 1) * kM * 4;
  static constexpr uint32_t kNumBars = 2 * STAGES + bf16::kMaxNC + 2 + 2 + 4 + 1 + 4;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr uint32_t oTiles = oMisc + 16;                   // int32 [kMaxEntries + 1]
  static constexpr size_t kBytes = oTiles + (kMaxEntries + 1) * 4;
  static_assert(oAx % 1024 == 0, "MMA operand tiles on 1 KiB boundaries");
};

// last entry whose first tile is <= t (entries without tiles are skipped
// because their successor starts at the same tile)
__device__ __forceinline__ int find_entry(const int32_t* tiles, int count, int64_t t) {
  int lo = 0, hi = count;  // tiles[lo] <= t < tiles[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((int64_t)tiles[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int64_t entry_points(const Entry& e) {
  int64_t n = e.n;
  if (e.n_dev) {
    const int64_t m = (int64_t)(*e.n_dev);
    n = m < n ? m : n;
  }
  return n < 0 ? 0 : n;
}

__device__ __forceinline__ void info_point(const SlotInfo& e, int64_t q, int64_t& p, float& x,
                                           float& y, float& z) {
  p = e.index ? (int64_t)e.index[q] : q;
  if (e.kind == MPL_POINTS_GRID) {
    grid_point(p, e.grid_n, e.voxel, e.off0, e.off1, e.off2, x, y, z);
  } else {
    x = e.xyz[3 * p + 0];
    y = e.xyz[3 * p + 1];
    z = e.xyz[3 * p + 2];
  }
}

template <int STAGES, int U, typename T>
__global__ void __launch_bounds__(bf16::Epi<U>::kThreads, 1) batch_kernel(const Args a) {
  using C = Cfg<STAGES, U>;
  using E = bf16::Epi<U>;
  using Op = bf16::Operand<T>;
  constexpr int kEpiWarps = E::kWarps;
  constexpr int kMmaWarp = E::kMmaWarp;
  constexpr int kTmaWarp = E::kTmaWarp;
  constexpr int kThreads = E::kThreads;
  constexpr int Q = E::kQ;
  constexpr int S = STAGES;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem + C::oA;
  uint8_t* sW = smem + C::oW;
  uint8_t* sSlot = smem + C::oSlot;
  float* red = reinterpret_cast<float*>(smem + C::oRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint64_t* wfull = bars;
  uint64_t* wempty = bars + S;
  uint64_t* achunk = bars + 2 * S;
  uint64_t* dfull = achunk + bf16::kMaxNC;
  uint64_t* dempty = dfull + 2;
  uint64_t* redfull = dempty + 2;
  uint64_t* redfree = redfull + 2;
  uint64_t* finalb = redfree + 2;
  uint64_t* cfull = finalb + 1;  // [2]
  uint64_t* cfree = cfull + 2;   // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);
  int32_t* tiles = reinterpret_cast<int32_t*>(smem + C::oTiles);
  uint8_t* sAx = smem + C::oAx;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int count = a.count;

  // ---- tile prefix of the entries
  for (int e = threadIdx.x; e < count; e += kThreads) {
    const int64_t n = entry_points(a.entries[e]);
    tiles[e + 1] = (int32_t)((n + kM - 1) / kM);
  }
  __syncthreads();
  if (warp == 0) {
    int32_t carry = 0;
    for (int base = 0; base < count; base += 32) {
      const int e = base + lane;
      int32_t v = e < count ? tiles[e + 1] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
      }
      if (e < count) tiles[e + 1] = carry + v;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
    if (lane == 0) tiles[0] = 0;
  }
  __syncthreads();
  const int64_t total = tiles[count];
  if ((int64_t)blockIdx.x >= total) return;

  // ---- set-up: barriers, TMEM, ones tile
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    for (int c = 0; c < bf16::kMaxNC; ++c) mbar_init(&achunk[c], kEpiWarps);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&dfull[b], 1);
      mbar_init(&dempty[b], kEpiWarps);
      mbar_init(&redfull[b], 4 * (Q - 1));
      mbar_init(&redfree[b], 4);
      mbar_init(&cfull[b], 1);
      mbar_init(&cfree[b], kEpiWarps);
    }
    mbar_init(finalb, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tmem_slot, 512);
  for (int i = threadIdx.x; i < kM * 16; i += kThreads) {
    const int m = i >> 4, k = i & 15;
    const uint32_t off =
        (uint32_t)(((k >> 3) * 16 + (m >> 3)) * 128 + (m & 7) * 16 + (k & 7) * 2);
    *reinterpret_cast<T*>(sAx + off) = Op::value(k < 2 ? 1.f : 0.f);
  }
  fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == kTmaWarp) {
    // ================= TMA producer: slot constants and weight K chunks ====
    if (lane == 0) {
      int64_t w = 0, tloc = 0;
      int entry0 = -1, entry1 = -1;  // entry whose constants each slot holds
      // the current entry, cached until a tile leaves its range
      int e = -1;
      int64_t e_end = -1;
      const char* pk = nullptr;
      int WP = 0, nh = 0;
      int64_t hw0 = 0, hw1 = 0;  // the entry's hidden weight images (kMaxHidden = 2)
      for (int64_t t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x, ++tloc) {
        if (t >= e_end || e < 0 || t < (int64_t)tiles[e]) {
          e = find_entry(tiles, count, t);
          e_end = tiles[e + 1];
          const Entry* en = a.entries + e;
          pk = en->packed;
          WP = en->WP;
          nh = en->nh;
          hw0 = en->hw[0];
          hw1 = en->hw[1];
        }
        const int slot = (int)(tloc & 1);
        if (tloc >= 2 && !bf16::mbar_wait_abort(&cfree[slot], (uint32_t)(((tloc >> 1) - 1) & 1),
                                                a.status, abort_flag))
          break;
        uint8_t* sl = sSlot + slot * kSlotBytes;
        if ((slot ? entry1 : entry0) != e) {
          const Entry* en = a.entries + e;
          SlotInfo* info = reinterpret_cast<SlotInfo*>(sl + C::sInfo);
          info->xyz = en->xyz;
          info->index = en->index;
          info->S = en->S;
          info->n = entry_points(*en);
          info->first_tile = tiles[e];
          info->bout = *reinterpret_cast<const float*>(pk + en->bout);
          info->WP = WP;
          info->nh = nh;
          info->kind = en->kind;
          info->grid_n = en->grid_n;
          info->store_mode = en->store_mode;
          info->voxel = en->voxel;
          info->off0 = en->off0;
          info->off1 = en->off1;
          info->off2 = en->off2;
          const uint32_t bytes = (uint32_t)(nh * WP * 32 + WP * 16 + WP * 4);
          mbar_arrive_expect_tx(&cfull[slot], bytes);
          for (int l = 0; l < nh; ++l)
            tma_bulk_g2s(sl + C::sBx + l * kBiasTile, pk + en->hbx[l], WP * 32, &cfull[slot]);
          tma_bulk_g2s(sl + C::sW0, pk + en->w0f, WP * 16, &cfull[slot]);
          tma_bulk_g2s(sl + C::sWout, pk + en->wout, WP * 4, &cfull[slot]);
          if (slot)
            entry1 = e;
          else
            entry0 = e;
        } else {
          mbar_arrive(&cfull[slot]);
        }
        const uint32_t stage = (uint32_t)WP * kKC * 2;
        const int NC = WP / kKC;
        bool ok = true;
        for (int l = 0; l < nh && ok; ++l) {
          const char* src = pk + (l ? hw1 : hw0);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            const int64_t u = w / S;
            if (u > 0 && !bf16::mbar_wait_abort(&wempty[s], (uint32_t)((u - 1) & 1), a.status,
                                                abort_flag)) {
              ok = false;
              break;
            }
            mbar_arrive_expect_tx(&wfull[s], stage);
            tma_bulk_g2s(sW + s * kStageMax, src + (size_t)c * stage, stage, &wfull[s]);
          }
        }
        if (!ok) {
          ++tloc;
          break;
        }
      }
      // copies still in flight land before the CTA exits
      const int64_t first = w > S ? w - S : 0;
      for (int64_t v = first; v < w; ++v)
        mbar_wait(&wfull[v % S], (uint32_t)((v / S) & 1), a.status);
      for (int64_t k = tloc > 2 ? tloc - 2 : 0; k < tloc; ++k)
        mbar_wait(&cfull[k & 1], (uint32_t)((k >> 1) & 1), a.status);
    }
  } else if (warp == kMmaWarp) {
    // ================= MMA issuer ==========================================
    if (lane == 0) {
      // descriptor bases; an operand at byte offset o adds o >> 4 (the start
      // address field, which stays below 2^14 inside shared memory)
      const uint64_t aDesc = tc::smem_desc(smem_u32(sA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      int64_t w = 0, g = 0, tloc = 0;
      uint32_t aph = 0;  // bit c: phase parity of achunk[c]
      bool ok = true;
      for (int64_t t = blockIdx.x; t < total && ok; t += gridDim.x, ++tloc) {
        const int slot = (int)(tloc & 1);
        if (!bf16::mbar_wait_abort(&cfull[slot], (uint32_t)((tloc >> 1) & 1), a.status,
                                   abort_flag)) {
          ok = false;
          break;
        }
        const uint8_t* sl = sSlot + slot * kSlotBytes;
        const SlotInfo* info = reinterpret_cast<const SlotInfo*>(sl + C::sInfo);
        const int WP = info->WP, nh = info->nh;
        const int NC = WP / kKC;
        const uint32_t idesc = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
        const uint32_t bx = smem_u32(sl + C::sBx);
        for (int l = 0; l < nh && ok; ++l, ++g) {
          // GEMM g uses accumulator g & 1, whose earlier uses number g >> 1
          const int b = (int)(g & 1);
          if (g >= 2 && !bf16::mbar_wait_abort(&dempty[b], (uint32_t)(((g >> 1) - 1) & 1),
                                               a.status, abort_flag)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t d_tmem = tmem + (uint32_t)(b * kWPMax);
          tc::mma_bf16(d_tmem, xDesc, tc::smem_desc(bx + (uint32_t)l * kBiasTile, 128u, 256u),
                       idesc, false);
          for (int c = 0; c < NC; ++c, ++w) {
            const int s = (int)(w % S);
            if (!bf16::mbar_wait_abort(&achunk[c], (aph >> c) & 1u, a.status, abort_flag) ||
                !bf16::mbar_wait_abort(&wfull[s], (uint32_t)((w / S) & 1), a.status,
                                       abort_flag)) {
              ok = false;
              break;
            }
            aph ^= 1u << c;
            tc::fence_after_sync();
            const uint64_t aC = aDesc + (uint64_t)((c * 8 * 2048) >> 4);
            const uint64_t wC = wDesc + (uint64_t)((s * kStageMax) >> 4);
#pragma unroll
            for (int ks = 0; ks < kKC / 16; ++ks)
              tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                           wC + (uint64_t)((ks * 256) >> 4), idesc, true);
            tc::commit(&wempty[s]);
          }
          if (!ok) break;
          tc::commit(&dfull[b]);
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
    int64_t g = 0, tloc = 0;
    bool ok = true;
    // first tile: its constants, its point, its layer 0
    int64_t t = blockIdx.x;
    int64_t p = -1;
    float x = 0.f, y = 0.f, z = 0.f;
    ok = bf16::warp_wait(&cfull[0], 0u, a.status, abort_flag);
    if (ok) {
      const SlotInfo& info = *reinterpret_cast<const SlotInfo*>(sSlot + C::sInfo);
      const int64_t qi = (t - info.first_tile) * kM + m;
      if (qi < info.n) info_point(info, qi, p, x, y, z);
      const float* w0s = reinterpret_cast<const float*>(sSlot + C::sW0);
      for (int c = 0; c < info.WP / kKC; ++c) {
        bf16::layer0_unit<T, false, U>(sA, w0s, info.WP, m, c * kKC + h * U, 0, 0.f, x, y, z);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&achunk[c]);
      }
    }
    for (; t < total && ok; t += gridDim.x, ++tloc) {
      const int slot = (int)(tloc & 1);
      const uint8_t* sl = sSlot + slot * kSlotBytes;
      const uint8_t* sn = sSlot + (slot ^ 1) * kSlotBytes;
      const SlotInfo& info = *reinterpret_cast<const SlotInfo*>(sl + C::sInfo);
      const SlotInfo& ninfo = *reinterpret_cast<const SlotInfo*>(sn + C::sInfo);
      const int nh = info.nh, NC = info.WP / kKC;
      const float* wout = reinterpret_cast<const float*>(sl + C::sWout);
      const float* w0n = reinterpret_cast<const float*>(sn + C::sW0);
      const int64_t tn = t + gridDim.x;
      const bool has_next = tn < total;
      int NCn = 0;
      int64_t pn = -1;
      float xn = 0.f, yn = 0.f, zn = 0.f;

      float part = 0.f;
      for (int l = 1; l <= nh; ++l, ++g) {
        const int b = (int)(g & 1);
        if (!bf16::warp_wait(&dfull[b], (uint32_t)((g >> 1) & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        if (l == nh && has_next) {
          if (!bf16::warp_wait(&cfull[slot ^ 1], (uint32_t)(((tloc + 1) >> 1) & 1), a.status,
                               abort_flag)) {
            ok = false;
            break;
          }
          NCn = ninfo.WP / kKC;
          const int64_t qn = (tn - ninfo.first_tile) * kM + m;
          if (qn < ninfo.n) info_point(ninfo, qn, pn, xn, yn, zn);
        }
        const uint32_t taddr = tl + (uint32_t)(b * kWPMax);
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
            if (l < nh) {
              float v[U];
#pragma unroll
              for (int jj = 0; jj < U; ++jj) v[jj] = bf16::sin_fast(__uint_as_float(r[jj]));
              bf16::store_a_unit<T, U>(sA, m, j0, v);
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
                for (int i = 0; i < 4; ++i)
                  part = __fmaf_rn(bf16::sin_fast(__uint_as_float(r[4 * j4 + i])), wa[i], part);
              }
              if (c < NCn) {
                bf16::layer0_unit<T, false, U>(sA, w0n, ninfo.WP, m, j0, 0, 0.f, xn, yn, zn);
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&achunk[c]);
              }
            }
          }
        }
        if (l == nh) {
          // a wider next entry: its remaining layer-0 chunks
          for (int c = NC; c < NCn; ++c) {
            bf16::layer0_unit<T, false, U>(sA, w0n, ninfo.WP, m, c * kKC + h * U, 0, 0.f, xn, yn,
                                           zn);
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&achunk[c]);
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&dempty[b]);
      }
      if (!ok) break;
      // this tile's scalars, then the slot is no longer read by this warp
      float* const Sp = info.S;
      const int store_mode = info.store_mode;
      const float bout = info.bout;
      __syncwarp();
      if (lane == 0) mbar_arrive(&cfree[slot]);

      const int rb = (int)(tloc & 1);
      if (h > 0) {
        if (tloc >= 2 && !bf16::warp_wait(&redfree[rb], (uint32_t)(((tloc >> 1) - 1) & 1),
                                          a.status, abort_flag)) {
          ok = false;
          break;
        }
        red[(rb * (Q - 1) + (h - 1)) * kM + m] = part;
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfull[rb]);
      } else {
        if (!bf16::warp_wait(&redfull[rb], (uint32_t)((tloc >> 1) & 1), a.status, abort_flag)) {
          ok = false;
          break;
        }
        float sum = part;
#pragma unroll
        for (int hh = 0; hh < Q - 1; ++hh) sum = __fadd_rn(sum, red[(rb * (Q - 1) + hh) * kM + m]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&redfree[rb]);
        if (p >= 0) {
          const float f = __fadd_rn(sum, bout);
          float* sp = Sp + p;
          *sp = store_mode == MPL_ACCUMULATE ? __fadd_rn(*sp, f) : f;
        }
      }
      p = pn;
    }
  }

  // ---- teardown
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, 512);
}

template <int STAGES, int U, typename T>
int launch(const Args& a, int ctas, cudaStream_t s) {
  using C = Cfg<STAGES, U>;
  static_assert(C::kBytes <= 227 * 1024, "shared memory of the batched kernel");
  MPL_CUDA_TRY(cudaFuncSetAttribute(batch_kernel<STAGES, U, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::kBytes));
  batch_kernel<STAGES, U, T><<<(unsigned)ctas, bf16::Epi<U>::kThreads, C::kBytes, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

}  // namespace batch
}  // namespace mpl
