// Batched evaluation of many levels of many models, two tiles in flight per
// CTA with dedicated first-layer warps (sm_103a): the serving form of the
// level kernel of level_l0w.cuh.
//
// One launch covers every entry of one padded width WP (the host groups a
// plan's entries by width when it prepares the plan and launches one kernel
// per width present), so the MMA shape, the K-chunk count, the weight ring
// and the shared-memory layout are compile-time as in the level kernel.
// Tiles are the concatenated 128-point tiles of the group's entries; the
// exclusive prefix of their tile counts is written to the workspace by a
// one-block kernel launched just before, and the entry of a tile is found
// by binary search in it.  A CTA takes the tiles of two slots in rounds:
// slot s of round r holds tile blockIdx.x + (2 r + s) gridDim.x, so each
// slot sees its tiles in increasing order and every role keeps, per slot,
// the entry of its current tile (looked up again only when a tile leaves
// that entry's range).  In every round the MMA warp interleaves the two
// slots' GEMMs layer by layer (GEMM l of slot 0, GEMM l of slot 1, ...); a
// slot whose tile has fewer hidden GEMMs drops out of the later layers.
// TMA, MMA and epilogue walk that same order.
//
// Per-entry data, one set per slot in shared memory: the bias tiles of the
// hidden layers (MMA operands), refilled by the TMA thread when a slot's
// tile changes entry; the omega0-scaled first layer, copied by the
// first-layer warps themselves, and the output row, copied by the epilogue
// warps (each warp the columns it reads).  Of each bias tile only the K core
// matrices 0..7 are kept (K columns 0 and 1 hold the bias and its remainder,
// the rest zero); the descriptor's K stride points the MMA's second K core
// matrix at the ones tile (finite values), which meets zero columns of the A
// ones tile, so the extra products are exactly zero and the sum is that of
// the full tile.
//
// Barriers per slot s, next to level_l0w.cuh's (achunk, l0chunk, dfull,
// dempty, redfull, redfree, afree): cfull[s] (TMA -> MMA, one phase per
// tile: the slot's bias tiles hold the tile's entry; with copies in flight on
// a refill, a plain arrival otherwise), before the weight chunks of the
// tile's first GEMM.  The TMA thread arrives for tile r of a slot only after
// afree[s] of tile r - 1 (the MMA finished that tile's GEMMs, so it has
// waited on its cfull phase and no longer reads the bias tiles).  Every wait
// is bounded (the abort protocol of level_bf16.cuh).
// Per element the arithmetic is the level kernels': the results equal
// single-level launches bit for bit under the same epilogue unit width.
#pragma once

#include "batch.cuh"
#include "level_l0w.cuh"

namespace mpl {
namespace batch {

template <int WP, int STAGES, int U>
struct PCfg {
  static constexpr int NC = WP / kKC;
  static constexpr int kQ = 64 / U;
  static constexpr uint32_t kStageBytes = WP * kKC * 2;
  static constexpr uint32_t kABytes = kM * WP * 2;
  static constexpr uint32_t kTmemCols = WP == 64 ? 128 : (WP == 128 ? 256 : 512);
  static constexpr uint32_t kBiasBytes = WP * 16;  // K core matrices 0..7 of a bias tile
  static constexpr uint32_t oA = 0;                           // [2] A operands
  static constexpr uint32_t oW = 2 * kABytes;                 // [S] weight K chunks
  static constexpr uint32_t oBx = oW + STAGES * kStageBytes;  // [2][kMaxHidden] bias tiles
  static constexpr uint32_t oAx = (oBx + 2 * kMaxHidden * kBiasBytes + 1023) & ~1023u;  // ones
  static constexpr uint32_t oRed = oAx + kM * 16 * 2;         // float [2][Q - 1][128]
  static constexpr uint32_t kRedSlot = (kQ > 1 ? kQ - 1 : 1) * kM * 4;
  static constexpr uint32_t oEpi = oRed + 2 * kRedSlot;       // [epilogue warps][2] EpiSlot
  static constexpr uint32_t oW0 = oEpi + 4 * kQ * 2 * 80;     // [2] float [4][WP] first layer
  static constexpr uint32_t oWout = oW0 + 2 * 16 * WP;        // [2] float [WP] output row
  static constexpr uint32_t oBar = oWout + 2 * 4 * WP;
  // wfull, wempty [S]; achunk, l0chunk [2][kMaxNC]; dfull, dempty, redfull,
  // redfree, afree, cfull [2]; final
  static constexpr uint32_t kNumBars = 2 * STAGES + 4 * bf16::kMaxNC + 6 * 2 + 1;
  static constexpr uint32_t oMisc = oBar + kNumBars * 8;
  static constexpr size_t kBytes = oMisc + 16;
  static_assert(oAx % 1024 == 0 && oBx % 1024 == 0, "MMA operand tiles on 1 KiB boundaries");
};

// The entry of a slot's current tile, looked up again only when a tile
// leaves [lo, hi).
struct EntryCursor {
  int e = -1;
  int64_t lo = 0, hi = 0;
  __device__ __forceinline__ bool move(const int32_t* tiles, int count, int64_t t) {
    if (e >= 0 && t >= lo && t < hi) return false;
    e = find_entry(tiles, count, t);
    lo = tiles[e];
    hi = tiles[e + 1];
    return true;
  }
};

// What an epilogue warp uses of a slot's entry, in shared memory (one copy
// per warp and slot, written by its lane 0) rather than in registers, which
// the accumulator rows fill.
struct EpiSlot {
  int64_t lo, hi;     // the entry's tiles
  const float* wout;  // the entry's output row in global memory
  float* S;
  const int32_t* index;
  int64_t n;
  float bout;
  int e, nh, store_mode;
  int held;  // entry whose output row this warp copied into the slot
  int pad[2];
  __device__ __forceinline__ void load(const Args& a, int64_t t) {
    e = find_entry(a.tiles, a.count, t);
    lo = a.tiles[e];
    hi = a.tiles[e + 1];
    const Entry& en = a.entries[e];
    wout = reinterpret_cast<const float*>(en.packed + en.wout);
    S = en.S;
    index = en.index;
    n = entry_points(en);
    bout = *reinterpret_cast<const float*>(en.packed + en.bout);
    nh = en.nh;
    store_mode = en.store_mode;
  }
};
static_assert(sizeof(EpiSlot) == 80, "epilogue slot record");

template <int WP, int STAGES, int U, int NL, typename T>
__global__ void __launch_bounds__(l0w::Roles<U, NL>::kThreads, 1) batch_l0w_kernel(const Args a) {
  using C = PCfg<WP, STAGES, U>;
  using R = l0w::Roles<U, NL>;
  using Op = bf16::Operand<T>;
  constexpr int kMaxNC = bf16::kMaxNC;
  constexpr int kEpiWarps = R::kEpiWarps;
  constexpr int kL0First = R::kL0First;
  constexpr int kMmaWarp = R::kMmaWarp;
  constexpr int kTmaWarp = R::kTmaWarp;
  constexpr int kThreads = R::kThreads;
  constexpr int Q = R::kQ;
  constexpr int NC = C::NC;
  constexpr int S = STAGES;
  constexpr uint32_t IDESC = tc::idesc_f16kind_f32(kM, WP, Op::kFormat);
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem + C::oW;
  uint8_t* sBx = smem + C::oBx;
  uint8_t* sAx = smem + C::oAx;
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
  uint64_t* cfull = afree + 2;              // [2]
  uint64_t* finalb = cfull + 2;             // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oMisc);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::oMisc + 4);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int count = a.count;
  const int32_t* tiles = a.tiles;  // the entries' tile prefix, [count + 1]
  const int64_t total = tiles[count];
  if ((int64_t)blockIdx.x >= total) return;
  const int64_t G = gridDim.x;
  auto tile_of = [&](int64_t r, int s) { return (int64_t)blockIdx.x + (2 * r + s) * G; };
  const int64_t nrounds = (total - blockIdx.x + 2 * G - 1) / (2 * G);

  // ---- set-up: barriers, TMEM, ones tile
  if (threadIdx.x == 0) {
    for (int st = 0; st < S; ++st) {
      mbar_init(&wfull[st], 1);
      mbar_init(&wempty[st], 1);
    }
    for (int c = 0; c < 2 * kMaxNC; ++c) {
      mbar_init(&achunk[c], kEpiWarps);
      mbar_init(&l0chunk[c], NL);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&dfull[b], 1);
      mbar_init(&dempty[b], kEpiWarps);
      mbar_init(&redfull[b], 4 * (Q - 1));
      mbar_init(&redfree[b], 4);
      mbar_init(&afree[b], 1);
      mbar_init(&cfull[b], 1);
    }
    mbar_init(finalb, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tmem_slot, C::kTmemCols);
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
    // ================= TMA: bias tiles per slot, weight K chunks ==========
    if (lane == 0) {
      EntryCursor cur0, cur1;
      int held0 = -1, held1 = -1;      // entry whose bias tiles each slot holds
      int64_t last0 = -1, last1 = -1;  // last round whose cfull phase this thread completed
      int64_t w = 0;                   // weight chunks issued
      bool ok = true;
      for (int64_t r = 0; r < nrounds && ok && !*abort_flag; ++r) {
        const int64_t t0 = tile_of(r, 0);
        const bool has1 = t0 + G < total;  // slot 0 has a tile in every round
        cur0.move(tiles, count, t0);
        if (has1) cur1.move(tiles, count, t0 + G);
        const Entry* e0 = a.entries + cur0.e;
        const Entry* e1 = a.entries + (has1 ? cur1.e : cur0.e);
        const int nh0 = e0->nh, nh1 = has1 ? e1->nh : 0;
        const int lmax = nh0 > nh1 ? nh0 : nh1;
#pragma unroll 1
        for (int l = 1; l <= lmax && ok; ++l) {
#pragma unroll 1
          for (int s = 0; s < 2; ++s) {
            if (!ok || l > (s ? nh1 : nh0)) continue;
            const Entry* en = s ? e1 : e0;
            const char* pk = en->packed;
            if (l == 1) {
              // the slot's previous tile finished its GEMMs (which precede
              // every chunk issued so far in the MMA's order, so the wait
              // rarely holds the ring back): its bias tiles are no longer
              // read and its cfull phase has been waited on
              if (r > 0 && !bf16::mbar_wait_abort(&afree[s], (uint32_t)((r - 1) & 1), a.status,
                                                  abort_flag)) {
                ok = false;
                continue;
              }
              const int ce = s ? cur1.e : cur0.e;
              if ((s ? held1 : held0) != ce) {
                const int nh = en->nh;
                mbar_arrive_expect_tx(&cfull[s], (uint32_t)(nh * C::kBiasBytes));
                // a cold path: kept rolled, out of the way of the hot loops
#pragma unroll 1
                for (int g = 0; g < nh * (WP / 8); ++g) {
                  const int hl = g / (WP / 8), gg = g % (WP / 8);
                  tma_bulk_g2s(sBx + (s * kMaxHidden + hl) * C::kBiasBytes + gg * 128,
                               pk + en->hbx[hl] + gg * 256, 128u, &cfull[s]);
                }
                if (s)
                  held1 = ce;
                else
                  held0 = ce;
              } else {
                mbar_arrive(&cfull[s]);
              }
              if (s)
                last1 = r;
              else
                last0 = r;
            }
            const char* src = pk + en->hw[l - 1];
#pragma unroll 1
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
      // copies still in flight land before the CTA exits
      for (int64_t v = w > S ? w - S : 0; v < w; ++v)
        mbar_wait(&wfull[v % S], (uint32_t)((v / S) & 1), a.status);
      if (last0 >= 0) mbar_wait(&cfull[0], (uint32_t)(last0 & 1), a.status);
      if (last1 >= 0) mbar_wait(&cfull[1], (uint32_t)(last1 & 1), a.status);
    }
  } else if (warp == kMmaWarp) {
    // ================= MMA issuer ==========================================
    if (lane == 0) {
      const uint64_t aDesc = tc::smem_desc(smem_u32(smem + C::oA), 2048u, 128u);
      const uint64_t wDesc = tc::smem_desc(smem_u32(sW), 128u, 1024u);
      const uint64_t xDesc = tc::smem_desc(smem_u32(sAx), 2048u, 128u);
      EntryCursor cur0, cur1;
      int nh0 = 0, nh1 = 0;      // hidden GEMMs of each slot's entry
      int64_t gs0 = 0, gs1 = 0;  // GEMMs issued per slot
      // bit 8 s + 4 (l > 1) + c: parity of the next phase of l0chunk[s][c]
      // (GEMM 1) or achunk[s][c] (later GEMMs)
      uint32_t ph = 0;
      int64_t w = 0;  // weight chunks consumed
      bool ok = true;
      for (int64_t r = 0; r < nrounds && ok; ++r) {
        const int64_t t0 = tile_of(r, 0);
        const bool has1 = t0 + G < total;  // slot 0 has a tile in every round
        if (cur0.move(tiles, count, t0)) nh0 = a.entries[cur0.e].nh;
        if (has1 && cur1.move(tiles, count, t0 + G)) nh1 = a.entries[cur1.e].nh;
        const int n1 = has1 ? nh1 : 0;
        const int lmax = nh0 > n1 ? nh0 : n1;
        for (int l = 1; l <= lmax && ok; ++l) {
#pragma unroll 1
          for (int s = 0; s < 2; ++s) {
            const int nh = s ? n1 : nh0;
            if (!ok || l > nh) continue;
            if (l == 1 && !bf16::mbar_wait_abort(&cfull[s], (uint32_t)(r & 1), a.status,
                                                 abort_flag)) {
              ok = false;
              continue;
            }
            const int64_t gsn = s ? gs1 : gs0;
            if (gsn > 0 && !bf16::mbar_wait_abort(&dempty[s], (uint32_t)((gsn - 1) & 1), a.status,
                                                  abort_flag)) {
              ok = false;
              continue;
            }
            tc::fence_after_sync();
            const uint32_t d_tmem = tmem + (uint32_t)(s * WP);
            const uint64_t aS = aDesc + (uint64_t)((s * C::kABytes) >> 4);
            const uint32_t bo = C::oBx + (uint32_t)(s * kMaxHidden + (l - 1)) * C::kBiasBytes;
            tc::mma_bf16(d_tmem, xDesc, tc::smem_desc(smem_u32(smem) + bo, C::oAx - bo, 128u),
                         IDESC, false);
            uint64_t* abar = (l == 1 ? l0chunk : achunk) + s * kMaxNC;
            const int pb = 8 * s + (l > 1 ? 4 : 0);
#pragma unroll 1
            for (int c = 0; c < NC; ++c, ++w) {
              const int st = (int)(w % S);
              if (!bf16::mbar_wait_abort(&abar[c], (ph >> (pb + c)) & 1u, a.status, abort_flag) ||
                  !bf16::mbar_wait_abort(&wfull[st], (uint32_t)((w / S) & 1), a.status,
                                         abort_flag)) {
                ok = false;
                break;
              }
              ph ^= 1u << (pb + c);
              tc::fence_after_sync();
              const uint64_t aC = aS + (uint64_t)((c * 8 * 2048) >> 4);
              const uint64_t wC = wDesc + (uint64_t)((st * C::kStageBytes) >> 4);
#pragma unroll
              for (int ks = 0; ks < kKC / 16; ++ks)
                tc::mma_bf16(d_tmem, aC + (uint64_t)((ks * 2 * 2048) >> 4),
                             wC + (uint64_t)((ks * 256) >> 4), IDESC, true);
              tc::commit(&wempty[st]);
            }
            if (!ok) continue;
            tc::commit(&dfull[s]);
            if (l == nh) tc::commit(&afree[s]);  // the tile's GEMMs are done
            if (s)
              ++gs1;
            else
              ++gs0;
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
    // The CTA's tiles in order k = 2 r + s (tile blockIdx.x + k gridDim.x);
    // the fields of the current entry are kept in registers.
    const int64_t nt = (total - blockIdx.x + G - 1) / G;
    EntryCursor cur;
    const float* w0g = nullptr;
    const float* xyz = nullptr;
    const int32_t* index = nullptr;
    int64_t npts = 0;
    int kind = 0, grid_n = 0;
    float voxel = 0.f, off0 = 0.f, off1 = 0.f, off2 = 0.f;
    int held0 = -1, held1 = -1;  // entry whose first layer this warp copied into slot 0, 1
    bool ok = true;
#pragma unroll 1
    for (int64_t k = 0; k < nt && ok; ++k) {
      const int64_t t = (int64_t)blockIdx.x + k * G;
      if (cur.move(tiles, count, t)) {
        const Entry& en = a.entries[cur.e];
        w0g = reinterpret_cast<const float*>(en.packed + en.w0f);
        xyz = en.xyz;
        index = en.index;
        npts = entry_points(en);
        kind = en.kind;
        grid_n = en.grid_n;
        voxel = en.voxel;
        off0 = en.off0;
        off1 = en.off1;
        off2 = en.off2;
      }
      float x = 0.f, y = 0.f, z = 0.f;
      const int64_t qi = (t - cur.lo) * kM + m;
      if (qi < npts) {
        const int64_t p = index ? (int64_t)index[qi] : qi;
        if (kind == MPL_POINTS_GRID) {
          grid_point(p, grid_n, voxel, off0, off1, off2, x, y, z);
        } else {
          x = xyz[3 * p + 0];
          y = xyz[3 * p + 1];
          z = xyz[3 * p + 2];
        }
      }
      const int64_t r = k >> 1;
      const int s = (int)(k & 1);
      // the slot's previous tile has finished its last GEMM (the reader of
      // the A operand written here), so every first-layer warp is past that
      // tile's layer 0 and the slot's first-layer image is free
      if (r > 0 &&
          !bf16::warp_wait(&afree[s], (uint32_t)((r - 1) & 1), a.status, abort_flag)) {
        ok = false;
        break;
      }
      float* w0s = reinterpret_cast<float*>(smem + C::oW0) + s * 4 * WP;
      if ((s ? held1 : held0) != cur.e) {
        // a new entry in the slot: this warp copies the columns it reads
        // (the warps that share them write the same values)
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const int j = c * kKC + f0 + (lane % kF);
          if (lane < kF)
#pragma unroll
            for (int i = 0; i < 4; ++i) w0s[i * WP + j] = __ldg(w0g + i * WP + j);
        }
        if (s)
          held1 = cur.e;
        else
          held0 = cur.e;
        __syncwarp();
      }
      uint8_t* sA = smem + C::oA + s * C::kABytes;
#pragma unroll 1
      for (int c = 0; c < NC; ++c) {
#pragma unroll
        for (int u = 0; u < kF / 16; ++u)
          bf16::layer0_unit<T, false, 16>(sA, w0s, WP, m, c * kKC + f0 + u * 16, 0, 0.f, x, y, z);
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
    EpiSlot* ee = reinterpret_cast<EpiSlot*>(smem + C::oEpi) + 2 * warp;
    if (lane == 0) {
      ee[0].e = ee[1].e = ee[0].held = ee[1].held = -1;
      ee[0].hi = ee[1].hi = 0;
    }
    __syncwarp();
    uint32_t dpar = 0;  // bit s: parity of slot s's next dfull phase
    bool ok = true;
    for (int64_t r = 0; r < nrounds && ok; ++r) {
      const int64_t t0 = tile_of(r, 0);
      const bool has1 = t0 + G < total;  // slot 0 has a tile in every round
#pragma unroll 1
      for (int s = 0; s < 2; ++s) {
        if (s && !has1) break;
        const int64_t t = t0 + s * G;
        if (t >= ee[s].hi) {  // tiles of a slot only increase (hi starts at 0)
          __syncwarp();
          if (lane == 0) ee[s].load(a, t);
          __syncwarp();
        }
      }
      const int lmax = has1 && ee[1].nh > ee[0].nh ? ee[1].nh : ee[0].nh;
      for (int l = 1; l <= lmax && ok; ++l) {
        for (int s = 0; s < 2 && ok; ++s) {
          if (s && !has1) continue;
          const int nh = ee[s].nh;  // hidden GEMMs of the slot's entry
          if (l > nh) continue;
          int64_t ps = -1;  // point of this row (last drain: the store)
          if (l == nh && h == 0) {
            const int64_t qi = (tile_of(r, s) - ee[s].lo) * kM + m;
            if (qi < ee[s].n) ps = ee[s].index ? (int64_t)ee[s].index[qi] : qi;
          }
          if (!bf16::warp_wait(&dfull[s], (dpar >> s) & 1u, a.status, abort_flag)) {
            ok = false;
            break;
          }
          dpar ^= 1u << s;
          tc::fence_after_sync();
          float* wout = reinterpret_cast<float*>(smem + C::oWout) + s * WP;
          if (l == 1 && ee[s].held != ee[s].e) {
            // a new entry in the slot: GEMM 1 of this tile was issued after
            // every epilogue warp drained the slot's previous tile, so no
            // warp reads the old row; this warp copies the columns it reads
            // (the warps that share them write the same values)
#pragma unroll
            for (int c = 0; c < NC; ++c)
              if (lane < U)
                wout[c * kKC + h * U + lane] = __ldg(ee[s].wout + c * kKC + h * U + lane);
            __syncwarp();
            if (lane == 0) ee[s].held = ee[s].e;
            __syncwarp();
          }
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
              if (l < nh) {
                float v[U];
#pragma unroll
                for (int jj = 0; jj < U; ++jj) v[jj] = bf16::sin_fast(__uint_as_float(rr[jj]));
                bf16::store_a_unit<T, U>(sA, m, j0, v);
              } else {
                const float4* wo4 = reinterpret_cast<const float4*>(wout + j0);
                float pt = part;
#pragma unroll
                for (int j4 = 0; j4 < U / 4; ++j4) {
                  const float4 wv = wo4[j4];
                  const float wa[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
                  for (int i = 0; i < 4; ++i)
                    pt = __fmaf_rn(bf16::sin_fast(__uint_as_float(rr[4 * j4 + i])), wa[i], pt);
                }
                part = pt;
              }
            }
          }
          // the slot's next GEMM waits for the whole drain (it overwrites the
          // accumulator), so the A chunks written here are handed over at once
          if (l < nh) fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) {
            if (l < nh)
#pragma unroll
              for (int c = 0; c < NC; ++c) mbar_arrive(&achunk[s * kMaxNC + c]);
            mbar_arrive(&dempty[s]);
          }
          if (l < nh) continue;

          // output layer: combine the feature splits, store (the slot's r-th)
          float* rs = red + s * (C::kRedSlot / 4);
          if (h > 0) {
            if (r >= 1 && !bf16::warp_wait(&redfree[s], (uint32_t)((r - 1) & 1), a.status,
                                           abort_flag)) {
              ok = false;
              break;
            }
            rs[(h - 1) * kM + m] = part;
            __syncwarp();
            if (lane == 0) mbar_arrive(&redfull[s]);
          } else {
            if (!bf16::warp_wait(&redfull[s], (uint32_t)(r & 1), a.status, abort_flag)) {
              ok = false;
              break;
            }
            float sum = part;
#pragma unroll
            for (int hh = 0; hh < Q - 1; ++hh) sum = __fadd_rn(sum, rs[hh * kM + m]);
            __syncwarp();
            if (lane == 0) mbar_arrive(&redfree[s]);
            if (ps >= 0) {
              const float f = __fadd_rn(sum, ee[s].bout);
              float* sp = ee[s].S + ps;
              *sp = ee[s].store_mode == MPL_ACCUMULATE ? __fadd_rn(*sp, f) : f;
            }
          }
        }
      }
    }
  }

  // ---- teardown
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, C::kTmemCols);
}

template <int WP, int STAGES, int U, int NL, typename T>
int launch_l0w_cfg(const Args& a, int ctas, cudaStream_t s) {
  using C = PCfg<WP, STAGES, U>;
  static_assert(C::kBytes <= 227 * 1024, "shared memory of the two-tile batched kernel");
  MPL_CUDA_TRY(cudaFuncSetAttribute(batch_l0w_kernel<WP, STAGES, U, NL, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::kBytes));
  batch_l0w_kernel<WP, STAGES, U, NL, T>
      <<<(unsigned)ctas, l0w::Roles<U, NL>::kThreads, C::kBytes, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

// The weight ring of the level kernel at each width: four stages at widths
// 64 and 128, two at 256 (where two A operands leave room for no more).
template <int U, int NL, typename T>
int launch_l0w(const Args& a, int WP, int ctas, cudaStream_t s) {
  switch (WP) {
    case 64: return launch_l0w_cfg<64, 4, U, NL, T>(a, ctas, s);
    case 128: return launch_l0w_cfg<128, 4, U, NL, T>(a, ctas, s);
    case 256: return launch_l0w_cfg<256, 2, U, NL, T>(a, ctas, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace batch
}  // namespace mpl
