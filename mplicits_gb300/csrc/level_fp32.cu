// Plain-form fused level evaluator: one SIREN level (i3d/model.py:88-129)
// over a point tile, FP32 SIMT FMAs, accurate sinf.  One CTA per SM; a tile
// is 128 rows x the padded width WP; activations stay in shared memory
// between layers; hidden-layer weights are streamed from L2 as 32-row
// K-chunks by the TMA engine into a double buffer.  Replaces the per-layer
// nn.Linear/addmm + SineLayer kernels of the reference and fuses the band
// test of i3d/meshing.py:223.
//
// GRAD mode also returns df/dx by forward-mode differentiation: a tile is
// 32 points x 4 rows (the value and its three tangents d/dx, d/dy, d/dz);
// the hidden GEMMs are unchanged, the epilogue of a tangent row is
// t' = omega cos(z) * (W t), and the output layer dots every row with W_L.
// This replaces the reference's forward-mode Normals GEMM chains
// (renderer/cuda/gemms.cu:206-337 with kernels.cu:277-313), which run three
// separate passes per level.
#include "level.cuh"

namespace mpl {

namespace {

constexpr int kTile = 128;  // points per tile
constexpr int kKC = 32;     // K rows per weight chunk

// Thread layout of a width: TX threads along the features (8 features each,
// two float4 groups 4*TX apart) x 16 along the rows (8 rows each: 4 + 4, 64
// apart), 2*WP threads in all.
template <int WP>
struct Fp32Threads {
  static constexpr int TX = WP / 8;
  static constexpr int kThreads = TX * 16;
};

template <int WP>
struct Fp32Smem {
  static constexpr int FPT = 8;  // features per thread
  static constexpr size_t act = (size_t)WP * kTile * 4;
  static constexpr size_t wbuf = 2ull * kKC * WP * 4;
  static size_t bytes(int nh) {
    return act + wbuf + 3 * WP * 4 + WP * 4 + (size_t)(nh > 0 ? nh : 1) * WP * 4 + WP * 4 +
           kTile * 3 * 4 + kTile * 8 + kTile * 4 + 2 * 8 + 16;
  }
};

template <int WP, bool GRAD>
__global__ void __launch_bounds__(Fp32Threads<WP>::kThreads, 1) level_fp32_kernel(const LevelArgs a) {
  constexpr int PT = GRAD ? kTile / 4 : kTile;  // points per tile
  constexpr int TX = Fp32Threads<WP>::TX;
  constexpr int kThreads = Fp32Threads<WP>::kThreads;
  constexpr int FPT = 8;
  constexpr int NQ = FPT / 4;  // float4 groups of features per thread
  constexpr int CPL = WP / kKC;  // chunks per hidden layer
  extern __shared__ __align__(128) unsigned char smem[];
  float* act = reinterpret_cast<float*>(smem);                  // [WP][128]
  float* wbuf = act + WP * kTile;                                // [2][KC][WP]
  float* w0t = wbuf + 2 * kKC * WP;                              // [3][WP]
  float* b0 = w0t + 3 * WP;                                      // [WP]
  const int nh = a.lay.nh;
  float* bh = b0 + WP;                                           // [nh][WP]
  float* wout = bh + (nh > 0 ? nh : 1) * WP;                     // [WP]
  float* pts = wout + WP;                                        // [128][3]
  int64_t* pidx = reinterpret_cast<int64_t*>(pts + kTile * 3);   // [128]
  float* fout = reinterpret_cast<float*>(pidx + kTile);          // [128]
  uint64_t* bar = reinterpret_cast<uint64_t*>(fout + kTile);     // [2]

  const int tid = threadIdx.x;
  const int tx = tid % TX;
  const int ty = tid / TX;
  const float4* act4 = reinterpret_cast<const float4*>(act);

  const int64_t n = level_point_count(a);
  const int64_t ntiles = (n + PT - 1) / PT;
  if ((int64_t)blockIdx.x >= ntiles) return;
  const int64_t my_tiles = (ntiles - 1 - blockIdx.x) / gridDim.x + 1;
  const int64_t cpt = (int64_t)nh * CPL;  // chunks per tile
  const int64_t total_chunks = my_tiles * cpt;

  // constants of this level into shared memory
  const float* pk = reinterpret_cast<const float*>(a.packed);
  for (int i = tid; i < 3 * WP; i += kThreads) w0t[i] = pk[a.lay.w0t / 4 + i];
  for (int i = tid; i < WP; i += kThreads) {
    b0[i] = pk[a.lay.b0 / 4 + i];
    wout[i] = pk[a.lay.wout / 4 + i];
  }
  for (int l = 1; l <= nh; ++l)
    for (int i = tid; i < WP; i += kThreads) bh[(l - 1) * WP + i] = pk[a.lay.bh[l] / 4 + i];
  const float bout = pk[a.lay.bout / 4];
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  __syncthreads();

  auto issue = [&](int64_t g) {
    const int within = (int)(g % cpt);
    const int l = 1 + within / CPL;
    const int c = within % CPL;
    const float* src = pk + a.lay.wht[l] / 4 + (int64_t)c * kKC * WP;
    uint64_t* b = &bar[g & 1];
    mbar_arrive_expect_tx(b, kKC * WP * 4);
    tma_bulk_g2s(wbuf + (g & 1) * kKC * WP, src, kKC * WP * 4, b);
  };
  int64_t issued = 0;  // chunks issued so far (thread 0)
  if (tid == 0 && total_chunks > 0) {
    issue(0);
    issued = 1;
  }

  int64_t g = 0;  // next chunk to consume
  bool ok = true;
  float acc[8][FPT];

  for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    // ---- points of this tile
    if (tid < PT) {
      const int64_t q = t * PT + tid;
      int64_t p = -1;
      float x = 0.f, y = 0.f, z = 0.f;
      if (q < n) load_point(a, q, p, x, y, z);
      pts[tid * 3 + 0] = x;
      pts[tid * 3 + 1] = y;
      pts[tid * 3 + 2] = z;
      pidx[tid] = p;
    }
    __syncthreads();

    // ---- layer 0: acc = W0 x (+ b0 in the epilogue)
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
      const int pt = GRAD ? row >> 2 : row;
      const int ch = GRAD ? (i & 3) : 0;  // 0: value row, 1..3: d/dx_(ch-1)
      const float x = pts[pt * 3 + 0], y = pts[pt * 3 + 1], z = pts[pt * 3 + 2];
#pragma unroll
      for (int f = 0; f < FPT; ++f) {
        const int j = tx * 4 + (f & 3) + 4 * TX * (f >> 2);
        if (ch == 0) {
          float s = __fmul_rn(x, w0t[j]);
          s = __fmaf_rn(y, w0t[WP + j], s);
          acc[i][f] = __fmaf_rn(z, w0t[2 * WP + j], s);
        } else {
          acc[i][f] = w0t[(ch - 1) * WP + j];
        }
      }
    }

    for (int layer = 0; layer <= nh; ++layer) {
      if (layer > 0) {
        // ---- hidden GEMM: acc[p][j] = sum_k act[k][p] * Wt[k][j]
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int f = 0; f < FPT; ++f) acc[i][f] = 0.f;
        for (int c = 0; c < CPL; ++c, ++g) {
          if (tid == 0 && g + 1 < total_chunks) {
            issue(g + 1);
            issued = g + 2;
          }
          // block-uniform decision, so a timeout never strands a barrier
          const bool got = mbar_wait(&bar[g & 1], (uint32_t)((g >> 1) & 1), a.status);
          if (!__syncthreads_and(got)) {
            ok = false;
            break;
          }
          const float4* w4 = reinterpret_cast<const float4*>(wbuf + (g & 1) * kKC * WP);
          const int k0 = c * kKC;
#pragma unroll 4
          for (int kk = 0; kk < kKC; ++kk) {
            const float4 a0 = act4[(k0 + kk) * (kTile / 4) + ty];
            const float4 a1 = act4[(k0 + kk) * (kTile / 4) + 16 + ty];
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
              const float4 w = w4[kk * (WP / 4) + tx + TX * q];
              const float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
              for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[i][q * 4 + r] = __fmaf_rn(av[i], wv[r], acc[i][q * 4 + r]);
            }
          }
          __syncthreads();
        }
        if (!ok) break;
      } else {
        __syncthreads();  // act free (previous tile done with it)
      }

      // ---- epilogue of this layer: s = sin(omega * (acc + b))
      const float om = a.omega[layer];
      const float* bias = layer == 0 ? b0 : bh + (layer - 1) * WP;
      if (GRAD && a.pre) {
        // training: keep the pre-activations of every row for the backward
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int row = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
          const int64_t qq = t * PT + (row >> 2);
          if (qq < n) {
            float* dst = a.pre + (((int64_t)layer * n + qq) * 4 + (i & 3)) * WP;
#pragma unroll
            for (int f4 = 0; f4 < FPT / 4; ++f4) {
              const int j = tx * 4 + 4 * TX * f4;
              float4 v;
              const bool val = (i & 3) == 0;
              v.x = val ? __fadd_rn(acc[i][4 * f4 + 0], bias[j + 0]) : acc[i][4 * f4 + 0];
              v.y = val ? __fadd_rn(acc[i][4 * f4 + 1], bias[j + 1]) : acc[i][4 * f4 + 1];
              v.z = val ? __fadd_rn(acc[i][4 * f4 + 2], bias[j + 2]) : acc[i][4 * f4 + 2];
              v.w = val ? __fadd_rn(acc[i][4 * f4 + 3], bias[j + 3]) : acc[i][4 * f4 + 3];
              *reinterpret_cast<float4*>(dst + j) = v;
            }
          }
        }
      }
      if (layer < nh) {
        float4* actw = reinterpret_cast<float4*>(act);
#pragma unroll
        for (int f = 0; f < FPT; ++f) {
          const int j = tx * 4 + (f & 3) + 4 * TX * (f >> 2);
          const float bj = bias[j];
          float s[8];
          if (GRAD) {
#pragma unroll
            for (int gq = 0; gq < 2; ++gq) {
              float sv, cv;
              sincosf(__fmul_rn(om, __fadd_rn(acc[4 * gq][f], bj)), &sv, &cv);
              cv = __fmul_rn(om, cv);
              s[4 * gq] = sv;
#pragma unroll
              for (int k = 1; k < 4; ++k) s[4 * gq + k] = __fmul_rn(cv, acc[4 * gq + k][f]);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) s[i] = sinf(__fmul_rn(om, __fadd_rn(acc[i][f], bj)));
          }
          actw[j * (kTile / 4) + ty] = make_float4(s[0], s[1], s[2], s[3]);
          actw[j * (kTile / 4) + 16 + ty] = make_float4(s[4], s[5], s[6], s[7]);
        }
        __syncthreads();
      } else {
        // last sine layer: fold straight into the output layer
        float part[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) part[i] = 0.f;
#pragma unroll
        for (int f = 0; f < FPT; ++f) {
          const int j = tx * 4 + (f & 3) + 4 * TX * (f >> 2);
          const float bj = bias[j], wj = wout[j];
          if (GRAD) {
#pragma unroll
            for (int gq = 0; gq < 2; ++gq) {
              float sv, cv;
              sincosf(__fmul_rn(om, __fadd_rn(acc[4 * gq][f], bj)), &sv, &cv);
              cv = __fmul_rn(om, cv);
              part[4 * gq] = __fmaf_rn(sv, wj, part[4 * gq]);
#pragma unroll
              for (int k = 1; k < 4; ++k)
                part[4 * gq + k] = __fmaf_rn(__fmul_rn(cv, acc[4 * gq + k][f]), wj, part[4 * gq + k]);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i)
              part[i] = __fmaf_rn(sinf(__fmul_rn(om, __fadd_rn(acc[i][f], bj))), wj, part[i]);
          }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
#pragma unroll
          for (int o = TX / 2; o >= 1; o >>= 1) part[i] += __shfl_xor_sync(0xffffffffu, part[i], o);
        }
        if (tx == 0) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int row = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
            const bool value_row = !GRAD || (i & 3) == 0;
            fout[row] = value_row ? __fadd_rn(part[i], bout) : part[i];
          }
        }
        __syncthreads();
      }
    }
    if (!ok) break;

    // ---- store / accumulate + fused band compaction
    if (tid < PT) {
      const int64_t q = t * PT + tid;
      if (GRAD) {
        const int64_t p = pidx[tid];
        if (q < n && a.G) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float gk = fout[4 * tid + 1 + k];
            a.G[3 * p + k] = a.store_mode == MPL_ACCUMULATE ? __fadd_rn(a.G[3 * p + k], gk) : gk;
          }
        }
        store_and_band(a, q < n, p, fout[4 * tid]);
      } else {
        store_and_band(a, q < n, pidx[tid], fout[tid]);
      }
    }
    __syncthreads();
  }
  if (!ok && tid == 0) {
    // a wait gave up: let copies already in flight land before exiting
    for (int64_t h = g; h < issued; ++h) mbar_wait(&bar[h & 1], (uint32_t)((h >> 1) & 1), a.status);
  }
}

template <int WP, bool GRAD>
int launch_fp32_wp(const LevelArgs& a, cudaStream_t s) {
  constexpr int PT = GRAD ? kTile / 4 : kTile;
  const size_t smem = Fp32Smem<WP>::bytes(a.lay.nh);
  MPL_CUDA_TRY(cudaFuncSetAttribute(level_fp32_kernel<WP, GRAD>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  if (!a.n_dev) {
    const int64_t ntiles = (a.n + PT - 1) / PT;
    grid = ntiles < grid ? ntiles : grid;
  }
  if (grid <= 0) return MPL_OK;
  level_fp32_kernel<WP, GRAD><<<(unsigned)grid, Fp32Threads<WP>::kThreads, smem, s>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

template <bool GRAD>
int launch_fp32_mode(const LevelArgs& a, cudaStream_t s) {
  switch (a.lay.WP) {
    case 64: return launch_fp32_wp<64, GRAD>(a, s);
    case 128: return launch_fp32_wp<128, GRAD>(a, s);
    case 256: return launch_fp32_wp<256, GRAD>(a, s);
    default: return MPL_ERR_UNSUPPORTED;
  }
}

}  // namespace

int launch_level_fp32(const LevelArgs& a, cudaStream_t s) {
  return a.grad ? launch_fp32_mode<true>(a, s) : launch_fp32_mode<false>(a, s);
}

}  // namespace mpl
