// Training kernels (FP32): the hand-written backward of one level through
// its forward-mode graph, so that one reverse pass yields the weight
// gradients of a loss on both f and df/dx (the double backward the eikonal
// and normal terms need), the residual-level loss of
// i3d/loss_functions.py:327-394 with its seeds, and Adam.
//
// Per layer l and point, the forward-mode rows are v (value) and t_k
// (d/dx_k).  With a_l the pre-activations (value row with bias), z = w a_v,
// s = sin z, c = w cos z:
//   out_v = s,  out_tk = c a_tk.
// Given d_out (the loss derivative w.r.t. out) the backward is
//   d_a_tk = c d_out_tk
//   d_z    = d_out_v cos z - w sin z sum_k d_out_tk a_tk
//   d_a_v  = w d_z
//   dW_l  += sum_rows d_a (x) in_l,  db_l += sum_points d_a_v,
//   d_out_(l-1) = d_a W_l  (for every row).
// The output layer starts it: d_out = seed_row * W_L, where the seeds are
// dL/df (value row) and dL/d(df/dx_k) (tangent rows).
#include <math.h>
#include <string.h>

#include "level.cuh"
#include "train_loss.cuh"

namespace mpl {

namespace {

constexpr int kRows = 128;  // rows per tile = 32 points x 4
constexpr int kPts = 32;
constexpr int kThreads = 256;
constexpr int kKC = 32;

struct TrainArgs {
  const char* packed;
  PackLayout lay;
  float omega[MPL_MAX_LAYERS];
  int64_t n;
  const float* xyz;   // [n, 3]
  const float* pre;   // [nh + 1][n][4][WP]
  const float* seed;  // [n][4]
  float* da;          // [nh + 1][n][4][WP]
  int* status;
};

// d_out of the last hidden layer from the seeds, then down the layers.
template <int WP>
__global__ void __launch_bounds__(kThreads, 1) train_backward_kernel(const TrainArgs a) {
  constexpr int FPT = WP / 16;
  constexpr int NQ = FPT / 4;
  constexpr int CPL = WP / kKC;
  extern __shared__ __align__(128) unsigned char smem[];
  float* act = reinterpret_cast<float*>(smem);  // d_a, [WP][128] feature-major
  float* wbuf = act + WP * kRows;                // [2][KC][WP]
  float* wout = wbuf + 2 * kKC * WP;             // [WP]
  uint64_t* bar = reinterpret_cast<uint64_t*>(wout + WP);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int nh = a.lay.nh;
  const int64_t ntiles = (a.n + kPts - 1) / kPts;
  if ((int64_t)blockIdx.x >= ntiles) return;
  const int64_t my_tiles = (ntiles - 1 - blockIdx.x) / gridDim.x + 1;
  const float* pk = reinterpret_cast<const float*>(a.packed);
  for (int i = tid; i < WP; i += kThreads) wout[i] = pk[a.lay.wout / 4 + i];
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  // weight chunks: hidden layers nh..1 (descending), CPL chunks each, per tile
  const int64_t cpt = (int64_t)nh * CPL;
  const int64_t total = my_tiles * cpt;
  auto issue = [&](int64_t g) {
    const int within = (int)(g % cpt);
    const int l = nh - within / CPL;
    const int c = within % CPL;
    const float* src = pk + a.lay.whn[l] / 4 + (int64_t)c * kKC * WP;
    mbar_arrive_expect_tx(&bar[g & 1], kKC * WP * 4);
    tma_bulk_g2s(wbuf + (g & 1) * kKC * WP, src, kKC * WP * 4, &bar[g & 1]);
  };
  int64_t issued = 0;
  if (tid == 0 && total > 0) {
    issue(0);
    issued = 1;
  }
  int64_t g = 0;
  bool ok = true;
  float dout[8][FPT];
  const float4* act4 = reinterpret_cast<const float4*>(act);
  for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    // d_out of the last hidden layer: seed of the row times W_L
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
      const int64_t q = t * kPts + (row >> 2);
      const float sd = q < a.n ? a.seed[q * 4 + (i & 3)] : 0.f;
#pragma unroll
      for (int f = 0; f < FPT; ++f) dout[i][f] = sd * wout[tx * 4 + (f & 3) + 64 * (f >> 2)];
    }
    for (int l = nh; l >= 0 && ok; --l) {
      const float om = a.omega[l];
      // d_a from d_out and this layer's pre-activations
#pragma unroll
      for (int gq = 0; gq < 2; ++gq) {
        const int row0 = gq == 0 ? ty * 4 : 64 + ty * 4;
        const int64_t q = t * kPts + (row0 >> 2);
        const bool valid = q < a.n;
        const float* pr = a.pre + (((int64_t)l * a.n + q) * 4) * WP;
        float* dar = a.da + (((int64_t)l * a.n + q) * 4) * WP;
#pragma unroll
        for (int f4 = 0; f4 < FPT / 4; ++f4) {
          const int j = tx * 4 + 64 * f4;
          float4 av[4] = {make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0),
                          make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
          if (valid) {
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) av[ch] = *reinterpret_cast<const float4*>(pr + ch * WP + j);
          }
          float4 dv[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const float* ar = reinterpret_cast<const float*>(av);  // av[ch] comp r -> ar[ch*4+r]
            float s, cz;
            sincosf(__fmul_rn(om, ar[0 * 4 + r]), &s, &cz);
            const float c = __fmul_rn(om, cz);
            const int f = 4 * f4 + r;
            const float dtx = dout[4 * gq + 1][f], dty = dout[4 * gq + 2][f],
                        dtz = dout[4 * gq + 3][f];
            float dc = __fmul_rn(dtx, ar[1 * 4 + r]);
            dc = __fmaf_rn(dty, ar[2 * 4 + r], dc);
            dc = __fmaf_rn(dtz, ar[3 * 4 + r], dc);
            const float dz = __fsub_rn(__fmul_rn(dout[4 * gq][f], cz), __fmul_rn(__fmul_rn(dc, om), s));
            reinterpret_cast<float*>(&dv[0])[r] = valid ? __fmul_rn(om, dz) : 0.f;
            reinterpret_cast<float*>(&dv[1])[r] = valid ? __fmul_rn(c, dtx) : 0.f;
            reinterpret_cast<float*>(&dv[2])[r] = valid ? __fmul_rn(c, dty) : 0.f;
            reinterpret_cast<float*>(&dv[3])[r] = valid ? __fmul_rn(c, dtz) : 0.f;
          }
          if (valid) {
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) *reinterpret_cast<float4*>(dar + ch * WP + j) = dv[ch];
          }
          if (l > 0) {
            // feature-major copy of d_a for the GEMM below
            float4* actw = reinterpret_cast<float4*>(act);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
              const int jj = j + r;
              actw[jj * (kRows / 4) + (gq == 0 ? ty : 16 + ty)] =
                  make_float4(reinterpret_cast<float*>(&dv[0])[r], reinterpret_cast<float*>(&dv[1])[r],
                              reinterpret_cast<float*>(&dv[2])[r], reinterpret_cast<float*>(&dv[3])[r]);
            }
          }
        }
      }
      if (l == 0) break;
      __syncthreads();
      // d_out of layer l-1 = d_a W_l (K = this layer's features)
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int f = 0; f < FPT; ++f) dout[i][f] = 0.f;
      for (int c = 0; c < CPL; ++c, ++g) {
        if (tid == 0 && g + 1 < total) {
          issue(g + 1);
          issued = g + 2;
        }
        const bool got = mbar_wait(&bar[g & 1], (uint32_t)((g >> 1) & 1), a.status);
        if (!__syncthreads_and(got)) {
          ok = false;
          break;
        }
        const float4* w4 = reinterpret_cast<const float4*>(wbuf + (g & 1) * kKC * WP);
        const int k0 = c * kKC;
#pragma unroll 4
        for (int kk = 0; kk < kKC; ++kk) {
          const float4 a0 = act4[(k0 + kk) * (kRows / 4) + ty];
          const float4 a1 = act4[(k0 + kk) * (kRows / 4) + 16 + ty];
          const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
          for (int q4 = 0; q4 < NQ; ++q4) {
            const float4 w = w4[kk * (WP / 4) + tx + 16 * q4];
            const float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
              for (int r = 0; r < 4; ++r)
                dout[i][q4 * 4 + r] = __fmaf_rn(av[i], wv[r], dout[i][q4 * 4 + r]);
          }
        }
        __syncthreads();
      }
    }
  }
  if (!ok && tid == 0) {
    for (int64_t h = g; h < issued; ++h) mbar_wait(&bar[h & 1], (uint32_t)((h >> 1) & 1), a.status);
  }
}

// in_l of a hidden layer l >= 1 for row ch of a point, feature k, from the
// pre-activations of layer l-1: value sin(w a_v), tangent w cos(w a_v) a_t.
__device__ __forceinline__ float layer_input(const float* pre_prev_point, int WP, int ch, int k,
                                             float om) {
  const float zv = __fmul_rn(om, pre_prev_point[k]);
  if (ch == 0) return sinf(zv);
  return __fmul_rn(__fmul_rn(om, cosf(zv)), pre_prev_point[ch * WP + k]);
}

// dW_l[j][k] += sum over rows of da_l[row][j] * in_l[row][k] (l >= 1), and
// db_l[j] += sum over points of da_l[value row][j].  CTA tile 64 x 64,
// split over points by blockIdx.z, partial sums added atomically.
__global__ void __launch_bounds__(256) train_wgrad_hidden_kernel(const TrainArgs a, int l, int WP,
                                                                 float* dW, float* db) {
  __shared__ float sA[32][65];  // d_a rows x j
  __shared__ float sB[32][65];  // in rows x k
  const int j0 = blockIdx.x * 64, k0 = blockIdx.y * 64;
  const int tid = threadIdx.x, tj = tid >> 4, tk = tid & 15;
  const int64_t per = (a.n + gridDim.z - 1) / gridDim.z;
  const int64_t q_begin = blockIdx.z * per;
  const int64_t q_end = q_begin + per < a.n ? q_begin + per : a.n;
  const float omp = a.omega[l - 1];
  float acc[4][4] = {};
  float bacc = 0.f;
  for (int64_t q0 = q_begin; q0 < q_end; q0 += 8) {
    // 8 points = 32 rows
    for (int e = tid; e < 32 * 64; e += 256) {
      const int r = e >> 6, c = e & 63;
      const int64_t q = q0 + (r >> 2);
      float va = 0.f, vb = 0.f;
      if (q < q_end) {
        va = a.da[(((int64_t)l * a.n + q) * 4 + (r & 3)) * WP + j0 + c];
        vb = layer_input(a.pre + (((int64_t)(l - 1) * a.n + q) * 4) * WP, WP, r & 3, k0 + c, omp);
      }
      sA[r][c] = va;
      sB[r][c] = vb;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < 32; ++r) {
      float av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        av[u] = sA[r][tj * 4 + u];
        bv[u] = sB[r][tk * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = __fmaf_rn(av[u], bv[v], acc[u][v]);
    }
    if (blockIdx.y == 0 && tid < 64) {
      for (int r = 0; r < 32; r += 4) bacc += sA[r][tid];
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + tj * 4 + u, k = k0 + tk * 4 + v;
      atomicAdd(&dW[(int64_t)j * WP + k], acc[u][v]);
    }
  if (blockIdx.y == 0 && tid < 64) atomicAdd(&db[j0 + tid], bacc);
}

// Layer 0 (3 inputs): dW0[j][c] += sum_q da_v[j] x_qc + da_tc[j]; db0[j] += da_v[j].
// Output layer: dWL[j] += sum_rows seed_row out_(L-1)[row][j]; dbL += seed_v.
// Thread j of a block, 8 points per step; each block covers a contiguous
// point range and adds its partial sums atomically.
__global__ void __launch_bounds__(256) train_wgrad_ends_kernel(const TrainArgs a, int WP,
                                                               float* dW0, float* db0, float* dWL,
                                                               float* dbL) {
  const int nh = a.lay.nh;
  const int64_t per = (a.n + gridDim.x - 1) / gridDim.x;
  const int64_t q_begin = blockIdx.x * per;
  const int64_t q_end = q_begin + per < a.n ? q_begin + per : a.n;
  const float om = a.omega[nh];
  for (int j = threadIdx.x; j < WP; j += blockDim.x) {
    float w0x = 0.f, w0y = 0.f, w0z = 0.f, b0 = 0.f, wl = 0.f;
    for (int64_t q = q_begin; q < q_end; ++q) {
      const float* d = a.da + (q * 4) * WP;  // layer 0
      const float dv = d[j];
      w0x = __fadd_rn(w0x, __fmaf_rn(dv, a.xyz[3 * q + 0], d[1 * WP + j]));
      w0y = __fadd_rn(w0y, __fmaf_rn(dv, a.xyz[3 * q + 1], d[2 * WP + j]));
      w0z = __fadd_rn(w0z, __fmaf_rn(dv, a.xyz[3 * q + 2], d[3 * WP + j]));
      b0 = __fadd_rn(b0, dv);
      const float* pr = a.pre + (((int64_t)nh * a.n + q) * 4) * WP;
      const float4 sd = *reinterpret_cast<const float4*>(a.seed + q * 4);
      float s, c;
      sincosf(__fmul_rn(om, pr[j]), &s, &c);
      const float oc = __fmul_rn(om, c);
      float t = __fmul_rn(sd.y, pr[1 * WP + j]);
      t = __fmaf_rn(sd.z, pr[2 * WP + j], t);
      t = __fmaf_rn(sd.w, pr[3 * WP + j], t);
      wl = __fmaf_rn(sd.x, s, __fmaf_rn(oc, t, wl));
    }
    atomicAdd(&dW0[j * 3 + 0], w0x);
    atomicAdd(&dW0[j * 3 + 1], w0y);
    atomicAdd(&dW0[j * 3 + 2], w0z);
    atomicAdd(&db0[j], b0);
    atomicAdd(&dWL[j], wl);
  }
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int64_t q = q_begin; q < q_end; ++q) b = __fadd_rn(b, a.seed[q * 4]);
    atomicAdd(dbL, b);
  }
}

// The trainers' losses per point (train_loss.cuh) and their seeds; the four
// term sums per block are added atomically.
__global__ void train_loss_kernel(int64_t n, const float* __restrict__ f, const float* __restrict__ g,
                                  const float* __restrict__ Ff, const float* __restrict__ Gf,
                                  const float* __restrict__ gt_sdf,
                                  const float* __restrict__ gt_n, const LossParams L,
                                  float* __restrict__ seed, float* __restrict__ loss) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float term[4] = {0.f, 0.f, 0.f, 0.f};
  if (q < n) {
    const float S = __fadd_rn(f[q], Ff ? Ff[q] : 0.f);
    float G[3], N[3];
    for (int c = 0; c < 3; ++c) {
      G[c] = __fadd_rn(g[3 * q + c], Gf ? Gf[3 * q + c] : 0.f);
      N[c] = gt_n[3 * q + c];
    }
    float phi, gam[3];
    point_loss(L, S, G, gt_sdf[q], N, phi, gam, term);
    seed[4 * q] = phi;
    for (int c = 0; c < 3; ++c) seed[4 * q + 1 + c] = gam[c];
  }
  for (int k = 0; k < 4; ++k) {
    float v = term[k];
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.f) atomicAdd(&loss[k], v);
  }
}

struct AdamTensor {
  float* p;
  const float* g;
  float* m;
  float* v;
  int64_t n;
};

constexpr int kMaxAdam = 2 * MPL_MAX_LAYERS;

struct AdamArgs {
  AdamTensor t[kMaxAdam];
  int count;
  float lr, beta1, beta2, eps, bc1, bc2_sqrt;
};

// torch.optim.Adam (no weight decay, no amsgrad): m, v moments, bias
// corrections bc1 = 1 - beta1^t and sqrt(1 - beta2^t) computed on the host.
__global__ void adam_kernel(const AdamArgs a) {
  const AdamTensor& T = a.t[blockIdx.y];
  const float step = a.lr / a.bc1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float g = T.g[i];
    const float m = __fmaf_rn(1.0f - a.beta1, __fsub_rn(g, T.m[i]), T.m[i]);  // lerp
    const float v = __fadd_rn(__fmul_rn(a.beta2, T.v[i]), __fmul_rn(__fmul_rn(1.0f - a.beta2, g), g));
    T.m[i] = m;
    T.v[i] = v;
    const float denom = __fadd_rn(__fdiv_rn(sqrtf(v), a.bc2_sqrt), a.eps);
    T.p[i] = __fsub_rn(T.p[i], __fmul_rn(step, __fdiv_rn(m, denom)));
  }
}

// Counter-based random numbers for batches drawn on the device: SplitMix64
// (Steele, Lea and Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014) applied to seed + index.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// create_training_data_on_neighborhood (experiment_scripts/utils.py:92-169)
// for sample i: surface row i, the normal offset row n + i and, with
// dithering, row 2n + i, each with the reference's float32 operation order.
__global__ void train_batch_kernel(const float* __restrict__ V, int64_t M, int C,
                                   const int64_t* __restrict__ idx, const float* __restrict__ u,
                                   int64_t n, float delta, float half_delta, float delta_eps,
                                   int neigh, int dither, uint64_t seed, float* __restrict__ pts,
                                   float* __restrict__ nrm, float* __restrict__ sdf, int* status) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r;
    if (idx) {
      r = idx[i];
    } else {
      r = (int64_t)((splitmix64(seed * 0x100000001b3ull + (uint64_t)i) >> 11) % (uint64_t)M);
    }
    float x[3] = {0.f, 0.f, 0.f}, nm[3] = {0.f, 0.f, 0.f}, dn = delta_eps, uu[3];
    if (r >= 0 && r < M) {
      const float* v = V + r * C;
      for (int c = 0; c < 3; ++c) {
        x[c] = v[c];
        nm[c] = v[3 + c];
      }
      if (neigh) dn = v[C - 1];
    } else {
      report_device_error(status, MPL_ERR_INVALID_ARG);
    }
    for (int c = 0; c < 3; ++c) {
      if (u) {
        uu[c] = u[3 * i + c];
      } else {
        const uint64_t h = splitmix64((seed ^ 0x5bd1e9955bd1e995ull) + 3ull * (uint64_t)i + c);
        uu[c] = (float)(h >> 40) * 0x1p-24f;
      }
    }
    const float s = __fmul_rn(dn, uu[2]);
    for (int c = 0; c < 3; ++c) {
      pts[3 * i + c] = x[c];
      pts[3 * (n + i) + c] = __fadd_rn(x[c], __fmul_rn(s, nm[c]));
      nrm[3 * i + c] = nm[c];
      nrm[3 * (n + i) + c] = nm[c];
    }
    sdf[i] = 0.f;
    sdf[n + i] = s;
    if (dither) {
      for (int c = 0; c < 3; ++c) {
        pts[3 * (2 * n + i) + c] =
            __fadd_rn(__fmul_rn(uu[c], delta), __fadd_rn(x[c], __fmul_rn(half_delta, nm[c])));
        nrm[3 * (2 * n + i) + c] = nm[c];
      }
      sdf[2 * n + i] = -1.f;
    }
  }
}

template <int WP>
int launch_backward_wp(const TrainArgs& t, cudaStream_t s) {
  const size_t smem = (size_t)WP * kRows * 4 + 2ull * kKC * WP * 4 + WP * 4 + 16;
  MPL_CUDA_TRY(cudaFuncSetAttribute(train_backward_kernel<WP>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = sm_count();
  const int64_t ntiles = (t.n + kPts - 1) / kPts;
  grid = ntiles < grid ? ntiles : grid;
  train_backward_kernel<WP><<<(unsigned)grid, kThreads, smem, s>>>(t);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

}  // namespace

}  // namespace mpl

using namespace mpl;

extern "C" int mpl_train_scratch_floats(const MplNet* net, int64_t n, int64_t* floats) {
  PackLayout lay;
  int st = make_layout(net, &lay);
  if (st != MPL_OK) return st;
  if (!floats || n < 0) return MPL_ERR_INVALID_ARG;
  *floats = (int64_t)(lay.nh + 1) * n * 4 * lay.WP;
  return MPL_OK;
}

extern "C" int mpl_train_forward(const MplNet* net, const void* packed, const float* xyz, int64_t n,
                                 float* S, float* G, float* pre, void* stream) {
  if (!net || !packed || (!xyz && n) || !S || !G || !pre || n < 0 || n > INT32_MAX)
    return MPL_ERR_INVALID_ARG;
  LevelArgs a;
  memset(&a, 0, sizeof(a));
  int st = make_layout(net, &a.lay);
  if (st != MPL_OK) return st;
  if (n == 0) return MPL_OK;
  a.packed = (const char*)packed;
  for (int l = 0; l < MPL_MAX_LAYERS; ++l) a.omega[l] = net->omega[l];
  a.pts.kind = MPL_POINTS_XYZ;
  a.pts.xyz = xyz;
  a.n = n;
  a.S = S;
  a.G = G;
  a.grad = 1;
  a.store_mode = MPL_STORE;
  a.pre = pre;
  a.status = device_status_ptr();
  return launch_level_fp32(a, (cudaStream_t)stream);
}

extern "C" int mpl_train_loss(int64_t n, const float* f, const float* g, const float* f_frozen,
                              const float* g_frozen, const float* gt_sdf, const float* gt_normals,
                              const MplLoss* loss, float* seeds, float* loss_sums, void* stream) {
  if (!f || !g || !gt_sdf || !gt_normals || !seeds || !loss_sums || n < 0) return MPL_ERR_INVALID_ARG;
  LossParams L;
  int st = loss_params(loss, n, &L);
  if (st != MPL_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  MPL_CUDA_TRY(cudaMemsetAsync(loss_sums, 0, 4 * sizeof(float), s));
  if (n == 0) return MPL_OK;
  train_loss_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      n, f, g, f_frozen, g_frozen, gt_sdf, gt_normals, L, seeds, loss_sums);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_train_backward(const MplNet* net, const void* packed, const float* xyz,
                                  int64_t n, const float* pre, const float* seeds, float* da,
                                  float* const* dW, float* const* db, void* stream) {
  if (!net || !packed || !pre || !seeds || !da || !dW || !db || n < 0 || n > INT32_MAX)
    return MPL_ERR_INVALID_ARG;
  TrainArgs t;
  memset(&t, 0, sizeof(t));
  int st = make_layout(net, &t.lay);
  if (st != MPL_OK) return st;
  const int L = t.lay.L, nh = t.lay.nh, WP = t.lay.WP;
  for (int l = 0; l < L; ++l)
    if (!dW[l] || !db[l]) return MPL_ERR_INVALID_ARG;
  // the gradient buffers use the padded widths; callers size them with WP
  if (n == 0) return MPL_OK;
  t.packed = (const char*)packed;
  for (int l = 0; l < MPL_MAX_LAYERS; ++l) t.omega[l] = net->omega[l];
  t.n = n;
  t.xyz = xyz;
  t.pre = pre;
  t.seed = seeds;
  t.da = da;
  t.status = device_status_ptr();
  cudaStream_t s = (cudaStream_t)stream;
  switch (WP) {
    case 64: st = launch_backward_wp<64>(t, s); break;
    case 128: st = launch_backward_wp<128>(t, s); break;
    case 256: st = launch_backward_wp<256>(t, s); break;
    default: return MPL_ERR_UNSUPPORTED;
  }
  if (st != MPL_OK) return st;
  const int splits = (int)((n + 4095) / 4096) < 64 ? (int)((n + 4095) / 4096) : 64;
  for (int l = 1; l <= nh; ++l) {
    dim3 grid(WP / 64, WP / 64, splits < 1 ? 1 : splits);
    train_wgrad_hidden_kernel<<<grid, 256, 0, s>>>(t, l, WP, dW[l], db[l]);
    MPL_LAUNCH_CHECK();
  }
  // about 64 points per block
  const int64_t eb = (n + 63) / 64 < 4096 ? (n + 63) / 64 : 4096;
  train_wgrad_ends_kernel<<<(unsigned)eb, WP < 256 ? WP : 256, 0, s>>>(t, WP, dW[0], db[0],
                                                                       dW[L - 1], db[L - 1]);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_train_batch(const float* vertices, int64_t n_vertices, int32_t row_floats,
                               const int64_t* sample_index, const float* uniforms, int64_t n,
                               float delta, float delta_eps, int32_t flags, uint64_t seed,
                               float* pts, float* normals, float* sdf, void* stream) {
  if (!vertices || !pts || !normals || !sdf || n < 0 || n > n_vertices || row_floats < 6 ||
      (flags & ~(MPL_BATCH_NEIGH_DELTA | MPL_BATCH_DITHER)))
    return MPL_ERR_INVALID_ARG;
  if ((flags & MPL_BATCH_NEIGH_DELTA) && row_floats < 7) return MPL_ERR_INVALID_ARG;
  if (n == 0) return MPL_OK;
  const int64_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  train_batch_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      vertices, n_vertices, row_floats, sample_index, uniforms, n, delta,
      (float)(0.5 * (double)delta), delta_eps, (flags & MPL_BATCH_NEIGH_DELTA) != 0,
      (flags & MPL_BATCH_DITHER) != 0, seed, pts, normals, sdf, device_status_ptr());
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}

extern "C" int mpl_adam_step(int32_t count, float* const* params, const float* const* grads,
                             float* const* exp_avg, float* const* exp_avg_sq, const int64_t* numel,
                             float lr, float beta1, float beta2, float eps, int64_t step,
                             void* stream) {
  if (count <= 0 || count > kMaxAdam || !params || !grads || !exp_avg || !exp_avg_sq || !numel ||
      step < 1)
    return MPL_ERR_INVALID_ARG;
  AdamArgs a;
  memset(&a, 0, sizeof(a));
  int64_t maxn = 0;
  for (int i = 0; i < count; ++i) {
    a.t[i] = AdamTensor{params[i], grads[i], exp_avg[i], exp_avg_sq[i], numel[i]};
    maxn = numel[i] > maxn ? numel[i] : maxn;
  }
  a.count = count;
  a.lr = lr;
  a.beta1 = beta1;
  a.beta2 = beta2;
  a.eps = eps;
  a.bc1 = (float)(1.0 - pow((double)beta1, (double)step));
  a.bc2_sqrt = (float)sqrt(1.0 - pow((double)beta2, (double)step));
  if (maxn == 0) return MPL_OK;
  dim3 grid((unsigned)((maxn + 255) / 256 < 1024 ? (maxn + 255) / 256 : 1024), (unsigned)count);
  adam_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(a);
  MPL_LAUNCH_CHECK();
  return MPL_OK;
}
