// Shared device/host helpers for libmplicits (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mplicits.h"

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
namespace mpl {

void set_last_cuda_error(cudaError_t e);

#define MPL_CUDA_TRY(expr)                         \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) {                       \
      ::mpl::set_last_cuda_error(_e);              \
      return MPL_ERR_CUDA;                         \
    }                                              \
  } while (0)

#define MPL_LAUNCH_CHECK()                         \
  do {                                             \
    cudaError_t _e = cudaGetLastError();           \
    if (_e != cudaSuccess) {                       \
      ::mpl::set_last_cuda_error(_e);              \
      return MPL_ERR_CUDA;                         \
    }                                              \
  } while (0)

// Device-side status word (one per device, in capi.cu): a bounded wait that
// gives up writes MPL_ERR_DEVICE_TIMEOUT there and its kernel returns early.
// Kernels receive its address as an argument.
int* device_status_ptr();

__device__ __forceinline__ void report_device_error(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// Iteration cap of every spin-wait (each try_wait itself may suspend for a
// bounded hardware time slice, so this is seconds of wall time at most).
constexpr uint32_t kSpinLimit = 1u << 22;

int sm_count();

// current value of a process-wide option (mpl_set_option)
int64_t option_value(int32_t option);

// ---------------------------------------------------------------------------
// grid coordinates of i3d/meshing.py:42-63 (float32 true division, fmod)
// ---------------------------------------------------------------------------
// fmod(a, b) for 0 <= a < 2^22 and an integer-valued float 2 <= b <= 2^11,
// inv_b = float32(1 / b).  The quotient estimate trunc(a * inv_b) is off by
// at most one; a - n b is a multiple of ulp(a) below 2b, so the FMA and the
// one correction are exact, and the result equals fmodf(a, b) bit for bit
// (checked on every index of the N^3 grids for N = 2..69 and for N = 127,
// 128, 129, 255, 256, 300, 384, 511, 512, 640, 777, 1000, 1023, 1024, 1290).
__device__ __forceinline__ float fmod_grid(float a, float b, float inv_b) {
  const float n = truncf(__fmul_rn(a, inv_b));
  float r = __fmaf_rn(-n, b, a);
  if (r < 0.f)
    r = __fadd_rn(r, b);
  else if (r >= b)
    r = __fsub_rn(r, b);
  return r;
}

__device__ __forceinline__ void grid_point(int64_t p, int32_t N, float vs, float off0, float off1,
                                           float off2, float& x, float& y, float& z) {
  const float fN = (float)N;
  float s0, s1, s2;
  if (p < 0x80000000ll && N <= 1290) {
    // 32-bit integer work and an exact fmod: no 64-bit division (which runs
    // on the FP64 pipe) and no library fmodf; same bits as the branch below
    const uint32_t p32 = (uint32_t)p;
    const float idx_f = __uint2float_rn(p32);
    s2 = (float)(p32 % (uint32_t)N);
    const float q1 = __fdiv_rn(idx_f, fN);
    const float inv = __frcp_rn(fN);
    s1 = fmod_grid(q1, fN, inv);
    s0 = fmod_grid(__fdiv_rn(q1, fN), fN, inv);
  } else {
    const float idx_f = __ll2float_rn(p);
    s2 = (float)(p % (int64_t)N);
    const float q1 = __fdiv_rn(idx_f, fN);
    s1 = fmodf(q1, fN);
    s0 = fmodf(__fdiv_rn(q1, fN), fN);
  }
  x = __fadd_rn(__fmul_rn(s0, vs), off0);
  y = __fadd_rn(__fmul_rn(s1, vs), off1);
  z = __fadd_rn(__fmul_rn(s2, vs), off2);
}

// ---------------------------------------------------------------------------
// mbarrier + bulk-copy (TMA) primitives, inline PTX
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// As mbar_try_wait, but the thread may be suspended in hardware for up to
// hint_ns nanoseconds while the phase is incomplete (it resumes as soon as
// the phase completes), so a waiting warp does not spin on the issue port.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wall-clock cap of a sleeping wait: far above any legitimate wait inside a
// launch (microseconds), so only a wait that can never complete reaches it.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Bounded wait for the phase with the given parity to complete.  Returns
// false (and records MPL_ERR_DEVICE_TIMEOUT) when the cap is reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  report_device_error(status, MPL_ERR_DEVICE_TIMEOUT);
  return false;
}

// 1-D bulk copy global -> shared through the TMA engine, completion counted
// in bytes on `bar`.  dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                             uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------------------
// packed weight image of one level (layout shared by host and device)
// ---------------------------------------------------------------------------
// FP32 section (plain kernels):
//   w0t   [3][WP]     W0 transposed          b0   [WP]
//   wht_l [WP][WP]    W_l transposed (k, j)  bh_l [WP]    l = 1..L-2
//   wout  [WP]        bout [4]
// BF16 section (tcgen05 kernels), omega folded in:
//   w0f   [4][WP]     rows omega0*W0[:,0], omega0*W0[:,1], omega0*W0[:,2], omega0*b0
//   hb_l  [WP]        omega_l * b_l
//   hw_l  bf16 omega_l*W_l in UMMA K-major no-swizzle core-matrix tiles,
//         split into K chunks of 64: chunk c, row n, col k lives at
//         c*WP*128 + ((n/8)*8 + (k%64)/8)*128 + (n%8)*16 + (k%8)*2 bytes.
//   hwT_l bf16 omega_l*W_l^T, same tiling (rows = input features): used by
//         the input-gradient kernels.
//   hbx_l bf16 [WP rows][16 K] bias tile of the MMA: K column 0 holds
//         bf16(omega_l*b_l), column 1 the bf16 remainder, the rest zero;
//         core-matrix layout ((n/8)*2 + k/8)*128 + (n%8)*16 + (k%8)*2 bytes
//         (LBO 128 B, SBO 256 B).  Multiplied by an A tile whose first two
//         K columns are 1, one extra K=16 MMA step adds the bias exactly to
//         ~16 bits.
//   hwh_l, hbxh_l, hwTh_l  hw_l, hbx_l and hwT_l with FP16 elements (the
//         FP16 operand mode).
//   whn_l [WP][WP] FP32 W_l untransposed (j, k): the B operand of the
//         backward GEMM d_in = d_a W_l.
struct PackLayout {
  int32_t L;    // nn.Linear layers
  int32_t WP;   // padded hidden width (64, 128 or 256)
  int32_t nh;   // hidden GEMMs = L - 2
  int64_t w0t, b0, wout, bout;
  int64_t wht[MPL_MAX_LAYERS], bh[MPL_MAX_LAYERS];
  int64_t w0f;
  int64_t hb[MPL_MAX_LAYERS];
  int64_t hw[MPL_MAX_LAYERS], hwT[MPL_MAX_LAYERS], hbx[MPL_MAX_LAYERS];
  int64_t hwh[MPL_MAX_LAYERS], hbxh[MPL_MAX_LAYERS];  // the same two tiles in FP16
  int64_t hwTh[MPL_MAX_LAYERS];                       // hwT in FP16
  int64_t whn[MPL_MAX_LAYERS];  // FP32 W_l as stored by nn.Linear, [j][k] (backward GEMM)
  int64_t total;
};

__host__ __device__ inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// Returns MPL_OK and fills `lay`, or an error for an unsupported topology.
int make_layout(const MplNet* net, PackLayout* lay);

}  // namespace mpl
