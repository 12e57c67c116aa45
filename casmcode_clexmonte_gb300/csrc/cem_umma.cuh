// The proposal network on the 5th-generation tensor cores: tcgen05.mma with
// the accumulator in tensor memory, one elected thread per warpgroup issuing
// the MMAs for the warpgroup's 128 environments (one per thread: warp q of
// the warpgroup owns rows 32q..32q+31, the tensor-memory lanes it may read).
//
//   layer 1: D[128 x 64] = X[128 x 48] * W1[48 x 64]   (3 MMAs, K = 16 each;
//            X holds the 0/1 neighbour occupants exactly in bf16, rows 42..47 0)
//   layer 2: D[128 x 64] = H1[128 x 64] * W2[64 x 64]  (4 MMAs), H1 = bf16(ReLU(D + b1))
//   logit  : z = b3 + sum_j ReLU(D_j + b2_j) w3_j, fp32, one row per thread
//
// Operands are bf16 in shared memory in the no-swizzle K-major layout of
// 8-row x 16-byte core matrices: element (row r, k) of a matrix with NK
// chunks of 8 K-elements per row sits at byte ((r / 8) * NK + k / 8) * 128 +
// (r % 8) * 16 + (k % 8) * 2, so the descriptors' leading-dimension offset
// (next K chunk) is 128 bytes and the stride-dimension offset (next 8 rows)
// NK * 128 bytes. D is fp32, 64 columns of tensor memory per warpgroup.
// MMA completion is tracked by an mbarrier (tcgen05.commit); every wait is
// bounded and reports a timeout to the caller.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "cem_kernels.cuh"
#include "cem_learned.cuh"

namespace cem {

constexpr int UMMA_NK1 = 6, UMMA_NK2 = 8;  // K chunks of 8: layer 1 (48), layer 2 (64)
constexpr int UMMA_B1_BYTES = 64 * 48 * 2, UMMA_B2_BYTES = 64 * 64 * 2;
constexpr int UMMA_A_BYTES = 128 * 64 * 2;  // one warpgroup's operand rows (layer 2 size)
constexpr int UMMA_COLS = 64;               // tensor-memory columns per warpgroup
constexpr int UMMA_WAIT_ITERS = 1 << 22;

// instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24
constexpr uint32_t UMMA_IDESC_BF16_M128_N64 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// shared-memory matrix descriptor: start address, leading-dimension and
// stride-dimension byte offsets (each >> 4, 14 bits), descriptor version 1
// (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t umma_off(int r, int chunk, int nk) {
  return (uint32_t)(((r >> 3) * nk + chunk) * 128 + (r & 7) * 16);
}

__device__ __forceinline__ void umma_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive fp32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Tensor-memory allocation by one whole warp; the base address is written to
// *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void wg_bar(int id) {
  asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory");
}

// Network tables in shared memory for the tensor-core path.
struct UmmaNet {
  unsigned char *b1, *b2;  // W1^T [64 x 48], W2^T [64 x 64], bf16 core-matrix layout
  const float *bias1, *bias2, *w3;
  float b3;
};

// W1^T and W2^T into the core-matrix layout (row n = hidden unit, K = inputs),
// fp32 biases and output weights. fb: b1[64], b2[64], w3[64], b3.
__device__ __forceinline__ void umma_load_net(const __nv_bfloat16 *__restrict__ P,
                                              unsigned char *b1, unsigned char *b2, float *fb,
                                              int tid, int nth) {
  for (int i = tid; i < 64 * 48; i += nth) {
    const int n = i / 48, k = i - 48 * (i / 48);
    const __nv_bfloat16 v = k < MLP_IN ? P[MLP_W1 + k * MLP_H + n] : __float2bfloat16_rn(0.f);
    *reinterpret_cast<__nv_bfloat16 *>(b1 + umma_off(n, k >> 3, UMMA_NK1) + (k & 7) * 2) = v;
  }
  for (int i = tid; i < 64 * 64; i += nth) {
    const int n = i >> 6, k = i & 63;
    *reinterpret_cast<__nv_bfloat16 *>(b2 + umma_off(n, k >> 3, UMMA_NK2) + (k & 7) * 2) =
        P[MLP_W2 + k * MLP_H + n];
  }
  for (int i = tid; i < MLP_H; i += nth) {
    fb[i] = __bfloat162float(P[MLP_B1 + i]);
    fb[64 + i] = __bfloat162float(P[MLP_B2 + i]);
    fb[128 + i] = __bfloat162float(P[MLP_W3 + i]);
  }
  if (tid == 0) fb[192] = __bfloat162float(P[MLP_B3]);
}

// bf16 pair of bits k and k + 1 of a 0/1 mask (lower half: element k)
__device__ __forceinline__ uint32_t umma_bits2(unsigned long long e, int k) {
  const uint32_t x = (uint32_t)(e >> k) & 3u;
  return ((x & 1u) * 0x3F80u) | ((x >> 1) * 0x3F800000u);
}

__device__ __forceinline__ uint32_t umma_pack(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// Logit of the environment `env` (bit k = neighbour k) of this thread's row.
// Collective over the warpgroup wg (all 128 threads call it together);
// abuf = the warpgroup's operand rows, tm = its 64 tensor-memory columns, bar
// = its mbarrier with phase bit `phase` (toggled twice per call). Sets
// *timeout when an MMA did not complete within the wait limit (the logit is
// then meaningless).
__device__ __forceinline__ float umma_network(const UmmaNet &N, unsigned char *abuf, uint32_t tm,
                                              uint64_t *bar, uint32_t &phase, int wg,
                                              unsigned long long env, bool &timeout) {
  const int lane = threadIdx.x & 31, wq = (threadIdx.x >> 5) & 3;
  const int row = 32 * wq + lane;
  const uint32_t tlane = tm + ((uint32_t)(32 * wq) << 16);
  // ---- layer 1 operand: the row's 48 inputs as bf16 0/1
#pragma unroll
  for (int c = 0; c < UMMA_NK1; ++c) {
    uint4 v;
    v.x = umma_bits2(env, 8 * c);
    v.y = umma_bits2(env, 8 * c + 2);
    v.z = umma_bits2(env, 8 * c + 4);
    v.w = umma_bits2(env, 8 * c + 6);
    *reinterpret_cast<uint4 *>(abuf + umma_off(row, c, UMMA_NK1)) = v;
  }
  fence_proxy_async_smem();
  tc_fence_before();
  wg_bar(1 + wg);
  if (wq == 0 && lane == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_u32(abuf), b0 = smem_u32(N.b1);
#pragma unroll
    for (int s = 0; s < UMMA_NK1 / 2; ++s)
      umma_mma(tm, umma_desc(a0 + 256 * s, 128, UMMA_NK1 * 128),
               umma_desc(b0 + 256 * s, 128, UMMA_NK1 * 128), UMMA_IDESC_BF16_M128_N64, s > 0);
    umma_commit(bar);
  }
  if (!mbar_wait(bar, phase, UMMA_WAIT_ITERS)) timeout = true;
  phase ^= 1u;
  tc_fence_after();
  // ---- layer 2 operand: bf16(ReLU(D + b1)), 32 columns at a time
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tmem_ld32(tlane + 32 * h, v);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float a[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = fmaxf(v[8 * c + i] + N.bias1[32 * h + 8 * c + i], 0.f);
      uint4 u;
      u.x = umma_pack(a[0], a[1]);
      u.y = umma_pack(a[2], a[3]);
      u.z = umma_pack(a[4], a[5]);
      u.w = umma_pack(a[6], a[7]);
      *reinterpret_cast<uint4 *>(abuf + umma_off(row, 4 * h + c, UMMA_NK2)) = u;
    }
  }
  fence_proxy_async_smem();
  tc_fence_before();
  wg_bar(1 + wg);
  if (wq == 0 && lane == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_u32(abuf), b0 = smem_u32(N.b2);
#pragma unroll
    for (int s = 0; s < UMMA_NK2 / 2; ++s)
      umma_mma(tm, umma_desc(a0 + 256 * s, 128, UMMA_NK2 * 128),
               umma_desc(b0 + 256 * s, 128, UMMA_NK2 * 128), UMMA_IDESC_BF16_M128_N64, s > 0);
    umma_commit(bar);
  }
  if (!mbar_wait(bar, phase, UMMA_WAIT_ITERS)) timeout = true;
  phase ^= 1u;
  tc_fence_after();
  float z = N.b3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tmem_ld32(tlane + 32 * h, v);
#pragma unroll
    for (int i = 0; i < 32; ++i)
      z = fmaf(fmaxf(v[i] + N.bias2[32 * h + i], 0.f), N.w3[32 * h + i], z);
  }
  tc_fence_before();  // the next call's MMAs come after these reads
  return z;
}

}  // namespace cem
