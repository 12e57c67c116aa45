// The proposal network on the 5th-generation tensor cores: tcgen05.mma with
// the accumulator in tensor memory, one elected thread per warpgroup issuing
// the MMAs for the warpgroup's 128 environments (one per thread: warp q of
// the warpgroup owns rows 32q..32q+31, the tensor-memory lanes it may read).
//
//   layer 1: D[128 x 64] = X[128 x 48] * W1'[48 x 64]  (3 MMAs, K = 16 each;
//            X holds the 0/1 neighbour occupants exactly in bf16 in columns
//            0..41 and 1 in column 42; W1' is W1 with the bias b1 as row 42,
//            so D = X W1 + b1 exactly in the bf16 parameters; columns 43..47 0)
//   layer 2: D[128 x 64] = H1[128 x 64] * W2[64 x 64]  (4 MMAs), H1 = bf16(ReLU(D))
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
// bf16 0/1 expansion of a byte: entry x = 8 bf16 (bit k of x -> element k)
constexpr int UMMA_BITS_BYTES = 256 * 16;

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
  unsigned char *b1, *b2;  // W1'^T [64 x 48], W2^T [64 x 64], bf16 core-matrix layout
  const uint4 *bits;       // byte -> 8 bf16 0/1 (UMMA_BITS_BYTES)
  const float *bias2, *w3;
  float b3;
};

// W1'^T (W1 with b1 as input row MLP_IN) and W2^T into the core-matrix layout
// (row n = hidden unit, K = inputs), the byte expansion table, fp32 layer-2
// biases and output weights. fb: b2[64], w3[64], b3 (64-float aligned).
__device__ __forceinline__ void umma_load_net(const __nv_bfloat16 *__restrict__ P,
                                              unsigned char *b1, unsigned char *b2, uint4 *bits,
                                              float *fb, int tid, int nth) {
  static_assert(MLP_IN < 48, "layer 1 keeps a spare input column for its bias");
  for (int i = tid; i < 64 * 48; i += nth) {
    const int n = i / 48, k = i - 48 * (i / 48);
    const __nv_bfloat16 v = k < MLP_IN    ? P[MLP_W1 + k * MLP_H + n]
                            : k == MLP_IN ? P[MLP_B1 + n]
                                          : __float2bfloat16_rn(0.f);
    *reinterpret_cast<__nv_bfloat16 *>(b1 + umma_off(n, k >> 3, UMMA_NK1) + (k & 7) * 2) = v;
  }
  for (int x = tid; x < 256; x += nth) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      w[j] = (((uint32_t)x >> (2 * j)) & 1u) * 0x3F80u +
             (((uint32_t)x >> (2 * j + 1)) & 1u) * 0x3F800000u;  // bf16 1.0 = 0x3F80
    bits[x] = make_uint4(w[0], w[1], w[2], w[3]);
  }
  for (int i = tid; i < 64 * 64; i += nth) {
    const int n = i >> 6, k = i & 63;
    *reinterpret_cast<__nv_bfloat16 *>(b2 + umma_off(n, k >> 3, UMMA_NK2) + (k & 7) * 2) =
        P[MLP_W2 + k * MLP_H + n];
  }
  for (int i = tid; i < MLP_H; i += nth) {
    fb[i] = __bfloat162float(P[MLP_B2 + i]);
    fb[64 + i] = __bfloat162float(P[MLP_W3 + i]);
  }
  if (tid == 0) fb[128] = __bfloat162float(P[MLP_B3]);
}

// bf16x2 of ReLU(lo), ReLU(hi), round to nearest even (lower half: lo)
__device__ __forceinline__ uint32_t umma_relu_pack(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// packed fp32 pairs (Blackwell f32x2 arithmetic)
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
  return ((unsigned long long)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// The network in three stages, so that a caller can do other work while an
// MMA runs. Each stage is collective over the warpgroup wg (all 128 threads
// call it together); abuf = the warpgroup's operand rows, tm = its 64
// tensor-memory columns, bar = its mbarrier with phase bit `phase` (toggled
// by each wait). A wait that runs out sets `timeout` (the logit is then
// meaningless); once it is set, this thread's later waits try once, so a
// kernel whose MMAs stopped completing still ends promptly (its control flow,
// and with it every warpgroup barrier, does not depend on the flag).
//
// Stage 1: write this thread's row of the layer-1 operand (env: bit k =
// neighbour k) and issue layer 1.
__device__ __forceinline__ void umma_layer1_issue(const UmmaNet &N, unsigned char *abuf,
                                                  uint32_t tm, uint64_t *bar, int wg,
                                                  unsigned long long env) {
  const int lane = threadIdx.x & 31, wq = (threadIdx.x >> 5) & 3;
  const int row = 32 * wq + lane;
  // the row's 42 inputs and the bias input as bf16 0/1
  const unsigned long long e = env | (1ull << MLP_IN);
#pragma unroll
  for (int c = 0; c < UMMA_NK1; ++c)
    *reinterpret_cast<uint4 *>(abuf + umma_off(row, c, UMMA_NK1)) = N.bits[(e >> (8 * c)) & 255u];
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
}

// Stage 2: wait for layer 1, write the layer-2 operand bf16(ReLU(D)) and
// issue layer 2.
__device__ __forceinline__ void umma_layer2_issue(const UmmaNet &N, unsigned char *abuf,
                                                  uint32_t tm, uint64_t *bar, uint32_t &phase,
                                                  int wg, bool &timeout) {
  const int lane = threadIdx.x & 31, wq = (threadIdx.x >> 5) & 3;
  const int row = 32 * wq + lane;
  const uint32_t tlane = tm + ((uint32_t)(32 * wq) << 16);
  if (!mbar_wait(bar, phase, timeout ? 1 : UMMA_WAIT_ITERS)) timeout = true;
  phase ^= 1u;
  tc_fence_after();
  // 32 columns at a time
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tmem_ld32(tlane + 32 * h, v);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      uint4 u;
      u.x = umma_relu_pack(v[8 * c], v[8 * c + 1]);
      u.y = umma_relu_pack(v[8 * c + 2], v[8 * c + 3]);
      u.z = umma_relu_pack(v[8 * c + 4], v[8 * c + 5]);
      u.w = umma_relu_pack(v[8 * c + 6], v[8 * c + 7]);
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
}

// Stage 3: wait for layer 2 and form this row's logit
// z = b3 + sum_j ReLU(D_j + b2_j) w3_j (two interleaved fp32 chains, even and
// odd hidden units, in f32x2).
__device__ __forceinline__ float umma_logit(const UmmaNet &N, uint32_t tm, uint64_t *bar,
                                            uint32_t &phase, bool &timeout) {
  const int wq = (threadIdx.x >> 5) & 3;
  const uint32_t tlane = tm + ((uint32_t)(32 * wq) << 16);
  if (!mbar_wait(bar, phase, timeout ? 1 : UMMA_WAIT_ITERS)) timeout = true;
  phase ^= 1u;
  tc_fence_after();
  unsigned long long z2 = 0ull;
  const float4 *b2v = reinterpret_cast<const float4 *>(N.bias2);
  const float4 *w3v = reinterpret_cast<const float4 *>(N.w3);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tmem_ld32(tlane + 32 * h, v);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float4 b = b2v[8 * h + i], w = w3v[8 * h + i];
      const unsigned long long t0 = f2_add(f2_pack(v[4 * i], v[4 * i + 1]), f2_pack(b.x, b.y));
      const unsigned long long t1 = f2_add(f2_pack(v[4 * i + 2], v[4 * i + 3]), f2_pack(b.z, b.w));
      const unsigned long long r0 =
          f2_pack(fmaxf(__uint_as_float((uint32_t)t0), 0.f), fmaxf(__uint_as_float((uint32_t)(t0 >> 32)), 0.f));
      const unsigned long long r1 =
          f2_pack(fmaxf(__uint_as_float((uint32_t)t1), 0.f), fmaxf(__uint_as_float((uint32_t)(t1 >> 32)), 0.f));
      z2 = f2_fma(r0, f2_pack(w.x, w.y), z2);
      z2 = f2_fma(r1, f2_pack(w.z, w.w), z2);
    }
  }
  tc_fence_before();  // the next call's MMAs come after these reads
  return N.b3 + (__uint_as_float((uint32_t)z2) + __uint_as_float((uint32_t)(z2 >> 32)));
}

// Logit of the environment `env` of this thread's row: the three stages back
// to back.
__device__ __forceinline__ float umma_network(const UmmaNet &N, unsigned char *abuf, uint32_t tm,
                                              uint64_t *bar, uint32_t &phase, int wg,
                                              unsigned long long env, bool &timeout) {
  umma_layer1_issue(N, abuf, tm, bar, wg, env);
  umma_layer2_issue(N, abuf, tm, bar, phase, wg, timeout);
  return umma_logit(N, tm, bar, phase, timeout);
}

}  // namespace cem
