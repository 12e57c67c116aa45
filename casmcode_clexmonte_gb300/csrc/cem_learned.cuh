// Learned proposal for canonical swaps: a small MLP scores each site's
// environment (its 42 neighbours in the first three shells), and swaps are
// proposed by drawing one site of each species with probability proportional
// to its weight. The Metropolis-Hastings ratio uses the exact forward and
// reverse proposal probabilities, so the canonical distribution is sampled
// whatever the network predicts.
//
// Network: 42 inputs (neighbour occupants 0/1) -> 64 (ReLU) -> 64 (ReLU) ->
// 1 logit z(env), trained toward -beta dE_AB(env) / 2, where dE_AB is the
// energy change of putting species B on the site in that environment. A site
// holding A gets weight exp(z) and a site holding B weight exp(-z) (the
// locally balanced weights sqrt(pi(flipped) / pi(current)) when the network
// is exact), so one evaluation serves both species. Parameters are stored in
// bf16 for inference; training keeps fp32 master copies; every dot product
// accumulates in fp32. Integer site weight: w = max(1, round(2^12 exp(+-z)))
// with z clamped to [-10, 10], so sums are exact integers and a drawn site
// has probability exactly w / W.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "cem_common.cuh"

namespace cem {

constexpr int MLP_IN = 42;
constexpr int MLP_H = 64;
// parameter block (fp32 masters / bf16 copies), offsets in elements
constexpr int MLP_W1 = 0;                        // [MLP_IN][MLP_H]  (input-major)
constexpr int MLP_B1 = MLP_W1 + MLP_IN * MLP_H;  // [MLP_H]
constexpr int MLP_W2 = MLP_B1 + MLP_H;           // [MLP_H in][MLP_H out]
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;   // [MLP_H]
constexpr int MLP_W3 = MLP_B2 + MLP_H;           // [MLP_H]
constexpr int MLP_B3 = MLP_W3 + MLP_H;           // [1]
constexpr int MLP_NPARAM = MLP_B3 + 1;

constexpr float LOGIT_MIN = -10.f, LOGIT_MAX = 10.f;
constexpr float WEIGHT_SCALE = 4096.f;

// Integer proposal weight of a logit (of a site holding A; a site holding B
// uses -z).
__host__ __device__ inline long long logit_weight(float z) {
  z = fminf(fmaxf(z, LOGIT_MIN), LOGIT_MAX);
#ifdef __CUDA_ARCH__
  const float w = WEIGHT_SCALE * __expf(z);
#else
  const float w = WEIGHT_SCALE * expf(z);
#endif
  const long long r = (long long)(w + 0.5f);
  return r < 1 ? 1 : r;
}

// Forward pass of one environment by one warp. x: 42 occupants (0/1) in
// shared memory; P: fp32 parameters in shared memory (converted from bf16).
// Returns the logit on every lane; h1, h2 receive this lane's hidden units
// (j and j + 32).
__device__ __forceinline__ float mlp_forward_warp(const float *__restrict__ P,
                                                  const int8_t *__restrict__ x, float h1[2],
                                                  float h2[2]) {
  const int lane = threadIdx.x & 31;
  float a0 = P[MLP_B1 + lane], a1 = P[MLP_B1 + lane + 32];
#pragma unroll 4
  for (int k = 0; k < MLP_IN; ++k) {
    if (x[k]) {
      a0 += P[MLP_W1 + k * MLP_H + lane];
      a1 += P[MLP_W1 + k * MLP_H + lane + 32];
    }
  }
  h1[0] = fmaxf(a0, 0.f);
  h1[1] = fmaxf(a1, 0.f);
  float c0 = P[MLP_B2 + lane], c1 = P[MLP_B2 + lane + 32];
#pragma unroll 8
  for (int i = 0; i < 32; ++i) {
    const float u = __shfl_sync(0xffffffffu, h1[0], i);
    const float v = __shfl_sync(0xffffffffu, h1[1], i);
    c0 = fmaf(P[MLP_W2 + i * MLP_H + lane], u, c0);
    c1 = fmaf(P[MLP_W2 + i * MLP_H + lane + 32], u, c1);
    c0 = fmaf(P[MLP_W2 + (i + 32) * MLP_H + lane], v, c0);
    c1 = fmaf(P[MLP_W2 + (i + 32) * MLP_H + lane + 32], v, c1);
  }
  h2[0] = fmaxf(c0, 0.f);
  h2[1] = fmaxf(c1, 0.f);
  float z = fmaf(P[MLP_W3 + lane], h2[0], P[MLP_W3 + lane + 32] * h2[1]);
#pragma unroll
  for (int off = 16; off; off >>= 1) z += __shfl_xor_sync(0xffffffffu, z, off);
  return z + P[MLP_B3];
}

// bf16 parameters -> fp32 in shared memory
__device__ __forceinline__ void mlp_load(float *__restrict__ P, const __nv_bfloat16 *__restrict__ g) {
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) P[i] = __bfloat162float(g[i]);
}

}  // namespace cem
