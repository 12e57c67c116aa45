// Learned-proposal kernels: MLP inference, gradient, Adam update, training
// features, and the Metropolis-Hastings sampler with sum-tree proposals.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "cem_kernels.cuh"
#include "cem_learned.cuh"

namespace cem {

// ---------------------------------------------------------------- inference
__global__ void k_mlp_forward(const __nv_bfloat16 *__restrict__ params,
                              const int8_t *__restrict__ X, long long n, float *__restrict__ z) {
  __shared__ float P[MLP_NPARAM];
  mlp_load(P, params);
  __syncthreads();
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (long long e = (long long)blockIdx.x * nw + warp; e < n; e += (long long)gridDim.x * nw) {
    const int8_t *x = X + e * MLP_IN;
    float h1[2], h2[2];
    const float zz = mlp_forward_warp(P, x, h1, h2);
    if (lane == 0) z[e] = zz;
  }
}

// ---------------------------------------------------------------- gradient
// Mean-squared error L = 1/(2n) sum (z - t)^2 over the batch [b0, b0 + n);
// gradients (fp32) added to grad[MLP_NPARAM]; loss sum added to loss[0].
__global__ void k_mlp_grad(const __nv_bfloat16 *__restrict__ params,
                           const int8_t *__restrict__ X, const float *__restrict__ t,
                           const int *__restrict__ order, long long b0, long long n, float inv_n,
                           float *__restrict__ grad, double *__restrict__ loss) {
  __shared__ float P[MLP_NPARAM];
  __shared__ float G[MLP_NPARAM];
  mlp_load(P, params);
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) G[i] = 0.f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  double lsum = 0.0;
  for (long long q = (long long)blockIdx.x * nw + warp; q < n; q += (long long)gridDim.x * nw) {
    const long long e = order ? order[b0 + q] : b0 + q;
    const int8_t *x = X + e * MLP_IN;
    float h1[2], h2[2];
    const float z = mlp_forward_warp(P, x, h1, h2);
    const float r = z - t[e];
    if (lane == 0) lsum += 0.5 * (double)r * (double)r;
    const float dz = r * inv_n;
    // output layer
    atomicAdd(&G[MLP_W3 + lane], dz * h2[0]);
    atomicAdd(&G[MLP_W3 + lane + 32], dz * h2[1]);
    if (lane == 0) atomicAdd(&G[MLP_B3], dz);
    const float d20 = (h2[0] > 0.f) ? dz * P[MLP_W3 + lane] : 0.f;
    const float d21 = (h2[1] > 0.f) ? dz * P[MLP_W3 + lane + 32] : 0.f;
    atomicAdd(&G[MLP_B2 + lane], d20);
    atomicAdd(&G[MLP_B2 + lane + 32], d21);
    // second layer weights W2[i][j] (input i, output j): dW2 = h1_i * d2_j
    // and first-layer deltas d1_i = [h1_i > 0] sum_j W2[i][j] d2_j
    float d1_0 = 0.f, d1_1 = 0.f;
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
      const float u = __shfl_sync(0xffffffffu, h1[0], i);
      const float v = __shfl_sync(0xffffffffu, h1[1], i);
      atomicAdd(&G[MLP_W2 + i * MLP_H + lane], u * d20);
      atomicAdd(&G[MLP_W2 + i * MLP_H + lane + 32], u * d21);
      atomicAdd(&G[MLP_W2 + (i + 32) * MLP_H + lane], v * d20);
      atomicAdd(&G[MLP_W2 + (i + 32) * MLP_H + lane + 32], v * d21);
    }
    // d1 for this lane's inputs i = lane, lane + 32: sum over outputs j
#pragma unroll 4
    for (int j = 0; j < 32; ++j) {
      const float a = __shfl_sync(0xffffffffu, d20, j);
      const float b = __shfl_sync(0xffffffffu, d21, j);
      d1_0 = fmaf(P[MLP_W2 + lane * MLP_H + j], a, d1_0);
      d1_0 = fmaf(P[MLP_W2 + lane * MLP_H + j + 32], b, d1_0);
      d1_1 = fmaf(P[MLP_W2 + (lane + 32) * MLP_H + j], a, d1_1);
      d1_1 = fmaf(P[MLP_W2 + (lane + 32) * MLP_H + j + 32], b, d1_1);
    }
    d1_0 = (h1[0] > 0.f) ? d1_0 : 0.f;
    d1_1 = (h1[1] > 0.f) ? d1_1 : 0.f;
    atomicAdd(&G[MLP_B1 + lane], d1_0);
    atomicAdd(&G[MLP_B1 + lane + 32], d1_1);
    for (int k = 0; k < MLP_IN; ++k) {
      if (x[k]) {
        atomicAdd(&G[MLP_W1 + k * MLP_H + lane], d1_0);
        atomicAdd(&G[MLP_W1 + k * MLP_H + lane + 32], d1_1);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x)
    if (G[i] != 0.f) atomicAdd(&grad[i], G[i]);
  if (lane == 0 && lsum != 0.0) atomicAdd(loss, lsum);
}

// ---------------------------------------------------------------- Adam
// Kingma & Ba, "Adam: A Method for Stochastic Optimization" (ICLR 2015).
__global__ void k_mlp_adam(float *__restrict__ master, __nv_bfloat16 *__restrict__ params,
                           float *__restrict__ grad, float *__restrict__ m, float *__restrict__ v,
                           float lr, float beta1, float beta2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MLP_NPARAM) return;
  const float g = grad[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * g;
  const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  const float w = master[i] - lr * mh / (sqrtf(vh) + eps);
  master[i] = w;
  params[i] = __float2bfloat16_rn(w);
  grad[i] = 0.f;
}

__global__ void k_mlp_pack(const float *__restrict__ master, __nv_bfloat16 *__restrict__ params) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < MLP_NPARAM) params[i] = __float2bfloat16_rn(master[i]);
}

// ---------------------------------------------------------------- features
// Environment of every site of one binary FCC replica (42 neighbours in the
// generated order) and the training target: half the log Metropolis weight
// of putting B on the site in that environment,
// t = clamp(-beta * dE_AB / 2, LOGIT_MIN, LOGIT_MAX) (for a site holding A
// that is half the log weight of flipping it; for a site holding B its
// flip's is -t).
__global__ void k_features(const int8_t *__restrict__ occ, int L, const double *__restrict__ w,
                           const int *__restrict__ orb_func, double beta,
                           int8_t *__restrict__ X, float *__restrict__ t) {
  const int n = L * L * L;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x) {
    const int x = l % L, y = (l / L) % L, z = l / (L * L);
    int v[gen_fcc::N_NB];
#pragma unroll
    for (int k = 0; k < gen_fcc::N_NB; ++k) {
      int xx = x + gen_fcc::NB_D[k][0], yy = y + gen_fcc::NB_D[k][1], zz = z + gen_fcc::NB_D[k][2];
      xx += (xx < 0) ? L : 0;
      xx -= (xx >= L) ? L : 0;
      yy += (yy < 0) ? L : 0;
      yy -= (yy >= L) ? L : 0;
      zz += (zz < 0) ? L : 0;
      zz -= (zz >= L) ? L : 0;
      v[k] = occ[xx + L * (yy + L * zz)];
      X[(long long)l * MLP_IN + k] = (int8_t)v[k];
    }
    int cnt[gen_fcc::N_ORBITS];
    for (int g = 0; g < gen_fcc::N_ORBITS; ++g) cnt[g] = 0;
    for (int c = 0; c < gen_fcc::N_CL; ++c) {
      int p = 1;
      for (int q = 0; q < 3; ++q) {
        const int k = gen_fcc::CL_P_D[c][q];
        if (k >= 0) p &= v[k];
      }
      cnt[gen_fcc::CL_ORBIT_D[c]] += p;
    }
    double de = 0.0;
    for (int g = 0; g < gen_fcc::N_ORBITS; ++g) de += w[orb_func[g]] * cnt[g];
    float tt = (float)(-0.5 * beta * de);
    t[l] = fminf(fmaxf(tt, LOGIT_MIN), LOGIT_MAX);
  }
}

// ---------------------------------------------------------------- sum trees
// Per replica and species: levels of int64 sums, 32 children per node; level
// 0 holds one leaf per site. `lvl_off[k]` is the offset of level k in the
// tree's storage, `lvl_n[k]` its padded size (multiple of 32 except the root).
struct TreeGeo {
  int n_levels;
  int lvl_off[8];
  int lvl_n[8];
  int size;  // elements per tree
};

__device__ __forceinline__ void tree_add(unsigned long long *tree, const TreeGeo &g, int leaf,
                                         long long delta) {
  int idx = leaf;
  for (int k = 0; k < g.n_levels; ++k) {
    atomicAdd(&tree[g.lvl_off[k] + idx], (unsigned long long)delta);
    idx >>= 5;
  }
}

// Warp-cooperative descent: the leaf whose cumulative interval holds r.
__device__ __forceinline__ int tree_find(const unsigned long long *tree, const TreeGeo &g,
                                         long long r) {
  const int lane = threadIdx.x & 31;
  int node = 0;
  for (int k = g.n_levels - 2; k >= 0; --k) {
    const int child = node * 32 + lane;
    long long v = (long long)tree[g.lvl_off[k] + child];
    long long s = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const long long o = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += o;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, s > r);
    const int sel = hit ? __ffs(hit) - 1 : 31;
    const long long before = __shfl_sync(0xffffffffu, s - v, sel);
    r -= before;
    node = node * 32 + sel;
  }
  return node;
}

// One uniform integer in [0, w) from the counter-based stream (Lemire's
// method with rejection, exact for any w < 2^63).
__device__ __forceinline__ long long uniform_below(long long w, uint32_t k0, uint32_t k1,
                                                   uint32_t c0, uint32_t c1, uint32_t c2,
                                                   uint32_t tag) {
  const unsigned long long range = (unsigned long long)w;
  const unsigned long long threshold = (0ull - range) % range;
  for (uint32_t it = 0;; ++it) {
    const U4 r = philox4x32_10(U4{c0, c1, c2, tag | (it << 8)}, k0, k1);
    const unsigned long long x = ((unsigned long long)r.x << 32) | r.y;
    const unsigned long long lo = x * range;
    if (lo >= threshold || it == 255) return (long long)__umul64hi(x, range);
  }
}

// Build leaves (weights from the network or 1 for the uniform proposal) and
// all tree levels for every replica; one CTA per replica.
__global__ void k_learned_init(const __nv_bfloat16 *__restrict__ params, int use_mlp,
                               const Replica *__restrict__ reps, const int8_t *__restrict__ occ_all,
                               long long *__restrict__ weights, unsigned long long *__restrict__ trees,
                               long long tree_stride, TreeGeo tg, long long w_stride) {
  constexpr int INIT_THREADS = 512;
  __shared__ float P[MLP_NPARAM];
  __shared__ int8_t env[INIT_THREADS / 32][MLP_IN + 5];  // one row per warp
  const Replica &R = reps[blockIdx.x];
  const int L = R.L[0];
  const int n = L * L * L;
  const int8_t *occ = occ_all + R.occ_offset;
  long long *wts = weights + blockIdx.x * w_stride;
  unsigned long long *tA = trees + blockIdx.x * 2 * tree_stride;
  unsigned long long *tB = tA + tree_stride;
  if (use_mlp) mlp_load(P, params);
  for (int i = threadIdx.x; i < tg.size; i += blockDim.x) tA[i] = tB[i] = 0ull;
  __syncthreads();
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int l = warp; l < n; l += nw) {
    const int x = l % L, y = (l / L) % L, z = l / (L * L);
    for (int k = lane; k < MLP_IN; k += 32) {
      int xx = (x + gen_fcc::NB_D[k][0] + L) % L, yy = (y + gen_fcc::NB_D[k][1] + L) % L,
          zz = (z + gen_fcc::NB_D[k][2] + L) % L;
      env[warp][k] = occ[xx + L * (yy + L * zz)];
    }
    __syncwarp();
    long long w = 1;
    if (use_mlp) {
      float h1[2], h2[2];
      const float zz = mlp_forward_warp(P, env[warp], h1, h2);
      w = logit_weight(occ[l] ? -zz : zz);
    }
    if (lane == 0) {
      wts[l] = w;
      (occ[l] == 0 ? tA : tB)[l] = (unsigned long long)w;
    }
    __syncwarp();
  }
  __syncthreads();
  for (int k = 1; k < tg.n_levels; ++k) {
    for (int i = threadIdx.x; i < tg.lvl_n[k]; i += blockDim.x) {
      unsigned long long a = 0, b = 0;
      for (int c = 0; c < 32; ++c) {
        const int ch = i * 32 + c;
        if (ch < tg.lvl_n[k - 1]) {
          a += tA[tg.lvl_off[k - 1] + ch];
          b += tB[tg.lvl_off[k - 1] + ch];
        }
      }
      tA[tg.lvl_off[k] + i] = a;
      tB[tg.lvl_off[k] + i] = b;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- sampler
struct LearnedParams {
  const Replica *reps;
  ReplicaStats *stats;
  int8_t *occ;
  const __nv_bfloat16 *params;
  int use_mlp;
  long long *weights;
  long long w_stride;
  unsigned long long *trees;
  long long tree_stride;
  TreeGeo tg;
  long long n_passes, n_equil;
  double *samples;  // [rep][capacity][3]: potential, x, order parameter
  long long sample_capacity;
  int max_affected;
};

constexpr int LEARNED_THREADS = 256;
constexpr int MAX_AFF = 2 * (gen_fcc::N_NB + 1);

// L1_2 sublattice (one of the four simple-cubic sublattices of FCC) of a
// site in primitive-cell coordinates.
__device__ __forceinline__ int fcc_sc_sublattice(int x, int y, int z) {
  return ((y + z) & 1) | (((x + z) & 1) << 1);
}

template <int PITCH>
__global__ void __launch_bounds__(LEARNED_THREADS, 1)
    k_learned(const __grid_constant__ CeTables T, const __grid_constant__ LearnedParams LP) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int rep = blockIdx.x;
  const Replica &R = LP.reps[rep];
  ReplicaStats &S = LP.stats[rep];
  const int L = R.L[0];
  const int n = L * L * L;
  constexpr int RH = 2;
  Geo G;
  G.L0 = G.L1 = G.L2 = L;
  G.R = RH;
  G.W = G.H = PITCH;
  G.V = PITCH * PITCH * (L + 2 * RH);
  int8_t *occ = reinterpret_cast<int8_t *>(smem);
  float *P = reinterpret_cast<float *>(smem + align16(G.V));
  int *aff_l = reinterpret_cast<int *>(P + ((MLP_NPARAM + 3) & ~3));
  long long *aff_wold = reinterpret_cast<long long *>(aff_l + MAX_AFF + 2);
  long long *aff_wnew = aff_wold + MAX_AFF;
  int8_t *env = reinterpret_cast<int8_t *>(aff_wnew + MAX_AFF);  // [8][48]
  __shared__ int s_nboff[gen_fcc::N_NB];
  __shared__ int s_nbd[gen_fcc::N_NB][3];
  __shared__ int s_sites[2];
  __shared__ unsigned char s_dup[MAX_AFF];
  __shared__ int s_accept;
  __shared__ double s_energy;
  __shared__ double s_de;
  __shared__ long long s_WA, s_WB;
  __shared__ long long s_sub[4];
  __shared__ long long s_n1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  if (LP.use_mlp) mlp_load(P, LP.params);
  for (int k = tid; k < gen_fcc::N_NB; k += blockDim.x) {
    s_nboff[k] = gen_fcc::NB_D[k][0] + PITCH * (gen_fcc::NB_D[k][1] + PITCH * gen_fcc::NB_D[k][2]);
    for (int a = 0; a < 3; ++a) s_nbd[k][a] = gen_fcc::NB_D[k][a];
  }
  const int8_t *gocc = LP.occ + R.occ_offset;
  for (int l = tid; l < n; l += blockDim.x) {
    const int x = l % L, y = (l / L) % L, z = l / (L * L);
    occ[G.addr(0, x, y, z)] = gocc[l];
  }
  __syncthreads();
  for (int h = tid; h < G.V; h += blockDim.x) {
    int r = h;
    const int xh = r % G.W;
    r /= G.W;
    const int yh = r % G.H, zh = r / G.H;
    const int x = xh - RH, y = yh - RH, z = zh - RH;
    if (x >= 0 && x < L && y >= 0 && y < L && z >= 0 && z < L) continue;
    if (x >= L + RH || y >= L + RH) continue;
    occ[h] = occ[G.addr(0, wrapc(x, L), wrapc(y, L), wrapc(z, L))];
  }
  if (tid == 0) {
    for (int k = 0; k < 4; ++k) s_sub[k] = 0;
    s_n1 = 0;
  }
  __syncthreads();
  // exact initial energy (flower counts / orbit size) and sublattice counts
  {
    long long cnt[gen_fcc::N_ORBITS] = {0, 0, 0, 0, 0, 0};
    long long sub[4] = {0, 0, 0, 0}, n1 = 0;
    for (int l = tid; l < n; l += blockDim.x) {
      const int x = l % L, y = (l / L) % L, z = l / (L * L);
      const int ad = G.addr(0, x, y, z);
      if (!occ[ad]) continue;
      int nn[gen_fcc::N_ORBITS];
      gen_fcc::counts<PITCH>(occ + ad, nn);
      for (int g = 0; g < gen_fcc::N_ORBITS; ++g) cnt[g] += nn[g];
      sub[fcc_sc_sublattice(x, y, z)]++;
      ++n1;
    }
    __shared__ long long red[gen_fcc::N_ORBITS];
    if (tid < gen_fcc::N_ORBITS) red[tid] = 0;
    __syncthreads();
    for (int g = 0; g < gen_fcc::N_ORBITS; ++g) atomicAdd((unsigned long long *)&red[g], (unsigned long long)cnt[g]);
    for (int k = 0; k < 4; ++k) atomicAdd((unsigned long long *)&s_sub[k], (unsigned long long)sub[k]);
    atomicAdd((unsigned long long *)&s_n1, (unsigned long long)n1);
    __syncthreads();
    if (tid == 0) {
      double e = T.w[0] * n;
      for (int g = 0; g < T.n_orbits; ++g) e += T.w[T.orb_func_base[g]] * (double)(red[g] / T.orb_size[g]);
      s_energy = e;
      const long long pass = S.pass, np = S.n_proposed, na = S.n_accepted;
      unsigned char *raw = reinterpret_cast<unsigned char *>(&S);
      for (int q = 0; q < (int)sizeof(ReplicaStats); ++q) raw[q] = 0;
      S.pass = pass;
      S.n_proposed = np;
      S.n_accepted = na;
      S.n_species[0] = n - s_n1;
      S.n_species[1] = s_n1;
    }
    __syncthreads();
  }
  unsigned long long *tA = LP.trees + (long long)rep * 2 * LP.tree_stride;
  unsigned long long *tB = tA + LP.tree_stride;
  long long *wts = LP.weights + (long long)rep * LP.w_stride;
  const int root = LP.tg.lvl_off[LP.tg.n_levels - 1];
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const double beta = R.beta;
  long long pass_global = S.pass;
  long long step = 0;
  long long n_acc_local = 0, n_prop_local = 0;
  for (long long ip = 0; ip < LP.n_passes; ++ip, ++pass_global) {
    for (int st = 0; st < n; ++st, ++step) {
      const uint32_t c0 = (uint32_t)st, c1 = (uint32_t)pass_global, c2 = (uint32_t)(pass_global >> 32);
      // ---- draw one site of each species (warps 0 and 1)
      if (warp < 2) {
        const unsigned long long *tr = warp == 0 ? tA : tB;
        const long long W = (long long)tr[root];
        long long r = 0;
        if (lane == 0) r = uniform_below(W, k0, k1, c0, c1, c2, 0x10u + warp);
        r = __shfl_sync(0xffffffffu, r, 0);
        const int s = tree_find(tr, LP.tg, r);
        if (lane == 0) {
          s_sites[warp] = s;
          if (warp == 0) s_WA = W;
          else s_WB = W;
        }
      }
      __syncthreads();
      const int a = s_sites[0], b = s_sites[1];
      const int xa = a % L, ya = (a / L) % L, za = a / (L * L);
      const int xb = b % L, yb = (b / L) % L, zb = b / (L * L);
      const int ada = G.addr(0, xa, ya, za), adb = G.addr(0, xb, yb, zb);
      // ---- exact dE (thread 0, sequential: a first, then b with a changed)
      //      while warps 1.. list the affected sites (a, b and their neighbours)
      if (tid == 0) {
        int na[gen_fcc::N_ORBITS], nb[gen_fcc::N_ORBITS];
        gen_fcc::counts<PITCH>(occ + ada, na);
        put_site(occ, G, 0, xa, ya, za, 1);
        gen_fcc::counts<PITCH>(occ + adb, nb);
        double de = 0.0;
        for (int g = 0; g < T.n_orbits; ++g)
          de += T.w[T.orb_func_base[g]] * (double)(na[g] - nb[g]);  // a: 0 -> 1, b: 1 -> 0
        put_site(occ, G, 0, xb, yb, zb, 0);  // proposed state fully applied
        s_de = de;
      }
      if (tid >= 32 && tid < 32 + MAX_AFF) {
        const int j = tid - 32;
        const int q = j / (gen_fcc::N_NB + 1), k = j % (gen_fcc::N_NB + 1) - 1;
        const int s0 = q == 0 ? a : b;
        int site = s0;
        if (k >= 0) {
          const int x = s0 % L, y = (s0 / L) % L, z = s0 / (L * L);
          site = wrapc(x + s_nbd[k][0], L) + L * (wrapc(y + s_nbd[k][1], L) + L * wrapc(z + s_nbd[k][2], L));
        }
        aff_l[j] = site;
      }
      __syncthreads();
      if (tid >= 32 && tid < 32 + MAX_AFF) {  // first occurrence of each site counts
        const int j = tid - 32, site = aff_l[j];
        bool dup = false;
        for (int i2 = 0; i2 < j; ++i2) dup = dup || (aff_l[i2] == site);
        s_dup[j] = dup ? 1 : 0;
      }
      __syncthreads();
      // ---- new weights of the affected sites in the proposed state
      for (int j = warp; j < MAX_AFF; j += nw) {
        if (s_dup[j]) continue;  // uniform across the warp
        const int s = aff_l[j];
        const int x = s % L, y = (s / L) % L, z = s / (L * L);
        const int ad = G.addr(0, x, y, z);
        int8_t *e = env + warp * 48;
        for (int k = lane; k < MLP_IN; k += 32) e[k] = occ[ad + s_nboff[k]];
        __syncwarp();
        long long w = 1;
        if (LP.use_mlp) {
          float h1[2], h2[2];
          const float zz = mlp_forward_warp(P, e, h1, h2);
          w = logit_weight(occ[ad] ? -zz : zz);  // the proposed state is applied
        }
        if (lane == 0) {
          aff_wnew[j] = w;
          aff_wold[j] = wts[s];
        }
        __syncwarp();
      }
      __syncthreads();
      // ---- Metropolis-Hastings with the exact proposal probabilities (warp 0)
      if (warp == 0) {
        long long dA = 0, dB = 0, wa = 0, wb = 0, wa2 = 0, wb2 = 0;
        for (int j = lane; j < MAX_AFF; j += 32) {
          if (s_dup[j]) continue;
          const int s = aff_l[j];
          const long long wo = aff_wold[j], wn = aff_wnew[j];
          if (s == a) {
            wa = wo;
            wa2 = wn;
            dA -= wo;
            dB += wn;
          } else if (s == b) {
            wb = wo;
            wb2 = wn;
            dB -= wo;
            dA += wn;
          } else {
            const int o = occ[G.addr(0, s % L, (s / L) % L, s / (L * L))];
            if (o == 0) dA += wn - wo;
            else dB += wn - wo;
          }
        }
        for (int off = 16; off; off >>= 1) {
          dA += __shfl_xor_sync(0xffffffffu, dA, off);
          dB += __shfl_xor_sync(0xffffffffu, dB, off);
          wa += __shfl_xor_sync(0xffffffffu, wa, off);
          wb += __shfl_xor_sync(0xffffffffu, wb, off);
          wa2 += __shfl_xor_sync(0xffffffffu, wa2, off);
          wb2 += __shfl_xor_sync(0xffffffffu, wb2, off);
        }
        if (lane == 0) {
          const double dE = s_de;
          const long long WA2 = s_WA + dA, WB2 = s_WB + dB;
          const double log_q = log((double)wb2) - log((double)WA2) + log((double)wa2) -
                               log((double)WB2) - log((double)wa) + log((double)s_WA) -
                               log((double)wb) + log((double)s_WB);
          const double lr = -beta * dE + log_q;
          const U4 u = philox4x32_10(U4{c0, c1, c2, 0x20u}, k0, k1);
          const double ud =
              ((double)(((unsigned long long)u.x << 21) ^ u.y) + 0.5) * 1.1102230246251565e-16;
          const int acc = (lr >= 0.0) || (log(ud) < lr);
          s_accept = acc;
          ++n_prop_local;
          if (acc) {
            ++n_acc_local;
            s_energy += dE;
            s_sub[fcc_sc_sublattice(xa, ya, za)] += 1;
            s_sub[fcc_sc_sublattice(xb, yb, zb)] -= 1;
          } else {
            put_site(occ, G, 0, xa, ya, za, 0);
            put_site(occ, G, 0, xb, yb, zb, 1);
          }
        }
      }
      __syncthreads();
      if (s_accept) {
        for (int j = tid; j < MAX_AFF; j += blockDim.x) {
          if (s_dup[j]) continue;
          const int s = aff_l[j];
          const long long wo = aff_wold[j], wn = aff_wnew[j];
          wts[s] = wn;
          if (s == a) {
            tree_add(tA, LP.tg, s, -wo);
            tree_add(tB, LP.tg, s, wn);
          } else if (s == b) {
            tree_add(tB, LP.tg, s, -wo);
            tree_add(tA, LP.tg, s, wn);
          } else if (wn != wo) {
            const int o = occ[G.addr(0, s % L, (s / L) % L, s / (L * L))];
            tree_add(o == 0 ? tA : tB, LP.tg, s, wn - wo);
          }
        }
      }
      __syncthreads();
    }
    // ---- sample once per pass
    if (tid == 0) {
      const double x = (double)S.n_species[1] / n;
      const double ef = s_energy / n;
      double op = 0.0;
      for (int k = 0; k < 4; ++k) {
        const double c = (double)s_sub[k] / (n / 4) - x;
        op += c * c;
      }
      op = sqrt(op);
      if (ip >= LP.n_equil) {
        S.n_samples += 1.0;
        S.sum_e += ef;
        S.sum_e2 += ef * ef;
        S.sum_f += ef;
        S.sum_x[0] += x;
        S.sum_xx[0] += x * x;
        S.sum_ex[0] += ef * x;
        if (LP.samples) {
          const long long si = (long long)S.n_samples - 1;
          if (si < LP.sample_capacity) {
            double *out = LP.samples + ((long long)rep * LP.sample_capacity + si) * 3;
            out[0] = ef;
            out[1] = x;
            out[2] = op;
          }
        }
      }
    }
    __syncthreads();
  }
  for (int l = tid; l < n; l += blockDim.x) {
    const int x = l % L, y = (l / L) % L, z = l / (L * L);
    LP.occ[R.occ_offset + l] = occ[G.addr(0, x, y, z)];
  }
  if (tid == 0) {
    S.energy = s_energy;
    S.pass = pass_global;
    S.n_proposed += n_prop_local;
    S.n_accepted += n_acc_local;
  }
}

// ---------------------------------------------------------------- launchers
cudaError_t mlp_forward(const __nv_bfloat16 *params, const int8_t *X, long long n, float *z,
                        cudaStream_t st) {
  long long grid = (n + 7) / 8;
  if (grid > 65535) grid = 65535;
  if (grid < 1) grid = 1;
  k_mlp_forward<<<(int)grid, 256, 0, st>>>(params, X, n, z);
  return cudaGetLastError();
}

cudaError_t mlp_grad(const __nv_bfloat16 *params, const int8_t *X, const float *t,
                     const int *order, long long b0, long long n, float *grad, double *loss,
                     cudaStream_t st) {
  long long grid = (n + 7) / 8;
  if (grid > 1024) grid = 1024;
  if (grid < 1) grid = 1;
  k_mlp_grad<<<(int)grid, 256, 0, st>>>(params, X, t, order, b0, n, 1.0f / (float)n, grad, loss);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float *master, __nv_bfloat16 *params, float *grad, float *m, float *v,
                     float lr, int step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(master, params, grad, m, v, lr, b1, b2,
                                                        eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t mlp_pack(const float *master, __nv_bfloat16 *params, cudaStream_t st) {
  k_mlp_pack<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(master, params);
  return cudaGetLastError();
}

cudaError_t learned_features(const int8_t *occ, int L, const double *w, const int *orb_func,
                             double beta, int8_t *X, float *t, cudaStream_t st) {
  const int n = L * L * L;
  k_features<<<(n + 255) / 256, 256, 0, st>>>(occ, L, w, orb_func, beta, X, t);
  return cudaGetLastError();
}

TreeGeo make_tree_geo(int n_sites) {
  TreeGeo g{};
  int n = (n_sites + 31) & ~31;
  int off = 0, k = 0;
  while (true) {
    g.lvl_off[k] = off;
    g.lvl_n[k] = n;
    off += n;
    ++k;
    if (n == 1) break;
    n = (n + 31) / 32;
    if (n > 1) n = (n + 31) & ~31;
  }
  g.n_levels = k;
  g.size = off;
  return g;
}

int learned_tree_size(int n_sites) { return make_tree_geo(n_sites).size; }

int learned_smem_bytes(int L, int pitch) {
  const int V = pitch * pitch * (L + 4);
  return align16(V) + ((MLP_NPARAM + 3) & ~3) * 4 + (MAX_AFF + 2) * 4 + 2 * MAX_AFF * 8 +
         (LEARNED_THREADS / 32) * 48 + 64;
}

cudaError_t learned_run(const CeTables &T, const Replica *reps, ReplicaStats *stats,
                        int8_t *occ, const __nv_bfloat16 *params, int use_mlp, long long *weights,
                        long long w_stride, unsigned long long *trees, long long tree_stride,
                        int n_sites, int n_replicas, int L, long long n_passes, long long n_equil,
                        double *samples, long long capacity, int pitch, cudaStream_t st) {
  TreeGeo tg = make_tree_geo(n_sites);
  k_learned_init<<<n_replicas, 512, 0, st>>>(params, use_mlp, reps, occ, weights, trees,
                                             tree_stride, tg, w_stride);  // 512 = INIT_THREADS
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  LearnedParams LP{};
  LP.reps = reps;
  LP.stats = stats;
  LP.occ = occ;
  LP.params = params;
  LP.use_mlp = use_mlp;
  LP.weights = weights;
  LP.w_stride = w_stride;
  LP.trees = trees;
  LP.tree_stride = tree_stride;
  LP.tg = tg;
  LP.n_passes = n_passes;
  LP.n_equil = n_equil;
  LP.samples = samples;
  LP.sample_capacity = capacity;
  const int smem = learned_smem_bytes(L, pitch);
  switch (pitch) {
#define CEM_LEARNED_CASE(PP)                                                                  \
  case PP:                                                                                    \
    e = cudaFuncSetAttribute(k_learned<PP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e != cudaSuccess) return e;                                                           \
    k_learned<PP><<<n_replicas, LEARNED_THREADS, smem, st>>>(T, LP);                          \
    break;
    CEM_LEARNED_CASE(14)
    CEM_LEARNED_CASE(28)
    CEM_LEARNED_CASE(36)
    CEM_LEARNED_CASE(52)
#undef CEM_LEARNED_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace cem
