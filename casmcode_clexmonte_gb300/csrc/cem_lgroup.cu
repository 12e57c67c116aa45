// Learned group sweep: the canonical Metropolis-Hastings sampler of binary
// FCC cluster expansions (generated topology) in which the proposal network
// chooses which swaps to propose inside random groups of non-interacting
// sites.
//
// A pass visits the colour classes of period 3 (sites whose cell coordinates
// agree modulo 3; no two of them share a cluster, since every flower offset
// has a component in {-2..2} \ {0}) in a random order. A class sub-step
//   1. evaluates, for every member, the exact energy change dE_AB of putting
//      B on the site (integer cluster counts, split ECI weights) and the
//      network logit z of its 42-neighbour environment; neither depends on
//      other members of the class, so both stay valid for the whole sub-step;
//   2. splits the class into groups of 32 members by a random affine
//      permutation of the member index (state independent, drawn per
//      sub-step), one group per warp;
//   3. runs `rounds` Metropolis-Hastings swaps inside each group: an A member
//      drawn with probability w_A / W_A, a B member with w_B / W_B (integer
//      weights of z, exact integer totals), accepted with
//      min(1, exp(-beta dE) q_rev / q_fwd) with the exact reverse
//      probabilities (the swapped members change their own weights only).
// Members of one group do not interact, so dE of a swap is the sum of the
// two members' flip energies. Classes of period 3 mix the four simple-cubic
// sublattices of the L1_2 order, so group swaps create and remove antisite
// pairs. `n_local` sub-steps of nearest-neighbour swaps per pass (plain
// Metropolis, pairs at anchors 6 cells apart) move atoms between classes, so
// the chain is ergodic in the canonical ensemble.
//
// Weights: mode 0 every weight 1 (uniform swaps inside groups), mode 1 the
// network (w_A = round(2^12 exp(z)), w_B = round(2^12 exp(-z)), z clamped),
// mode 2 the exact locally balanced weights z = -beta dE_AB / 2 that the
// network is trained to predict.
//
// One replica runs on a thread-block cluster of 1, 2 or 4 CTAs (one per SM):
// every CTA holds a full copy of the replica in its shared memory, takes a
// share of the groups (and of the nearest-neighbour anchors) of each
// sub-step, and writes every accepted change into all copies through
// distributed shared memory; a cluster barrier ends each sub-step. A group's
// draws depend only on (pass, sub-step, group, round), so the chain is the
// same for every cluster size.
//
// Network evaluation on the 5th-generation tensor cores (cem_umma.cuh): the
// four warps of a warpgroup evaluate their 4 groups (128 sites) together,
// one tcgen05.mma issuer per warpgroup, bf16 operands in shared memory, fp32
// accumulators in tensor memory (64 columns per warpgroup), one site per
// thread in the epilogue.
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "cem_kernels.cuh"
#include "cem_learned.cuh"
#include "cem_umma.cuh"

namespace cem {

constexpr int LG_THREADS = 512;
constexpr int LG_NW = LG_THREADS / 32;
constexpr int LG_CLASSES = 27;
constexpr uint32_t TAG_LG_SCHED = 0x5u, TAG_LG_GROUP = 0x6u, TAG_LG_LOCAL = 0x7u;
// network tables of the tcgen05 path: W1^T, W2^T, one operand buffer per
// warpgroup, biases (193 floats), per-warpgroup mbarriers, tensor-memory slot
constexpr int LG_NET_BYTES =
    UMMA_B1_BYTES + UMMA_B2_BYTES + 4 * UMMA_A_BYTES + UMMA_BITS_BYTES + 1024;

struct LGroupParams {
  const Replica *reps;
  ReplicaStats *stats;
  int8_t *occ;
  const __nv_bfloat16 *params;
  int mode;  // 0 uniform, 1 network, 2 exact local energies
  int rounds, n_local;
  long long n_passes, n_equil;
  double *samples;  // [rep][capacity][3]: energy per unit cell, x_B, order parameter
  long long sample_capacity;
  const volatile int *stop;  // host-mapped stop flag (null: none)
  int cluster;               // CTAs per replica (thread-block cluster size)
};

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return ((unsigned long long)hi << 32) | lo;
}

// a^-1 mod n for gcd(a, n) = 1 (extended Euclid)
__device__ __forceinline__ uint32_t lg_inverse(uint32_t a, uint32_t n) {
  long long t = 0, nt = 1, r = n, nr = a;
  while (nr != 0) {
    const long long q = r / nr;
    long long tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  if (t < 0) t += n;
  return (uint32_t)t;
}

__device__ __forceinline__ uint32_t lg_gcd(uint32_t a, uint32_t b) {
  while (b) {
    const uint32_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// Exact flip energy A -> B of a site from its cluster counts: int32 sum of the
// integer weight multiples times the quantum, plus the f32 remainder chain.
__device__ __forceinline__ float lg_eab(const CeTables &T, const int (&n)[gen_fcc::N_ORBITS]) {
  int I = 0;
  float r = 0.f;
#pragma unroll
  for (int g = 0; g < gen_fcc::N_ORBITS; ++g) {
    I += T.wq[g] * n[g];
    r = FFMA(T.wr[g], (float)n[g], r);
  }
  return FFMA((float)I, T.wq_scale, r);
}

template <int PITCH>
__global__ void __launch_bounds__(LG_THREADS, 1)
    k_lgroup(const __grid_constant__ CeTables T, const __grid_constant__ LGroupParams LP) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int L = PITCH - 4, RH = 2, M = L / 3;
  static_assert(L % 6 == 0, "the learned group sweep needs L a multiple of 6");
  constexpr int N_SITES = L * L * L, N_C = M * M * M, N_GROUPS = (N_C + 31) / 32;
  constexpr int V = PITCH * PITCH * (L + 2 * RH);
  namespace cg = cooperative_groups;
  const cg::cluster_group cluster = cg::this_cluster();
  const int CL = LP.cluster;
  const int crank = (int)cluster.block_rank();
  const int rep = blockIdx.x / CL;
  const Replica &R = LP.reps[rep];
  ReplicaStats &S = LP.stats[rep];
  Geo G;
  G.L0 = G.L1 = G.L2 = L;
  G.R = RH;
  G.W = G.H = PITCH;
  G.V = V;
  int8_t *occ = reinterpret_cast<int8_t *>(smem);
  unsigned char *nb1 = smem + ((align16(V) + 127) & ~127);  // 128-byte aligned operands
  unsigned char *nb2 = nb1 + UMMA_B1_BYTES;
  unsigned char *abufs = nb2 + UMMA_B2_BYTES;  // [4 warpgroups][UMMA_A_BYTES]
  uint4 *nbits = reinterpret_cast<uint4 *>(abufs + 4 * UMMA_A_BYTES);  // byte -> 8 bf16 0/1
  float *fb = reinterpret_cast<float *>(abufs + 4 * UMMA_A_BYTES + UMMA_BITS_BYTES);  // b2, w3, b3
  uint64_t *nbar = reinterpret_cast<uint64_t *>(fb + 132);  // [4]
  uint32_t *tslot = reinterpret_cast<uint32_t *>(nbar + 4);
  __shared__ int s_order[LG_CLASSES];
  __shared__ uint32_t s_key[LG_CLASSES], s_ainv[LG_CLASSES], s_boff[LG_CLASSES];
  __shared__ int s_local[64];  // class | parity << 5 | neighbour << 8
  __shared__ int s_red[LG_NW][12];
  __shared__ int s_part[4][12];  // per-CTA pass totals, gathered in rank 0
  __shared__ long long s_cnt[gen_fcc::N_ORBITS], s_sub[4], s_n1;
  __shared__ double s_energy;
  __shared__ int s_stop;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int mode = LP.mode;
  const int rounds = LP.rounds, n_local = LP.n_local;
  const float beta_f = R.beta_f;
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);

  if (mode == 1) {
    umma_load_net(LP.params, nb1, nb2, nbits, fb, tid, LG_THREADS);
    if (tid < 4) mbar_init(&nbar[tid], 1);
    if (warp == 0) tmem_alloc(tslot, 4 * UMMA_COLS);
    mbar_init_fence();
    fence_proxy_async_smem();
    tc_fence_before();
  }
  // ---- stage the replica with its periodic halo
  const int8_t *gocc = LP.occ + R.occ_offset;
  for (int l = tid; l < N_SITES; l += LG_THREADS) {
    const int x = l % L, y = (l / L) % L, z = l / (L * L);
    occ[G.addr(0, x, y, z)] = gocc[l];
  }
  __syncthreads();
  for (int h = tid; h < V; h += LG_THREADS) {
    const int xh = h % PITCH, yh = (h / PITCH) % PITCH, zh = h / (PITCH * PITCH);
    const int x = xh - RH, y = yh - RH, z = zh - RH;
    if (x >= 0 && x < L && y >= 0 && y < L && z >= 0 && z < L) continue;
    occ[h] = occ[G.addr(0, wrapc(x, L), wrapc(y, L), wrapc(z, L))];
  }
  if (tid < gen_fcc::N_ORBITS) s_cnt[tid] = 0;
  if (tid < 4) s_sub[tid] = 0;
  if (tid == 0) {
    s_n1 = 0;
    s_stop = 0;
  }
  __syncthreads();
  // ---- exact initial energy (owned clusters) and species / sublattice counts
  // (rank 0 keeps the replica's running statistics)
  if (crank == 0) {
    long long cnt[gen_fcc::N_ORBITS] = {0, 0, 0, 0, 0, 0};
    long long sub[4] = {0, 0, 0, 0}, n1 = 0;
    for (int l = tid; l < N_SITES; l += LG_THREADS) {
      const int x = l % L, y = (l / L) % L, z = l / (L * L);
      const int ad = G.addr(0, x, y, z);
      if (!occ[ad]) continue;
      int nn[gen_fcc::N_ORBITS];
      gen_fcc::owned_counts<PITCH>(occ + ad, nn);
      for (int g = 0; g < gen_fcc::N_ORBITS; ++g) cnt[g] += nn[g];
      sub[sc_sublattice(x, y, z)]++;
      ++n1;
    }
    for (int g = 0; g < gen_fcc::N_ORBITS; ++g)
      atomicAdd((unsigned long long *)&s_cnt[g], (unsigned long long)cnt[g]);
    for (int k = 0; k < 4; ++k) atomicAdd((unsigned long long *)&s_sub[k], (unsigned long long)sub[k]);
    atomicAdd((unsigned long long *)&s_n1, (unsigned long long)n1);
  }
  __syncthreads();
  if (tid == 0 && crank == 0) {
    double e = T.w[0] * (double)N_SITES;
    for (int g = 0; g < T.n_orbits; ++g) e += T.w[T.orb_func_base[g]] * (double)s_cnt[g];
    s_energy = e;
    const long long pass = S.pass, np = S.n_proposed, na = S.n_accepted;
    unsigned char *raw = reinterpret_cast<unsigned char *>(&S);
    for (int q = 0; q < (int)sizeof(ReplicaStats); ++q) raw[q] = 0;
    S.pass = pass;
    S.n_proposed = np;
    S.n_accepted = na;
    S.n_species[0] = N_SITES - s_n1;
    S.n_species[1] = s_n1;
    for (int k = 0; k < 4; ++k) S.n_sub[k] = s_sub[k];
  }
  __syncthreads();

  if (mode == 1) tc_fence_after();  // the barriers above ordered the allocation
  const UmmaNet net{nb1, nb2, nbits, fb, fb + 64, mode == 1 ? fb[128] : 0.f};
  const int wg = warp >> 2;
  const uint32_t tm = mode == 1 ? *tslot + (uint32_t)(wg * UMMA_COLS) : 0u;
  uint32_t nphase = 0;
  bool ntimeout = false;
  // every copy of the replica (own and peers' shared memory) receives each
  // accepted change
  auto put_all = [&](int x, int y, int z, int8_t v) {
    for (int r = 0; r < CL; ++r) put_site(cluster.map_shared_rank(occ, r), G, 0, x, y, z, v);
  };
  cluster.sync();  // every copy is staged before any peer writes into it
  long long pass_global = S.pass;
  long long nsub[4];
  for (int k = 0; k < 4; ++k) nsub[k] = s_sub[k];
  const long long n_b = s_n1;
  for (long long ip = 0; ip < LP.n_passes; ++ip, ++pass_global) {
    const uint32_t plo = (uint32_t)pass_global, phi = (uint32_t)(pass_global >> 32) & 0xFFFFu;
    // the host's stop flag, read here and published at the end of the pass
    const int stop_seen = (tid == 0 && crank == 0 && LP.stop) ? *LP.stop : 0;
    // ---- schedule: class order, group permutations, local sub-steps
    if (tid < LG_CLASSES) {
      const U4 r = philox4x32_10(U4{(uint32_t)tid, 0u, plo, phi | (TAG_LG_SCHED << 16)}, k0, k1);
      s_key[tid] = r.x;
      // multiplier coprime with N_C (bounded search; 1 always qualifies)
      uint32_t a = 1u;
      for (int tries = 0; tries < 8; ++tries) {
        const U4 q = philox4x32_10(U4{(uint32_t)tid, 1u + (uint32_t)tries, plo, phi | (TAG_LG_SCHED << 16)},
                                   k0, k1);
        const uint32_t cand = 1u + q.x % (uint32_t)(N_C > 1 ? N_C - 1 : 1);
        if (lg_gcd(cand, (uint32_t)N_C) == 1u) {
          a = cand;
          break;
        }
      }
      s_ainv[tid] = N_C > 1 ? lg_inverse(a % (uint32_t)N_C, (uint32_t)N_C) : 0u;
      s_boff[tid] = r.y % (uint32_t)N_C;
    } else if (tid >= 32 && tid < 32 + n_local) {
      const int j = tid - 32;
      const U4 r = philox4x32_10(U4{(uint32_t)j, 2u, plo, phi | (TAG_LG_LOCAL << 16)}, k0, k1);
      s_local[j] = (int)(r.x % LG_CLASSES) | (int)((r.y & 7u) << 5) | (int)((r.z % 12u) << 8);
    }
    __syncthreads();
    if (tid < LG_CLASSES) {
      int rank = 0;
      for (int c2 = 0; c2 < LG_CLASSES; ++c2)
        rank += (s_key[c2] < s_key[tid]) || (s_key[c2] == s_key[tid] && c2 < tid);
      s_order[rank] = tid;
    }
    __syncthreads();
    if (s_stop) break;  // the host asked the run to stop

    int n_prop = 0, n_acc = 0;
    int dcn[gen_fcc::N_ORBITS] = {0, 0, 0, 0, 0, 0};
    RegCounts<4> dsub;
    // ---- group sub-steps
    for (int sub = 0; sub < LG_CLASSES; ++sub) {
      const int c = s_order[sub];
      const int cx = c % 3, cy = (c / 3) % 3, cz = c / 9;
      const uint32_t ainv = s_ainv[c], boff = s_boff[c];
      // warps iterate in step so that the four warps of a warpgroup evaluate
      // the network together; a warpgroup stops when its first warp has no
      // group left (the later warps then have none either)
      const int n_iter = (N_GROUPS + CL * LG_NW - 1) / (CL * LG_NW);
      for (int it = 0; it < n_iter; ++it) {
        const int grp0 = it * CL * LG_NW + crank * LG_NW;
        if (grp0 + 4 * wg >= N_GROUPS) break;
        const int grp = grp0 + warp;
        const int r = grp * 32 + lane;
        const bool act = grp < N_GROUPS && r < N_C;
        int x = 0, y = 0, z = 0, ad = 0, o = 0;
        int n[gen_fcc::N_ORBITS] = {0, 0, 0, 0, 0, 0};
        unsigned long long env = 0ull;
        if (act) {
          const uint32_t q = (uint32_t)(((unsigned long long)ainv *
                                         (unsigned long long)(((uint32_t)r + (uint32_t)N_C - boff) %
                                                              (uint32_t)N_C)) %
                                        (unsigned long long)N_C);
          const int i = (int)(q % M), j = (int)((q / M) % M), k = (int)(q / (M * M));
          x = cx + 3 * i;
          y = cy + 3 * j;
          z = cz + 3 * k;
          ad = G.addr(0, x, y, z);
          o = occ[ad];
          gen_fcc::counts_env<PITCH>(occ + ad, n, env);
        }
        const float eab = lg_eab(T, n);
        // this lane's round: two Philox blocks (64-bit uniforms for both
        // draws, 24 bits for the acceptance). Even warpgroups draw them before
        // the network and odd ones after it, so that the warpgroups of a CTA
        // do not all wait on their MMAs at the same time.
        unsigned long long ua_own = 0ull, ub_own = 0ull;
        uint32_t uu_own = 0u;
        auto draw = [&]() {
          if (lane < rounds) {
            const uint32_t ctr = (uint32_t)grp | ((uint32_t)sub << 16);
            const U4 p = philox4x32_10(U4{ctr, (uint32_t)lane, plo, phi | (TAG_LG_GROUP << 16)}, k0, k1);
            const U4 p2 = philox4x32_10(U4{ctr, (uint32_t)lane | 0x100u, plo, phi | (TAG_LG_GROUP << 16)},
                                        k0, k1);
            ua_own = ((unsigned long long)p.x << 32) | p.y;
            ub_own = ((unsigned long long)p.z << 32) | p.w;
            uu_own = p2.x;
          }
        };
        if ((wg & 1) == 0) draw();
        float zl = 0.f;
        if (mode == 1) zl = umma_network(net, abufs + wg * UMMA_A_BYTES, tm, &nbar[wg], nphase, wg, env, ntimeout);
        else if (mode == 2) zl = FMUL(-0.5f * beta_f, eab);
        if (wg & 1) draw();
        const uint32_t wA = mode ? (uint32_t)logit_weight(zl) : 1u;
        const uint32_t wB = mode ? (uint32_t)logit_weight(-zl) : 1u;
        const int o0 = o;
        uint32_t wc = o ? wB : wA, wa = o ? wA : wB;
        float eme = o ? -eab : eab;  // this member's flip energy in its current state
        // inclusive prefix sums of the A and B weights over the lanes; they
        // change only when a swap is accepted
        uint32_t sa = 0u, sb = 0u, WA = 0u, WB = 0u;
        bool dirty = true;
        for (int t = 0; t < rounds; ++t) {
          if (dirty) {
            sa = (act && o == 0) ? wc : 0u;
            sb = (act && o == 1) ? wc : 0u;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
              const uint32_t va = __shfl_up_sync(0xffffffffu, sa, off);
              const uint32_t vb = __shfl_up_sync(0xffffffffu, sb, off);
              if (lane >= off) {
                sa += va;
                sb += vb;
              }
            }
            WA = __shfl_sync(0xffffffffu, sa, 31);
            WB = __shfl_sync(0xffffffffu, sb, 31);
            dirty = false;
          }
          if (WA == 0u || WB == 0u) break;  // one species absent from the group
          const unsigned long long ua = shfl64(ua_own, t), ub = shfl64(ub_own, t);
          const uint32_t uu = __shfl_sync(0xffffffffu, uu_own, t);
          const uint32_t xa = (uint32_t)__umul64hi(ua, (unsigned long long)WA);
          const uint32_t xb = (uint32_t)__umul64hi(ub, (unsigned long long)WB);
          const int la = __ffs(__ballot_sync(0xffffffffu, sa > xa)) - 1;
          const int lb = __ffs(__ballot_sync(0xffffffffu, sb > xb)) - 1;
          const float ea = __shfl_sync(0xffffffffu, eme, la), eb = __shfl_sync(0xffffffffu, eme, lb);
          const uint32_t wca = __shfl_sync(0xffffffffu, wc, la), waa = __shfl_sync(0xffffffffu, wa, la);
          const uint32_t wcb = __shfl_sync(0xffffffffu, wc, lb), wab = __shfl_sync(0xffffffffu, wa, lb);
          const uint32_t WA2 = WA - wca + wab, WB2 = WB - wcb + waa;
          const float dE = FADD(ea, eb);
          bool accept;
          if (mode == 0) {
            accept = accept_de(dE, beta_f, u24(uu));
          } else {
            // q_rev / q_fwd = (W_A W_B / (W_A' W_B')) (w'_a w'_b / (w_a w_b)); each
            // product stays below 2^32 x 2^32 x 2^27 x 2^27 < 2^128
            const float num = FMUL(FMUL((float)WA, (float)WB), FMUL((float)waa, (float)wab));
            const float den = FMUL(FMUL((float)WA2, (float)WB2), FMUL((float)wca, (float)wcb));
            const float ratio = __fdiv_rn(num, den);
            const float lr = FFMA(-beta_f, dE, logf(ratio));
            accept = (lr >= 0.f) || (u24(uu) < cem_expf_neg(lr));
          }
          if (lane == 0) {
            ++n_prop;
            n_acc += accept ? 1 : 0;
          }
          if (accept) {
            dirty = true;
            if (lane == la || lane == lb) {
              o ^= 1;
              eme = -eme;
              const uint32_t tmp = wc;
              wc = wa;
              wa = tmp;
            }
          }
        }
        if (act && o != o0) {
          put_all(x, y, z, (int8_t)o);
          const int d = o - o0;
#pragma unroll
          for (int g = 0; g < gen_fcc::N_ORBITS; ++g) dcn[g] += d * n[g];
          dsub.add(sc_sublattice(x, y, z), d);
        }
      }
      cluster.sync();  // the class's changes are in every copy
    }
    // ---- nearest-neighbour swaps (plain Metropolis) between classes
    constexpr int H = M / 2, N_ANCHOR = H * H * H;
    for (int ls = 0; ls < n_local; ++ls) {
      const int code = s_local[ls];
      const int c = code & 31, par = (code >> 5) & 7, dl = code >> 8;
      const int cx = c % 3, cy = (c / 3) % 3, cz = c / 9;
      const int dx = gen_fcc::NB_D[dl][0], dy = gen_fcc::NB_D[dl][1], dz = gen_fcc::NB_D[dl][2];
      for (int q = crank * LG_THREADS + tid; q < N_ANCHOR; q += CL * LG_THREADS) {
        const int i = q % H, j = (q / H) % H, k = q / (H * H);
        const int xa = cx + 3 * (2 * i + (par & 1)), ya = cy + 3 * (2 * j + ((par >> 1) & 1)),
                  za = cz + 3 * (2 * k + ((par >> 2) & 1));
        const int xb = wrapc(xa + dx, L), yb = wrapc(ya + dy, L), zb = wrapc(za + dz, L);
        const int ada = G.addr(0, xa, ya, za), adb = G.addr(0, xb, yb, zb);
        const int oa = occ[ada], ob = occ[adb];
        if (oa == ob) continue;
        const int la = xa + L * (ya + L * za);
        const U4 rr = philox4x32_10(U4{(uint32_t)la, (uint32_t)(LG_CLASSES + ls), plo,
                                       phi | (TAG_LG_LOCAL << 16)},
                                    k0, k1);
        // the first change is applied (in this CTA's copy) before either
        // flower is read (a site's flower never contains the site): a sees
        // the original state, b sees a changed, as for a sequence of two
        // changes
        put_site(occ, G, 0, xa, ya, za, (int8_t)ob);
        int na[gen_fcc::N_ORBITS], nb[gen_fcc::N_ORBITS];
        gen_fcc::counts<PITCH>(occ + ada, na);
        gen_fcc::counts<PITCH>(occ + adb, nb);
        const int d = ob - oa;  // a: oa -> ob, b: ob -> oa
        int I = 0;
        float rm = 0.f;
        int dc[gen_fcc::N_ORBITS];
#pragma unroll
        for (int g = 0; g < gen_fcc::N_ORBITS; ++g) {
          dc[g] = d * (na[g] - nb[g]);
          I += T.wq[g] * dc[g];
          rm = FFMA(T.wr[g], (float)dc[g], rm);
        }
        const float de = FFMA((float)I, T.wq_scale, rm);
        ++n_prop;
        if (accept_de(de, beta_f, u24(rr.x))) {
          ++n_acc;
          put_all(xa, ya, za, (int8_t)ob);
          put_all(xb, yb, zb, (int8_t)oa);
#pragma unroll
          for (int g = 0; g < gen_fcc::N_ORBITS; ++g) dcn[g] += dc[g];
          dsub.add(sc_sublattice(xa, ya, za), d);
          dsub.add(sc_sublattice(xb, yb, zb), -d);
        } else {
          put_site(occ, G, 0, xa, ya, za, (int8_t)oa);
        }
      }
      cluster.sync();
    }
    // ---- end of pass: reduce, update the exact running energy, sample
    {
      int vals[12];
      vals[0] = n_prop;
      vals[1] = n_acc;
#pragma unroll
      for (int g = 0; g < gen_fcc::N_ORBITS; ++g) vals[2 + g] = dcn[g];
#pragma unroll
      for (int k = 0; k < 4; ++k) vals[8 + k] = dsub.v[k];
#pragma unroll
      for (int k = 0; k < 12; ++k)
        for (int off = 16; off; off >>= 1) vals[k] += __shfl_xor_sync(0xffffffffu, vals[k], off);
      if (lane == 0)
        for (int k = 0; k < 12; ++k) s_red[warp][k] = vals[k];
      __syncthreads();
      if (tid == 0) {  // this CTA's totals -> rank 0
        int *part = cluster.map_shared_rank(&s_part[0][0], 0) + 12 * crank;
        for (int k = 0; k < 12; ++k) {
          int t = 0;
          for (int w = 0; w < LG_NW; ++w) t += s_red[w][k];
          part[k] = t;
        }
      }
      cluster.sync();
      if (tid == 0 && crank == 0) {
        for (int r = 0; r < CL; ++r) *cluster.map_shared_rank(&s_stop, r) = stop_seen;
        long long tot[12];
        for (int k = 0; k < 12; ++k) {
          tot[k] = 0;
          for (int r = 0; r < CL; ++r) tot[k] += s_part[r][k];
        }
        double de = 0.0;
        for (int g = 0; g < T.n_orbits; ++g) de += T.w[T.orb_func_base[g]] * (double)tot[2 + g];
        s_energy += de;
        S.n_proposed += tot[0];
        S.n_accepted += tot[1];
        for (int k = 0; k < 4; ++k) nsub[k] += tot[8 + k];
        const double xb = (double)n_b / N_SITES;
        double op = 0.0;
        for (int k = 0; k < 4; ++k) {
          const double cc = (double)nsub[k] / (0.25 * N_SITES) - xb;
          op += cc * cc;
        }
        op = sqrt(op);
        const double ef = s_energy / N_SITES;
        if (ip >= LP.n_equil) {
          S.n_samples += 1.0;
          S.sum_e += ef;
          S.sum_e2 += ef * ef;
          S.sum_f += ef;
          S.sum_x[0] += xb;
          S.sum_xx[0] += xb * xb;
          S.sum_ex[0] += ef * xb;
          if (LP.samples) {
            const long long si = (long long)S.n_samples - 1;
            if (si < LP.sample_capacity) {
              double *out = LP.samples + ((long long)rep * LP.sample_capacity + si) * 3;
              out[0] = ef;
              out[1] = xb;
              out[2] = op;
            }
          }
        }
      }
      cluster.sync();  // the stop decision is in every CTA
    }
  }
  // ---- write back (rank 0; every copy is identical)
  if (crank == 0) {
    for (int l = tid; l < N_SITES; l += LG_THREADS) {
      const int x = l % L, y = (l / L) % L, z = l / (L * L);
      LP.occ[R.occ_offset + l] = occ[G.addr(0, x, y, z)];
    }
    if (tid == 0) {
      S.energy = s_energy;
      S.pass = pass_global;
      for (int k = 0; k < 4; ++k) S.n_sub[k] = nsub[k];
    }
  }
  if (mode == 1) {
    if (ntimeout) {
      atomicExch(&S.status, 8);  // an MMA wait ran out: results are invalid
      // let the last committed MMA land before the tensor memory is freed
      // (bounded; its parity is the one before the last toggle)
      mbar_wait(&nbar[wg], nphase ^ 1u, UMMA_WAIT_ITERS);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(*tslot, 4 * UMMA_COLS);
  }
  cluster.sync();  // no CTA leaves while a peer may still write to it
}

// Inference of n environments on tcgen05 (the network of umma_network): 4
// warpgroups per CTA, 128 environments per warpgroup and batch; status[0]
// is set when an MMA wait ran out.
constexpr int UMMA_FWD_THREADS = 512;
constexpr int UMMA_FWD_SMEM =
    UMMA_B1_BYTES + UMMA_B2_BYTES + 4 * UMMA_A_BYTES + UMMA_BITS_BYTES + 1024;
__global__ void __launch_bounds__(UMMA_FWD_THREADS)
    k_mlp_forward_tc(const __nv_bfloat16 *__restrict__ params, const int8_t *__restrict__ X,
                       long long n, float *__restrict__ z, int *status) {
  extern __shared__ __align__(128) unsigned char usm[];
  unsigned char *b1 = usm, *b2 = usm + UMMA_B1_BYTES;
  unsigned char *abufs = b2 + UMMA_B2_BYTES;
  uint4 *bits = reinterpret_cast<uint4 *>(abufs + 4 * UMMA_A_BYTES);
  float *fb = reinterpret_cast<float *>(abufs + 4 * UMMA_A_BYTES + UMMA_BITS_BYTES);  // 129 floats
  uint64_t *bars = reinterpret_cast<uint64_t *>(fb + 132);  // 4 mbarriers
  uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5, wg = warp >> 2;
  umma_load_net(params, b1, b2, bits, fb, tid, UMMA_FWD_THREADS);
  if (tid < 4) mbar_init(&bars[tid], 1);
  if (warp == 0) tmem_alloc(slot, 4 * UMMA_COLS);
  mbar_init_fence();
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = *slot + (uint32_t)(wg * UMMA_COLS);
  const UmmaNet net{b1, b2, bits, fb, fb + 64, fb[128]};
  unsigned char *abuf = abufs + wg * UMMA_A_BYTES;
  uint32_t phase = 0;
  bool timeout = false;
  const int row = tid & 127;
  for (long long t = (long long)blockIdx.x * 4 + wg; t * 128 < n; t += (long long)gridDim.x * 4) {
    const long long e = t * 128 + row;
    unsigned long long env = 0ull;
    if (e < n)
      for (int k = 0; k < MLP_IN; ++k) env |= (unsigned long long)(X[e * MLP_IN + k] != 0) << k;
    const float zz = umma_network(net, abuf, tm, &bars[wg], phase, wg, env, timeout);
    if (e < n) z[e] = zz;
  }
  if (timeout) {
    atomicExch(status, 1);
    // let the last committed MMA land before the tensor memory is freed
    mbar_wait(&bars[wg], phase ^ 1u, UMMA_WAIT_ITERS);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(*slot, 4 * UMMA_COLS);
}

cudaError_t mlp_forward_tc(const __nv_bfloat16 *params, const int8_t *X, long long n, float *z,
                             int *status, cudaStream_t st) {
  cudaError_t e =
      cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, UMMA_FWD_SMEM);
  if (e != cudaSuccess) return e;
  long long grid = (n + 511) / 512;
  if (grid > 304) grid = 304;  // two CTAs per SM: 2 x 256 tensor-memory columns
  if (grid < 1) grid = 1;
  k_mlp_forward_tc<<<(int)grid, UMMA_FWD_THREADS, UMMA_FWD_SMEM, st>>>(params, X, n, z, status);
  return cudaGetLastError();
}

int lgroup_smem_bytes(int L) {
  const int pitch = L + 4;
  return ((align16(pitch * pitch * pitch) + 127) & ~127) + LG_NET_BYTES;
}

bool lgroup_supported(int L) { return L == 12 || L == 24 || L == 36 || L == 48; }

cudaError_t lgroup_run(const CeTables &T, const Replica *reps, ReplicaStats *stats, int8_t *occ,
                       const __nv_bfloat16 *params, int mode, int rounds, int n_local,
                       int n_replicas, int L, long long n_passes, long long n_equil,
                       double *samples, long long capacity, const volatile int *stop,
                       int cluster, cudaStream_t st) {
  LGroupParams LP{};
  LP.stop = stop;
  LP.reps = reps;
  LP.stats = stats;
  LP.occ = occ;
  LP.params = params;
  LP.mode = mode;
  LP.rounds = rounds;
  LP.n_local = n_local;
  LP.n_passes = n_passes;
  LP.n_equil = n_equil;
  LP.samples = samples;
  LP.sample_capacity = capacity;
  LP.cluster = cluster;
  const int smem = lgroup_smem_bytes(L);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n_replicas * cluster));
  cfg.blockDim = dim3(LG_THREADS);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaSuccess;
  switch (L) {
#define CEM_LGROUP_CASE(LL)                                                                      \
  case LL:                                                                                       \
    e = cudaFuncSetAttribute(k_lgroup<LL + 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e != cudaSuccess) return e;                                                              \
    e = cudaLaunchKernelEx(&cfg, k_lgroup<LL + 4>, T, LP);                                       \
    if (e != cudaSuccess) return e;                                                              \
    break;
    CEM_LGROUP_CASE(12)
    CEM_LGROUP_CASE(24)
    CEM_LGROUP_CASE(36)
    CEM_LGROUP_CASE(48)
#undef CEM_LGROUP_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace cem
