// Kernels of the GB300 cluster-expansion Metropolis hot path.
//
//  k_energy   : integer function counts of a whole occupation (per_supercell)
//  k_delta    : batched occ_delta_per_supercell, one thread per event
//  k_replay   : occupation_metropolis_v2 restated step by step, one warp per
//               chain, consuming the std::mt19937_64 stream
//  k_sweep    : parallel Metropolis, one CTA per replica, occupation resident
//               in shared memory with a periodic halo, colour classes of
//               non-interacting sites updated at once
//
// Delta correlations are integer counts: for each orbit g, the number of
// flower clusters whose decoration changes in or out of each function class.
// Binary systems (two occupants) count products of partner occupations;
// systems with more occupants look the decoration up in a per-cluster table
// and accumulate +1/-1 in 8-bit fields of a 64-bit word per orbit.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "cem_common.cuh"
#include "cem_internal.h"
#include "gen_fcc_binary.cuh"

namespace cem {

// ------------------------------------------------------------ accumulators
template <int NOCC>
struct Acc {
  unsigned long long p[MAX_ORBITS], m[MAX_ORBITS];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int g = 0; g < MAX_ORBITS; ++g) p[g] = m[g] = 0ull;
  }
};
template <>
struct Acc<2> {
  int c[MAX_ORBITS];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int g = 0; g < MAX_ORBITS; ++g) c[g] = 0;
  }
};

// Delta counts of one orbit for one changed site (centre of sublattice b,
// o_i -> o_f): binary systems an integer count change, other systems packed
// 8-bit counts of the decorations gained (p) and lost (m) per local function.
// rd(c, j) returns the occupant of partner j of cluster c.
template <int NOCC>
struct OrbAcc {
  unsigned long long p = 0ull, m = 0ull;
};
template <>
struct OrbAcc<2> {
  int c = 0;
};

template <int NOCC, class Reader>
__device__ __forceinline__ void orbit_site(const CeTables &T, int b, int g, int o_i, int o_f,
                                           const int *__restrict__ lutoff,
                                           const uint8_t *__restrict__ lut, Reader rd,
                                           OrbAcc<NOCC> &a) {
  const int c0 = T.fl_begin[b][g], c1 = T.fl_begin[b][g + 1];
  const int size = T.orb_size[g];
  if constexpr (NOCC == 2) {
    int cnt = 0;
    if (size == 1) {
      cnt = c1 - c0;
    } else if (size == 2) {
      for (int c = c0; c < c1; ++c) cnt += rd(c, 0);
    } else if (size == 3) {
      for (int c = c0; c < c1; ++c) cnt += rd(c, 0) & rd(c, 1);
    } else {
      for (int c = c0; c < c1; ++c) cnt += rd(c, 0) & rd(c, 1) & rd(c, 2);
    }
    a.c += (o_f - o_i) * cnt;
  } else {
    constexpr int NSF = NOCC - 1;
    for (int c = c0; c < c1; ++c) {
      int code = 0, mul = NSF;
      bool ok = true;
      for (int j = 0; j < size - 1; ++j) {
        int v = rd(c, j);
        ok = ok && (v != 0);
        code += (v - 1) * mul;
        mul *= NSF;
      }
      if (ok) {
        const int base = lutoff[c] + code;
        if (o_f) a.p += 1ull << (8 * lut[base + o_f - 1]);
        if (o_i) a.m += 1ull << (8 * lut[base + o_i - 1]);
      }
    }
  }
}

// Add the float-float terms W_f dC_f of orbit g's functions to r (functions
// in increasing order; binary systems add the orbit's one term even when it is
// zero, other systems skip zero terms).
template <int NOCC>
__device__ __forceinline__ void orbit_fold(const CeTables &T, int g, const OrbAcc<NOCC> &a,
                                           const float *__restrict__ whi,
                                           const float *__restrict__ wlo, FF &r) {
  const int base = T.orb_func_base[g];
  if constexpr (NOCC == 2) {
    ff_add_term(r, whi[base], wlo[base], a.c);
  } else {
    const int nf = T.orb_n_funcs[g];
    for (int fl = 0; fl < nf; ++fl) {
      const int dc = (int)((a.p >> (8 * fl)) & 255ull) - (int)((a.m >> (8 * fl)) & 255ull);
      if (dc) ff_add_term(r, whi[base + fl], wlo[base + fl], dc);
    }
  }
}

// Add the delta counts of changing the centre site of sublattice b from o_i
// to o_f, for the first MAX_ORBITS orbits (register accumulators).
template <int NOCC, class Reader>
__device__ __forceinline__ void accumulate_site(const CeTables &T, int b, int o_i, int o_f,
                                                const int *__restrict__ lutoff,
                                                const uint8_t *__restrict__ lut, Reader rd,
                                                Acc<NOCC> &acc) {
#pragma unroll
  for (int g = 0; g < MAX_ORBITS; ++g) {
    if (g < T.n_orbits) {
      OrbAcc<NOCC> a;
      orbit_site<NOCC>(T, b, g, o_i, o_f, lutoff, lut, rd, a);
      if constexpr (NOCC == 2) {
        acc.c[g] += a.c;
      } else {
        acc.p[g] += a.p;
        acc.m[g] += a.m;
      }
    }
  }
}

template <int NOCC>
__device__ __forceinline__ int acc_dc(const Acc<NOCC> &acc, int g, int fl) {
  if constexpr (NOCC == 2) {
    return acc.c[g];
  } else {
    return (int)((acc.p[g] >> (8 * fl)) & 255ull) - (int)((acc.m[g] >> (8 * fl)) & 255ull);
  }
}

// sum_f W_f dC_f in float-float, functions in increasing order.
template <int NOCC>
__device__ __forceinline__ FF acc_dot(const CeTables &T, const Acc<NOCC> &acc,
                                      const float *__restrict__ whi,
                                      const float *__restrict__ wlo) {
  FF r{0.f, 0.f};
#pragma unroll
  for (int g = 0; g < MAX_ORBITS; ++g) {
    if (g < T.n_orbits) {
      const int base = T.orb_func_base[g];
      if constexpr (NOCC == 2) {
        ff_add_term(r, whi[base], wlo[base], acc.c[g]);  // a zero term adds exact zeros
      } else {
        const int nf = T.orb_n_funcs[g];
        for (int fl = 0; fl < nf; ++fl) {
          const int dc = acc_dc<NOCC>(acc, g, fl);
          if (dc) ff_add_term(r, whi[base + fl], wlo[base + fl], dc);
        }
      }
    }
  }
  return r;
}

__device__ __forceinline__ int wrapc(int x, int L) {
  x = (x < 0) ? x + L : x;
  return (x >= L) ? x - L : x;
}

// ------------------------------------------------------------ full energy
template <int NOCC>
__global__ void k_energy(const __grid_constant__ CeTables T, const int8_t *__restrict__ occ,
                         Cells C, unsigned long long *__restrict__ counts) {
  __shared__ int hist[MAX_FUNCS];
  for (int f = threadIdx.x; f < MAX_FUNCS; f += blockDim.x) hist[f] = 0;
  __syncthreads();
  const int L0 = C.L0, L1 = C.L1;
  const int n_uc = L0 * L1 * C.L2;
  const int n = n_uc * T.n_sublat;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x) {
    const int b = l / n_uc, uc = l - b * n_uc;
    const int i = uc % L0, j = (uc / L0) % L1, k = uc / (L0 * L1);
    const int o0 = occ[l];
    if (o0 == 0) continue;  // every owned cluster contains its anchor
    for (int g = 0; g < T.n_orbits; ++g) {
      const int size = T.orb_size[g];
      for (int c = T.ow_begin[b][g]; c < T.ow_begin[b][g + 1]; ++c) {
        const int cc = T.n_fl + c;
        int code = o0 - 1, mul = NOCC - 1;
        bool ok = true;
        for (int q = 0; q < size - 1; ++q) {
          const int pb = T.cl_pb[cc * 3 + q];
          const int *du = T.cl_du + cc * 9 + q * 3;
          const int site = pb * n_uc + C.index(i + du[0], j + du[1], k + du[2]);
          const int v = occ[site];
          ok = ok && (v != 0);
          code += (v - 1) * mul;
          mul *= (NOCC - 1);
        }
        if (ok) atomicAdd(&hist[T.orb_func_base[g] + T.lut[T.cl_lut[cc] + code]], 1);
      }
    }
  }
  __syncthreads();
  for (int f = threadIdx.x; f < T.n_funcs; f += blockDim.x)
    if (hist[f]) atomicAdd(&counts[f], (unsigned long long)hist[f]);
}

// Exact initial state of every replica (one CTA per replica): function
// counts -> formation energy, species counts; clears the sampled moments.
// The replica's occupation is staged in shared memory when it fits
// (smem_cap bytes), else read from global memory.
template <int NOCC>
__global__ void k_init_stats(const __grid_constant__ CeTables T, const Replica *__restrict__ reps,
                             ReplicaStats *__restrict__ stats, const int8_t *__restrict__ occ_all,
                             int smem_cap) {
  extern __shared__ __align__(16) int8_t socc[];
  __shared__ unsigned long long hist[MAX_FUNCS];
  __shared__ unsigned long long spec[8];
  const Replica &R = reps[blockIdx.x];
  for (int f = threadIdx.x; f < MAX_FUNCS; f += blockDim.x) hist[f] = 0ull;
  if (threadIdx.x < 8) spec[threadIdx.x] = 0ull;
  const Cells C = R.cells();
  const int L0 = C.L0, L1 = C.L1;
  const int n_uc = L0 * L1 * C.L2, n = n_uc * T.n_sublat;
  const int8_t *gocc = occ_all + R.occ_offset;
  const bool staged = n <= smem_cap;
  if (staged)
    for (int l = threadIdx.x; l < n; l += blockDim.x) socc[l] = gocc[l];
  __syncthreads();
  const int8_t *occ = staged ? socc : gocc;
  int lspec[NOCC];
  for (int a = 0; a < NOCC; ++a) lspec[a] = 0;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    const int b = l / n_uc, uc = l - b * n_uc;
    const int i = uc % L0, j = (uc / L0) % L1, k = uc / (L0 * L1);
    const int o0 = occ[l];
    lspec[o0]++;
    if (o0 == 0) continue;
    for (int g = 0; g < T.n_orbits; ++g) {
      const int size = T.orb_size[g];
      for (int c = T.ow_begin[b][g]; c < T.ow_begin[b][g + 1]; ++c) {
        const int cc = T.n_fl + c;
        int code = o0 - 1, mul = NOCC - 1;
        bool ok = true;
        for (int q = 0; q < size - 1; ++q) {
          const int pb = T.cl_pb[cc * 3 + q];
          const int *du = T.cl_du + cc * 9 + q * 3;
          const int site = pb * n_uc + C.index(i + du[0], j + du[1], k + du[2]);
          const int v = occ[site];
          ok = ok && (v != 0);
          code += (v - 1) * mul;
          mul *= (NOCC - 1);
        }
        if (ok) atomicAdd(&hist[T.orb_func_base[g] + T.lut[T.cl_lut[cc] + code]], 1ull);
      }
    }
  }
  for (int a = 0; a < NOCC; ++a)
    if (lspec[a]) atomicAdd(&spec[a], (unsigned long long)lspec[a]);
  __syncthreads();
  if (threadIdx.x == 0) {
    ReplicaStats &S = stats[blockIdx.x];
    double e = T.w[0] * n_uc;
    for (int f = 1; f < T.n_funcs; ++f) e += T.w[f] * (double)hist[f];
    const long long pass = S.pass, np = S.n_proposed, na = S.n_accepted;
    unsigned char *raw = reinterpret_cast<unsigned char *>(&S);
    for (int q = 0; q < (int)sizeof(ReplicaStats); ++q) raw[q] = 0;
    S.energy = e;
    for (int a = 0; a < NOCC; ++a) S.n_species[a] = (int64_t)spec[a];
    S.pass = pass;
    S.n_proposed = np;
    S.n_accepted = na;
  }
}

// ------------------------------------------------------------ batched delta
template <int NOCC>
__global__ void k_delta(const __grid_constant__ CeTables T, const int8_t *__restrict__ occ,
                        Cells C, int n_events, int k_sites,
                        const long long *__restrict__ sites, const int *__restrict__ new_occ,
                        const double *__restrict__ dmu, double *__restrict__ dE,
                        long long *__restrict__ dcount) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_events) return;
  const int L0 = C.L0, L1 = C.L1;
  const int n_uc = L0 * L1 * C.L2;
  double mu_term = 0.0;
  // sequential semantics: site s sees the changes of sites 0 .. s-1
  int ov_site[4], ov_val[4], sb[4], si[4], sj[4], sk[4], soi[4], sof[4];
  for (int s = 0; s < k_sites; ++s) {
    const int l = (int)sites[e * k_sites + s];
    const int b = l / n_uc, uc = l - b * n_uc;
    sb[s] = b;
    si[s] = uc % L0;
    sj[s] = (uc / L0) % L1;
    sk[s] = uc / (L0 * L1);
    int o_i = occ[l];
    for (int q = 0; q < s; ++q)
      if (ov_site[q] == l) o_i = ov_val[q];
    soi[s] = o_i;
    sof[s] = new_occ[e * k_sites + s];
    if (dmu) mu_term += dmu[o_i * NOCC + sof[s]];
    ov_site[s] = l;
    ov_val[s] = sof[s];
  }
  FF d{0.f, 0.f};
  long long *dc_out = dcount ? dcount + (long long)e * T.n_funcs : nullptr;
  if (dc_out) dc_out[0] = 0;
  for (int g = 0; g < T.n_orbits; ++g) {
    OrbAcc<NOCC> a;
    for (int s = 0; s < k_sites; ++s) {
      const int i = si[s], j = sj[s], k = sk[s];
      auto rd = [&](int c, int jj) -> int {
        const int pb = T.cl_pb[c * 3 + jj];
        const int *du = T.cl_du + c * 9 + jj * 3;
        const int site = pb * n_uc + C.index(i + du[0], j + du[1], k + du[2]);
        int v = occ[site];
        for (int q = 0; q < s; ++q)
          if (ov_site[q] == site) v = ov_val[q];
        return v;
      };
      orbit_site<NOCC>(T, sb[s], g, soi[s], sof[s], T.cl_lut, T.lut, rd, a);
    }
    orbit_fold<NOCC>(T, g, a, T.w_hi, T.w_lo, d);
    if (dc_out) {
      const int base = T.orb_func_base[g];
      if constexpr (NOCC == 2) {
        dc_out[base] = a.c;
      } else {
        for (int fl = 0; fl < T.orb_n_funcs[g]; ++fl)
          dc_out[base + fl] =
              (int)((a.p >> (8 * fl)) & 255ull) - (int)((a.m >> (8 * fl)) & 255ull);
      }
    }
  }
  dE[e] = ((double)d.s + (double)d.e) - mu_term;
}

// ------------------------------------------------------------ replay
// std::uniform_int_distribution<long>(0, max) over a 64-bit engine, as
// libstdc++ implements it: Lemire's nearly divisionless method (Lemire,
// "Fast Random Integer Generation in an Interval", ACM TOMACS 2019) with a
// 128-bit product. The oracle tests pin this against the host library.
struct MtState {
  unsigned long long mt[MT_N];
  int idx;
  unsigned long long draws;
};

__device__ inline unsigned long long mt_draw(MtState &s) {
  if (s.idx >= MT_N) {
    for (int i = 0; i < MT_N; ++i) {
      s.mt[i] = mt_next_word(s.mt[i], s.mt[(i + 1) % MT_N], s.mt[(i + MT_M) % MT_N]);
    }
    s.idx = 0;
  }
  s.draws++;
  return mt_temper(s.mt[s.idx++]);
}

__device__ inline long long std_random_int(MtState &s, long long maxv) {
  const unsigned long long range = (unsigned long long)maxv + 1ull;  // 0 means 2^64
  unsigned long long x = mt_draw(s);
  if (range == 0ull) return (long long)x;
  unsigned long long lo = x * range, hi = __umul64hi(x, range);
  if (lo < range) {
    const unsigned long long threshold = (0ull - range) % range;
    while (lo < threshold) {
      x = mt_draw(s);
      lo = x * range;
      hi = __umul64hi(x, range);
    }
  }
  return (long long)hi;
}

// std::uniform_real_distribution<double>(0, 1) over a 64-bit engine:
// generate_canonical<double, 53> takes one draw, x / 2^64 rounded to double,
// with 1.0 mapped to the largest double below 1.
__device__ inline double std_random_real(MtState &s) {
  const unsigned long long x = mt_draw(s);
  double r = __ull2double_rn(x) * 5.42101086242752217e-20;  // 2^-64
  if (r >= 1.0) r = 0.99999999999999988898;                 // nextafter(1, 0)
  return r;
}

template <int NOCC>
__global__ void k_replay(const __grid_constant__ CeTables T, ReplayParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  MtState &mt = *reinterpret_cast<MtState *>(smem);
  int8_t *occ = reinterpret_cast<int8_t *>(smem + sizeof(MtState));
  const int N = P.n_sites;
  int *pos = reinterpret_cast<int *>(smem + sizeof(MtState) + ((N + 15) & ~15));
  int *lists = pos + N;  // NOCC lists of capacity N
  __shared__ int list_size[NOCC];
  __shared__ long long ev_site[2];
  __shared__ int ev_new[2], ev_n, ev_stop;
  const int lane = threadIdx.x;
  const Cells C{P.L[0], P.L[1], P.L[2], P.tw[0], P.tw[1], P.tw[2]};
  const int L0 = C.L0, L1 = C.L1;
  const int n_uc = L0 * L1 * C.L2;

  for (int l = lane; l < N; l += 32) occ[l] = P.occ[l];
  __syncwarp();
  if (lane == 0) {
    mt.mt[0] = P.mt_seed;
    for (int i = 1; i < MT_N; ++i)
      mt.mt[i] = 6364136223846793005ull * (mt.mt[i - 1] ^ (mt.mt[i - 1] >> 62)) + (unsigned long long)i;
    mt.idx = MT_N;
    mt.draws = 0;
    for (int a = 0; a < NOCC; ++a) list_size[a] = 0;
    for (int l = 0; l < N; ++l) {
      const int a = occ[l];
      pos[l] = list_size[a];
      lists[a * N + list_size[a]] = l;
      list_size[a]++;
    }
    ev_stop = 0;
  }
  __syncwarp();
  long long n_acc = 0;
  const double beta = P.beta;
  for (long long step = 0; step < P.n_steps; ++step) {
    // ---- propose (lane 0): swap type by integer count, then candidates
    if (lane == 0) {
      long long cum[NOCC * NOCC];
      int ta[NOCC * NOCC], tb[NOCC * NOCC];
      int nt = 0;
      long long tsum = 0;
      for (int a = 0; a < NOCC; ++a)
        for (int bb = 0; bb < NOCC; ++bb) {
          if (a == bb) continue;
          if (P.ensemble == 1 && bb < a) continue;
          long long w = list_size[a];
          if (P.ensemble == 1) w *= list_size[bb];
          tsum += w;
          cum[nt] = tsum;
          ta[nt] = a;
          tb[nt] = bb;
          nt++;
        }
      if (tsum == 0) {
        ev_stop = 1;
      } else {
        const long long cnt = std_random_int(mt, tsum - 1);
        int it = 0;
        while (cum[it] <= cnt) ++it;  // upper_bound
        const int a = ta[it], bb = tb[it];
        if (P.ensemble == 1) {
          const long long ia = std_random_int(mt, list_size[a] - 1);
          const long long ib = std_random_int(mt, list_size[bb] - 1);
          ev_site[0] = lists[a * N + ia];
          ev_site[1] = lists[bb * N + ib];
          ev_new[0] = bb;
          ev_new[1] = a;
          ev_n = 2;
        } else {
          const long long ia = std_random_int(mt, list_size[a] - 1);
          ev_site[0] = lists[a * N + ia];
          ev_new[0] = bb;
          ev_n = 1;
        }
      }
    }
    __syncwarp();
    if (ev_stop) break;
    // ---- delta correlations: lanes split each centre's flower clusters;
    // one orbit at a time, both changed sites, folded into the float-float
    // energy change in function order. The first change is applied before
    // any cluster is read: a site's own flower never contains the site, so
    // site 0 sees the original state and site 1 sees site 0 changed (the
    // reference's sequential semantics).
    const int n = ev_n;
    int saved = 0;
    if (n > 1) {
      if (lane == 0) {
        saved = occ[ev_site[0]];
        occ[ev_site[0]] = (int8_t)ev_new[0];
      }
      __syncwarp();
    }
    int sb[2], si[2], sj[2], sk[2], soi[2], sof[2];
    for (int s = 0; s < n; ++s) {
      const int l = (int)ev_site[s];
      const int b = l / n_uc, uc = l - b * n_uc;
      sb[s] = b;
      si[s] = uc % L0;
      sj[s] = (uc / L0) % L1;
      sk[s] = uc / (L0 * L1);
      soi[s] = (s == 0 && n > 1) ? __shfl_sync(0xffffffffu, saved, 0) : (int)occ[l];
      sof[s] = ev_new[s];
    }
    FF d{0.f, 0.f};
    for (int g = 0; g < T.n_orbits; ++g) {
      const int size = T.orb_size[g];
      int cnt_tot = 0;
      unsigned long long p_tot = 0ull, m_tot = 0ull;
      for (int s = 0; s < n; ++s) {
        const int b = sb[s], i = si[s], j = sj[s], k = sk[s], o_i = soi[s], o_f = sof[s];
        const int c0 = T.fl_begin[b][g], c1 = T.fl_begin[b][g + 1];
        int cnt = 0;
        unsigned long long pp = 0ull, mm = 0ull;
        for (int c = c0 + lane; c < c1; c += 32) {
          int code = 0, mul = NOCC - 1, prod = 1;
          bool ok = true;
          for (int q = 0; q < size - 1; ++q) {
            const int pb = T.cl_pb[c * 3 + q];
            const int *du = T.cl_du + c * 9 + q * 3;
            const int site = pb * n_uc + C.index(i + du[0], j + du[1], k + du[2]);
            const int v = occ[site];
            prod &= v;
            ok = ok && (v != 0);
            code += (v - 1) * mul;
            mul *= (NOCC - 1);
          }
          if constexpr (NOCC == 2) {
            cnt += prod;
          } else {
            if (ok) {
              const int base = T.cl_lut[c] + code;
              if (o_f) pp += 1ull << (8 * T.lut[base + o_f - 1]);
              if (o_i) mm += 1ull << (8 * T.lut[base + o_i - 1]);
            }
          }
        }
        if constexpr (NOCC == 2) {
          for (int off = 16; off; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
          cnt_tot += (o_f - o_i) * cnt;
        } else {
          for (int off = 16; off; off >>= 1) {
            pp += __shfl_xor_sync(0xffffffffu, pp, off);
            mm += __shfl_xor_sync(0xffffffffu, mm, off);
          }
          p_tot += pp;
          m_tot += mm;
        }
      }
      OrbAcc<NOCC> a;
      if constexpr (NOCC == 2) {
        a.c = cnt_tot;
      } else {
        a.p = p_tot;
        a.m = m_tot;
      }
      orbit_fold<NOCC>(T, g, a, T.w_hi, T.w_lo, d);
    }
    __syncwarp();
    // ---- dE, acceptance and application (lane 0)
    if (lane == 0) {
      if (n > 1) occ[ev_site[0]] = (int8_t)saved;
      double de = (double)d.s + (double)d.e;
      if (P.ensemble == 0) de -= P.dmu[occ[ev_site[0]] * NOCC + ev_new[0]];
      bool accept = true;
      if (!(de < 0.0)) accept = std_random_real(mt) < exp(-de * beta);
      if (P.accept_seq) P.accept_seq[step] = accept ? 1 : 0;
      if (P.de_seq) P.de_seq[step] = de;
      if (P.site_seq) {
        P.site_seq[2 * step] = ev_site[0];
        P.site_seq[2 * step + 1] = (n > 1) ? ev_site[1] : -1;
      }
      if (accept) {
        ++n_acc;
        for (int s = 0; s < n; ++s) {
          const int l = (int)ev_site[s];
          const int from = occ[l], to = ev_new[s];
          int *la = lists + from * N;
          const int p = pos[l];
          const int last = la[list_size[from] - 1];
          la[p] = last;
          pos[last] = p;
          list_size[from]--;
          pos[l] = list_size[to];
          lists[to * N + list_size[to]] = l;
          list_size[to]++;
          occ[l] = (int8_t)to;
        }
      }
    }
    __syncwarp();
  }
  __syncwarp();
  for (int l = lane; l < N; l += 32) P.occ[l] = occ[l];
  if (lane == 0) {
    P.result[0] = n_acc;
    P.result[1] = (long long)mt.draws;
    P.result[2] = ev_stop;
  }
}

// ------------------------------------------------------------ parallel sweep
// A pass = n_pair_sweeps sweeps of pair swaps inside each colour class plus
// n_local_sweeps sweeps of swaps with a nearest neighbour (canonical), or one
// sweep of flips over every class (semi-grand canonical). Each sweep visits
// the classes in a random order drawn per pass.
constexpr uint32_t TAG_SITE = 0x1u, TAG_SCHED = 0x2u;
constexpr int MAX_SWEEPS = 8;

struct SweepSmem {
  // carved from dynamic shared memory; offsets in bytes
  int occ, cl_off, lutoff, lut, whi, wlo, dmu, ax, sched, red, clist, wkept, stats, desc, initq,
      bar, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline int clist_capacity(int L0, int L1, int L2) {
  return (L0 * L1 * L2) / 8 + 32;
}

// pitch > 0: fixed x/y pitch of the generated evaluator; 0: L + 2 reach
__host__ __device__ inline void sweep_layout(const CeTables &T, int L0, int L1, int L2,
                                             int n_sub_max, int pitch, SweepSmem &s) {
  const int R = T.reach;
  const int W = pitch > 0 ? pitch : L0 + 2 * R, H = pitch > 0 ? pitch : L1 + 2 * R;
  const int V = W * H * (L2 + 2 * R);
  const bool tables = (pitch <= 0);
  int o = 0;
  s.occ = o;
  o += align16(T.n_sublat * V);
  s.cl_off = o;
  o += tables ? align16(T.n_fl * 3 * 4) : 0;
  s.lutoff = o;
  o += tables ? align16(T.n_fl * 4) : 0;
  s.lut = o;  // pitch -2: per-cluster f32 remainder weights instead
  o += tables ? align16(pitch == -2 ? T.n_fl * 4 : T.n_fl * (T.n_sf * T.n_sf * T.n_sf * T.n_sf)) : 0;
  s.whi = o;
  o += align16(T.n_funcs * 4);
  s.wlo = o;
  o += align16(T.n_funcs * 4);
  s.dmu = o;  // hi[16], lo[16] floats
  o += 128;
  s.ax = o;  // per axis: begin[MAX_COLOURS], cnt[MAX_COLOURS], coord[MAX_L]
  o += align16(3 * (2 * MAX_COLOURS + MAX_L) * 4);
  s.sched = o;  // key[n], par[n], order[n] (u32 each), n = sub-steps per pass
  o += align16(3 * n_sub_max * 4);
  s.red = o;  // block reduction scratch: 32 warps x 16 slots of 8 bytes
  o += 32 * 16 * 8;
  s.stats = o;  // the replica's running statistics, resident for the launch
  o += align16((int)sizeof(ReplicaStats));
  // [clist, bar): unused while the replica is staged in and written back,
  // so the bulk copies go through it
  s.clist = o;  // kept canonical candidates (u16), two buffers: a class holds <= n_uc / 8 sites
  o += 2 * align16(2 * clist_capacity(L0, L1, L2));
  s.wkept = o;  // kept candidates per warp, two buffers
  o += 2 * 32 * 4;
  s.desc = o;  // decoded sub-steps of the current pass
  o += n_sub_max * 80;
  s.initq = o;  // per-warp queues of occupied sites (initial energy)
  o += 32 * 96 * 4;
  s.bar = o;  // two mbarriers of the staging copies
  o += 16;
  s.total = o;
}

inline int sweep_smem_bytes_impl(const CeTables &T, int L0, int L1, int L2, int n_sub,
                                 int pitch) {
  SweepSmem s;
  sweep_layout(T, L0, L1, L2, n_sub, pitch, s);
  return s.total;
}

// ------------------------------------------------------------ bulk copies
// One-dimensional TMA bulk copies (cp.async.bulk) between global and shared
// memory, completing on an mbarrier (loads) or a bulk group (stores). Both
// addresses must be 16-byte aligned and the size a multiple of 16 bytes.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Bounded wait for the completion of the mbarrier phase with this parity.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int max_iter) {
  const uint32_t a = smem_u32(bar);
  for (int i = 0; i < max_iter; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_store(void *dst_gmem, const void *src_smem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem),
               "r"(smem_u32(src_smem)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// floor(n / d) for a block-uniform divisor d >= 1 and numerators n >= 0 with
// n * d < 2^32: umulhi(n, m) with m = floor((2^32 - 1) / d) + 1 (= ceil(2^32 / d),
// or 2^32 / d for powers of two); exact because the rounding error of m is
// below d (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994).
struct FastDiv {
  int d;
  uint32_t m;
  __host__ __device__ __forceinline__ static uint32_t magic(int dd) {
    return dd > 1 ? 0xFFFFFFFFu / (uint32_t)dd + 1u : 0u;
  }
  __device__ __forceinline__ explicit FastDiv(int dd) : d(dd), m(magic(dd)) {}
  __device__ __forceinline__ FastDiv(int dd, uint32_t mm) : d(dd), m(mm) {}
  __device__ __forceinline__ int div(int n) const {
    return d > 1 ? (int)__umulhi((uint32_t)n, m) : n;
  }
};

struct Geo {
  int L0, L1, L2, R, W, H, V;
  __device__ __forceinline__ int addr(int b, int x, int y, int z) const {
    return b * V + (x + R) + W * ((y + R) + H * (z + R));
  }
};

// Linear site index l = b n_uc + x + L0 (y + L1 z) -> (b, x, y, z) without
// hardware division (n_uc L0 < 2^32 for every supercell that fits in shared
// memory; at most 4 sublattices).
struct SiteIndex {
  int n_uc, L0, L1;
  FastDiv f0, f1;
  __device__ __forceinline__ SiteIndex(int n, int l0, int l1)
      : n_uc(n), L0(l0), L1(l1), f0(l0), f1(l1) {}
  __device__ __forceinline__ void operator()(int l, int &b, int &x, int &y, int &z) const {
    b = (l >= n_uc) + (l >= 2 * n_uc) + (l >= 3 * n_uc);
    const int uc = l - b * n_uc;
    const int t = f0.div(uc);
    x = uc - t * L0;
    z = f1.div(t);
    y = t - z * L1;
  }
};

// Write occupant v to core site (b,x,y,z) and all of its periodic halo images.
__device__ __forceinline__ void put_site(int8_t *occ, const Geo &G, int b, int x, int y, int z,
                                         int8_t v) {
  const int base = G.addr(b, x, y, z);
  occ[base] = v;
  // periodic images: along each axis at most one, L cells away
  const int ox = x < G.R ? G.L0 : (x >= G.L0 - G.R ? -G.L0 : 0);
  const int oy = (y < G.R ? G.L1 : (y >= G.L1 - G.R ? -G.L1 : 0)) * G.W;
  const int oz = (z < G.R ? G.L2 : (z >= G.L2 - G.R ? -G.L2 : 0)) * (G.W * G.H);
  if ((ox | oy | oz) == 0) return;
  if (ox) occ[base + ox] = v;
  if (oy) occ[base + oy] = v;
  if (oz) occ[base + oz] = v;
  if (ox && oy) occ[base + ox + oy] = v;
  if (ox && oz) occ[base + ox + oz] = v;
  if (oy && oz) occ[base + oy + oz] = v;
  if (ox && oy && oz) occ[base + ox + oy + oz] = v;
}

// Write occupant v to core site (b,x,y,z) and every periodic image of it in
// the halo'd box of a supercell in Hermite normal form C (twisted images: a
// step of L0 along x shifts y and z by t10, t20; a step of L1 along y shifts
// z by t21). Each box cell [-R, L + R) per axis is an image of exactly one
// core cell, so the halo holds what the box's gathers read, for boxes thinner
// than the reach too.
__device__ __forceinline__ void put_site_cells(int8_t *occ, const Geo &G, const Cells &C, int b,
                                               int x, int y, int z, int8_t v) {
  const int R = G.R;
  for (int xi = x - floor_div(x + R, C.L0) * C.L0; xi < C.L0 + R; xi += C.L0) {
    const int i = (xi - x) / C.L0;  // exact
    const int yb = y + i * C.t10, zb = z + i * C.t20;
    for (int yj = yb - floor_div(yb + R, C.L1) * C.L1; yj < C.L1 + R; yj += C.L1) {
      const int zc = zb + ((yj - yb) / C.L1) * C.t21;
      for (int zk = zc - floor_div(zc + R, C.L2) * C.L2; zk < C.L2 + R; zk += C.L2)
        occ[G.addr(b, xi, yj, zk)] = v;
    }
  }
}

// Energy change of a sweep proposal (f32, minus the chemical potential term
// mu_hi + mu_lo). Binary systems: exact int32 sum of wq * dC scaled by the
// power-of-two quantum, plus the f32 remainder terms (one FMA chain); other
// systems: float-float dot, also returned in d for the FP64 bookkeeping.
template <int NOCC>
__device__ __forceinline__ float sweep_de(const CeTables &T, const Acc<NOCC> &acc,
                                          const float *whi, const float *wlo, float mu_hi,
                                          float mu_lo, FF &d) {
  if constexpr (NOCC == 2) {
    int n = 0;
    float r = 0.f;
#pragma unroll
    for (int g = 0; g < MAX_ORBITS; ++g) {
      n += T.wq[g] * acc.c[g];
      r = FFMA(T.wr[g], (float)acc.c[g], r);
    }
    d = FF{0.f, 0.f};
    return FADD(FADD(FFMA((float)n, T.wq_scale, r), -mu_hi), -mu_lo);
  } else {
    d = acc_dot<NOCC>(T, acc, whi, wlo);
    ff_add_ff(d, -mu_hi, -mu_lo);
    return FADD(d.s, d.e);
  }
}

// Warp-cooperative energy change of one binary site change (PITCH -2):
// the lanes split the centre's flower clusters (points, pairs, triplets,
// quadruplets: seg[0..4] bounds in the size-sorted flower); every cluster
// carries its orbit's weight split w = A q + r (A integer, |r| <= q/2), so a
// lane sums A * product exactly in int32 and r * product in an f32 FMA chain.
// Returns the lane's partial sums (the caller reduces over the warp).
// Partner offsets are stored partner-major (off0[c], off1[c], off2[c] at
// stride n_fl), so each warp-wide load reads 32 consecutive words: one
// shared-memory wavefront instead of three for a 12-byte record per cluster.
__device__ __forceinline__ void coop_site(const int8_t *__restrict__ occ, int ad,
                                          const int *__restrict__ cl_off, int n_fl,
                                          const int *__restrict__ cw_a,
                                          const float *__restrict__ cw_r, const int *seg,
                                          int lane, int &n, float &r) {
  const int *off0 = cl_off, *off1 = cl_off + n_fl, *off2 = cl_off + 2 * n_fl;
  for (int c = seg[0] + lane; c < seg[1]; c += 32) {
    n += cw_a[c];
    r = FADD(r, cw_r[c]);
  }
#pragma unroll 2
  for (int c = seg[1] + lane; c < seg[2]; c += 32) {
    const int v = occ[ad + off0[c]];
    n += v * cw_a[c];
    r = FFMA(cw_r[c], (float)v, r);
  }
#pragma unroll 4
  for (int c = seg[2] + lane; c < seg[3]; c += 32) {
    const int v = occ[ad + off0[c]] & occ[ad + off1[c]];
    n += v * cw_a[c];
    r = FFMA(cw_r[c], (float)v, r);
  }
#pragma unroll 4
  for (int c = seg[3] + lane; c < seg[4]; c += 32) {
    const int v = occ[ad + off0[c]] & occ[ad + off1[c]] & occ[ad + off2[c]];
    n += v * cw_a[c];
    r = FFMA(cw_r[c], (float)v, r);
  }
}

// The same with 16-bit records (batches whose partner offsets and integer
// weights fit in int16): pk0[c] = off0 | off1 << 16, pk1[c] = off2 | A << 16,
// one word fewer per triplet and two fewer per quadruplet than the 32-bit
// records (the kernel is bound by shared-memory load wavefronts).
__device__ __forceinline__ int lo16(int w) { return (int)(int16_t)(w & 0xFFFF); }
__device__ __forceinline__ int hi16(int w) { return w >> 16; }  // arithmetic shift
__device__ __forceinline__ int pack16(int lo, int hi) {
  return (int)(((unsigned)lo & 0xFFFFu) | ((unsigned)hi << 16));
}

__device__ __forceinline__ void coop_site16(const int8_t *__restrict__ occ, int ad,
                                            const int *__restrict__ pk0,
                                            const int *__restrict__ pk1,
                                            const float *__restrict__ cw_r, const int *seg,
                                            int lane, int &n, float &r) {
  for (int c = seg[0] + lane; c < seg[1]; c += 32) {
    n += hi16(pk1[c]);
    r = FADD(r, cw_r[c]);
  }
#pragma unroll 2
  for (int c = seg[1] + lane; c < seg[2]; c += 32) {
    const int v = occ[ad + lo16(pk0[c])];
    n += v * hi16(pk1[c]);
    r = FFMA(cw_r[c], (float)v, r);
  }
#pragma unroll 4
  for (int c = seg[2] + lane; c < seg[3]; c += 32) {
    const int w0 = pk0[c];
    const int v = occ[ad + lo16(w0)] & occ[ad + hi16(w0)];
    n += v * hi16(pk1[c]);
    r = FFMA(cw_r[c], (float)v, r);
  }
#pragma unroll 4
  for (int c = seg[3] + lane; c < seg[4]; c += 32) {
    const int w0 = pk0[c], w1 = pk1[c];
    const int v = occ[ad + lo16(w0)] & occ[ad + hi16(w0)] & occ[ad + lo16(w1)];
    n += v * hi16(w1);
    r = FFMA(cw_r[c], (float)v, r);
  }
}

// Sum over the warp (butterfly: every lane ends with the same bits, float
// addition being commutative).
__device__ __forceinline__ void warp_sum_nr(int &n, float &r) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, off);
    r = FADD(r, __shfl_xor_sync(0xffffffffu, r, off));
  }
}

__device__ __forceinline__ bool accept_de(float de, float beta_f, float u) {
  if (de < 0.f) return true;
  return u < cem_expf_neg(FMUL(-beta_f, de));
}

// One sub-step of a pass, decoded once per pass by the thread that ranks its
// class (so the serial sub-step loop only loads it).
struct SubDesc {
  int cb, mode, n, chunk;  // mode: 0 flips, 1 pairs inside the class, 2 neighbour swaps
  int d0, d1, d2, bb;      // class extent per axis; sublattice of the partner site
  int cxo, cyo, czo, g0;   // class coordinate lists; candidate grid extent along x
  int g1, m0, m1, mpm;     // candidate grid extent along y; FastDiv magics (g0, g1, pm)
  int par, du0, du1, du2;  // packed sub-step parameters; neighbour displacement
};
static_assert(sizeof(SubDesc) == 80, "SubDesc is five 16-byte words");
static_assert(sizeof(ReplicaStats) % 8 == 0, "ReplicaStats is copied as 8-byte words");

// Small counters indexed by a run-time value, kept in registers (unrolled
// selects rather than a local-memory array).
template <int N>
struct RegCounts {
  int v[N];
  __device__ __forceinline__ RegCounts() {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = 0;
  }
  __device__ __forceinline__ void add(int i, int d) {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] += (k == i) ? d : 0;
  }
};

// Per-pass sample values of a replica: param composition per unit cell x,
// potential energy per unit cell ep = E_f / n_uc - mu . x, formation energy per
// unit cell ef. Explicitly rounded double operations, so every kernel that
// samples gets the same bits.
template <int NOCC>
__device__ __forceinline__ void sample_values(const double *RT, const double *mu,
                                              const long long *nspec, int n_sites, int n_uc,
                                              double energy, double x[3], double &ef, double &ep) {
  double mux = 0.0;
  for (int k = 0; k < NOCC - 1; ++k) {
    double t = 0.0;
    for (int a = 0; a < NOCC; ++a) {
      const double cnt = (double)nspec[a] - (a == 0 ? (double)n_sites : 0.0);
      t = __dadd_rn(t, __dmul_rn(RT[k * NOCC + a], cnt));
    }
    x[k] = __ddiv_rn(t, (double)n_uc);
    mux = __dadd_rn(mux, __dmul_rn(mu[k], x[k]));
  }
  ef = __ddiv_rn(energy, (double)n_uc);
  ep = __dsub_rn(ef, mux);
}

// One of the four simple-cubic sublattices of FCC (L1_2 order parameter), for
// a site in primitive-cell coordinates.
__device__ __forceinline__ int sc_sublattice(int x, int y, int z) {
  return ((y + z) & 1) | (((x + z) & 1) << 1);
}

// Parameters of one sub-step, from its Philox draw r: pairs inside the
// class (axis, shift m, rotation) or swaps with a neighbour (parity pattern,
// neighbour index, rotations); 0xFFFFFFFF = no pair along any axis.
__device__ __forceinline__ uint32_t sched_param(const U4 &r, int ensemble, int sweep,
                                                int n_pair_sw, const int dims[3], int nnb) {
  uint32_t par = 0;
  if (ensemble == 1 && sweep < n_pair_sw) {
    int a = r.y % 3, tries = 0;
    while (dims[a] < 2 && tries < 3) {
      a = (a + 1) % 3;
      ++tries;
    }
    if (dims[a] >= 2) {
      const int m = 1 + (int)(r.z % (uint32_t)(dims[a] / 2));
      const int rot = (int)(r.w % (uint32_t)dims[a]);
      par = (uint32_t)a | ((uint32_t)m << 2) | ((uint32_t)rot << 10);
    } else {
      par = 0xFFFFFFFFu;
    }
  } else if (ensemble == 1) {
    const int dlt = (int)(r.y % (uint32_t)(nnb > 0 ? nnb : 1));
    const uint32_t parity = r.z & 7u;
    uint32_t rots = 0;
    for (int a = 0; a < 3; ++a) {
      const uint32_t ra = (r.w >> (8 * a)) & 255u;
      rots |= (uint32_t)(ra % (uint32_t)dims[a]) << (7 * a);
    }
    par = parity | ((uint32_t)dlt << 3) | (rots << 7);
  }
  return par;
}

// Site evaluation policy: PITCH > 0 uses the generated binary FCC evaluator
// (compile-time neighbour offsets); PITCH == 0 walks the run-time tables with
// register accumulators for up to MAX_ORBITS orbits; PITCH == -1 walks them
// one orbit at a time (any number of orbits).
template <int NOCC, int PITCH>
struct SiteEval {
  const CeTables *T;
  const int *cl_off;
  const int *lutoff;
  const uint8_t *lut;
  __device__ __forceinline__ void add(int b, int o_i, int o_f, const int8_t *occ, int ad,
                                      Acc<NOCC> &acc) const {
    if constexpr (PITCH > 0) {
      int n[gen_fcc::N_ORBITS];
      gen_fcc::counts<PITCH>(occ + ad, n);
      const int d = o_f - o_i;
#pragma unroll
      for (int g = 0; g < gen_fcc::N_ORBITS; ++g) acc.c[g] += d * n[g];
    } else {
      auto rd = [&](int cl, int j) -> int { return occ[ad + cl_off[cl * 3 + j]]; };
      accumulate_site<NOCC>(*T, b, o_i, o_f, lutoff, lut, rd, acc);
    }
  }
  __device__ __forceinline__ void orbit(int b, int g, int o_i, int o_f, const int8_t *occ, int ad,
                                        OrbAcc<NOCC> &a) const {
    auto rd = [&](int cl, int j) -> int { return occ[ad + cl_off[cl * 3 + j]]; };
    orbit_site<NOCC>(*T, b, g, o_i, o_f, lutoff, lut, rd, a);
  }
};

// running energy as an FP64 sum of accepted energy changes (any system)
struct EnergyAccF64 {
  double de = 0.0;
  template <class A>
  __device__ __forceinline__ void add(const A &, const FF &d, double extra) {
    de += (double)d.s + (double)d.e + extra;
  }
};

// running energy bookkeeping: exact integer delta correlations per orbit for
// binary systems, FP64 sums of dE otherwise
template <int NOCC>
struct EnergyAcc {
  double de = 0.0;
  __device__ __forceinline__ void add(const Acc<NOCC> &, const FF &d, double extra) {
    de += (double)d.s + (double)d.e + extra;
  }
};
template <>
struct EnergyAcc<2> {
  int dc[MAX_ORBITS] = {0, 0, 0, 0, 0, 0, 0, 0};
  __device__ __forceinline__ void add(const Acc<2> &a, const FF &, double) {
#pragma unroll
    for (int g = 0; g < MAX_ORBITS; ++g) dc[g] += a.c[g];
  }
};

// Candidate pairs of a canonical sub-step: pairs inside the class along axis
// pa at class distance pm, rotated by prot (mode 1), or every other class
// coordinate (parity bits, rotations r0..r2) paired with the neighbour
// (bb, du) (mode 2). Candidate q indexes a g0 x g1 x g2 grid.
struct PairGeom {
  const int *cx, *cy, *cz;
  int cb, bb, d0, d1, d2, pa, pm, prot, pna, parity, r0, r1, r2, du0, du1, du2;
  bool local;
  FastDiv fe0, fe1, fpm;
  __device__ __forceinline__ PairGeom(const SubDesc &D, int *const *ax_coord)
      : cx(ax_coord[0] + D.cxo), cy(ax_coord[1] + D.cyo), cz(ax_coord[2] + D.czo), cb(D.cb),
        bb(D.bb), d0(D.d0), d1(D.d1), d2(D.d2), pa(D.par & 3), pm(((uint32_t)D.par >> 2) & 255),
        prot((int)((uint32_t)D.par >> 10)), pna(0), parity(D.par & 7),
        r0((int)(((uint32_t)D.par >> 7) & 127)), r1((int)(((uint32_t)D.par >> 14) & 127)),
        r2((int)(((uint32_t)D.par >> 21) & 127)), du0(D.du0), du1(D.du1), du2(D.du2),
        local(D.mode == 2), fe0(D.g0, (uint32_t)D.m0), fe1(D.g1, (uint32_t)D.m1),
        fpm(pm, (uint32_t)D.mpm) {
    pna = pa == 0 ? d0 : (pa == 1 ? d1 : d2);
  }
  __device__ __forceinline__ void sites(int q, const Geo &G, int &xa, int &ya, int &za, int &xb,
                                        int &yb, int &zb) const {
    auto wrap_lt2 = [](int v, int L) { return v >= L ? v - L : v; };  // v < 2L
    const int t = fe0.div(q), i2 = fe1.div(t);
    const int i0 = q - t * fe0.d, i1 = t - i2 * fe1.d;
    if (!local) {
      const int jj = pa == 0 ? i0 : (pa == 1 ? i1 : i2);
      const int jq = fpm.div(jj);
      const int u = 2 * pm * jq + (jj - jq * pm);
      const int ja = wrap_lt2(u + prot, pna), jb = wrap_lt2(u + pm + prot, pna);
      xa = cx[pa == 0 ? ja : i0];
      xb = cx[pa == 0 ? jb : i0];
      ya = cy[pa == 1 ? ja : i1];
      yb = cy[pa == 1 ? jb : i1];
      za = cz[pa == 2 ? ja : i2];
      zb = cz[pa == 2 ? jb : i2];
    } else {
      xa = cx[d0 >= 2 ? wrap_lt2(r0 + (parity & 1) + 2 * i0, d0) : 0];
      ya = cy[d1 >= 2 ? wrap_lt2(r1 + ((parity >> 1) & 1) + 2 * i1, d1) : 0];
      za = cz[d2 >= 2 ? wrap_lt2(r2 + ((parity >> 2) & 1) + 2 * i2, d2) : 0];
      xb = wrapc(xa + du0, G.L0);
      yb = wrapc(ya + du1, G.L1);
      zb = wrapc(za + du2, G.L2);
    }
  }
};

// Phase A of a canonical sub-step: warp w scans candidates [v chunk,
// (v + 1) chunk) of its virtual warp v and keeps, in order, those whose two
// occupants differ (the only proposals) in cl[w chunk ...]; wk[w] = number
// kept.
__device__ __forceinline__ void compact_pairs(const PairGeom &pg, const Geo &G, const int8_t *occ,
                                              int n, int chunk, int warp, int vwarp, int lane,
                                              uint16_t *cl, int *wk) {
  // scan range of virtual warp vwarp (= warp, or rank x warps + warp when a
  // cluster of CTAs shares the sub-step); kept candidates stored from
  // cl[warp chunk]
  const int q_begin = vwarp * chunk;
  const int q_end = min(n, q_begin + chunk);
  const int s_begin = warp * chunk;
  int kept = 0;
  for (int q0 = q_begin; q0 < q_end; q0 += 32) {
    const int q = q0 + lane;
    bool act = false;
    if (q < q_end) {
      int xa, ya, za, xb, yb, zb;
      pg.sites(q, G, xa, ya, za, xb, yb, zb);
      act = occ[G.addr(pg.cb, xa, ya, za)] != occ[G.addr(pg.bb, xb, yb, zb)];
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (act) cl[s_begin + kept + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
    kept += __popc(m);
  }
  if (lane == 0) wk[warp] = kept;
}

// Replica staging through a shared-memory buffer of cap bytes (a multiple
// of 16): each round, one thread issues bulk copies of up to 32 KB for as
// much of the replica as fits, all completing on one mbarrier; then every
// thread scatters the round into the halo'd layout. Returns 0 when every
// round completed (the mbarrier is then invalidated, so its word can be
// reused as ordinary shared memory); STAGE_TIMEOUT when a round did not
// complete within the wait limit but a second bounded wait saw its copies
// land (nothing in flight); STAGE_IN_FLIGHT when that second wait ran out
// too, so copies may still be writing into this CTA's shared memory.
constexpr int STAGE_TIMEOUT = 5, STAGE_IN_FLIGHT = 6;
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
static __device__ __noinline__ int stage_replica_bulk(const int8_t *gocc, int n_sites, int8_t *occ,
                                                      const Geo &G, const SiteIndex &site_of,
                                                      uint8_t *buf, int cap, uint64_t *bar) {
  const int tid = threadIdx.x, nth = blockDim.x;
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  int round = 0;
  for (int off0 = 0; off0 < n_sites; off0 += cap, ++round) {
    const int bytes = min(cap, n_sites - off0);
    if (tid == 0) {
      if (round) fence_proxy_async_smem();
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                   "r"((uint32_t)bytes)
                   : "memory");
      for (int o = 0; o < bytes; o += 32768) {
        const uint32_t piece = (uint32_t)min(32768, bytes - o);
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                "r"(smem_u32(buf + o)),
            "l"(gocc + off0 + o), "r"(piece), "r"(smem_u32(bar))
            : "memory");
      }
    }
    const bool ok = mbar_wait(bar, (uint32_t)(round & 1), 1 << 22);
    if (__syncthreads_or(!ok)) {
      bool landed = true;
      if (tid == 0) landed = mbar_wait(bar, (uint32_t)(round & 1), 1 << 22);  // let the copies land
      return __syncthreads_or(!landed) ? STAGE_IN_FLIGHT : STAGE_TIMEOUT;
    }
    for (int i = tid; i < bytes; i += nth) {
      int b, x, y, z;
      site_of(off0 + i, b, x, y, z);
      put_site(occ, G, b, x, y, z, (int8_t)buf[i]);
    }
    __syncthreads();
  }
  if (tid == 0) mbar_inval(bar);
  __syncthreads();
  return 0;
}

// Occupations back to global memory: each round gathers as much of the
// replica as fits in the buffer from the halo'd layout, then one thread
// issues bulk stores of up to 32 KB and waits until they have read the
// buffer.
static __device__ __noinline__ void writeback_replica_bulk(int8_t *gout, int n_sites,
                                                           const int8_t *occ, const Geo &G,
                                                           const SiteIndex &site_of, uint8_t *buf,
                                                           int cap) {
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int off0 = 0; off0 < n_sites; off0 += cap) {
    const int bytes = min(cap, n_sites - off0);
    for (int i = tid; i < bytes; i += nth) {
      int b, x, y, z;
      site_of(off0 + i, b, x, y, z);
      buf[i] = (uint8_t)occ[G.addr(b, x, y, z)];
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      for (int o = 0; o < bytes; o += 32768)
        bulk_store(gout + off0 + o, buf + o, (uint32_t)min(32768, bytes - o));
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
    __syncthreads();
  }
  if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Exact initial statistics of a binary replica staged in shared memory,
// written to S: count_g = number of clusters of orbit g with every site
// occupant 1. Kept out of line, so that the sweep loop's register allocation
// does not depend on it.
template <int PITCH, int NW>
__device__ __noinline__ void init_binary_stats(const CeTables &T, const int8_t *occ,
                                               const Geo &G, const SiteIndex &site_of,
                                               const SiteEval<2, PITCH> &ev, int n_sites,
                                               int n_uc, int *qbase, unsigned char *red,
                                               ReplicaStats &S) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // exact initial state: every cluster of orbit g with all sites occupant 1
  // is seen from each of its size_g sites, so count_g = sum over sites with
  // occupant 1 of its flower count / size_g
  // Occupied sites are queued per warp and evaluated 64 at a time (two
  // independent sites per lane), so no lane idles on an empty site.
  long long cnt[MAX_ORBITS];
  for (int g = 0; g < MAX_ORBITS; ++g) cnt[g] = 0;
  long long n1 = 0, sub[4] = {0, 0, 0, 0};
  int *q = qbase + warp * 96;
  int qn = 0;
  auto eval_site = [&](int l) {
    int b, x, y, z;
    site_of(l, b, x, y, z);
    if constexpr (PITCH > 0) {
      // clusters anchored at the site, each counted once: scale by the
      // orbit size for the division below
      int nn[gen_fcc::N_ORBITS];
      gen_fcc::owned_counts<PITCH>(occ + G.addr(b, x, y, z), nn);
#pragma unroll
      for (int g = 0; g < gen_fcc::N_ORBITS; ++g) cnt[g] += nn[g] * T.orb_size[g];
    } else {
      Acc<2> acc;
      acc.zero();
      ev.add(b, 0, 1, occ, G.addr(b, x, y, z), acc);
      for (int g = 0; g < MAX_ORBITS; ++g) cnt[g] += acc.c[g];
    }
    ++n1;
    sub[sc_sublattice(x, y, z)]++;
  };
  const int per_warp = (n_sites + NW - 1) / NW;
  const int l_begin = warp * per_warp, l_end = min(n_sites, l_begin + per_warp);
  for (int l0 = l_begin; l0 < l_end; l0 += 32) {
    const int l = l0 + lane;
    bool one = false;
    if (l < l_end) {
      int b, x, y, z;
      site_of(l, b, x, y, z);
      one = occ[G.addr(b, x, y, z)] != 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, one);
    if (one) q[qn + __popc(m & ((1u << lane) - 1u))] = l;
    qn += __popc(m);
    __syncwarp();
    if (qn >= 64) {
      eval_site(q[lane]);
      eval_site(q[32 + lane]);
      __syncwarp();
      if (lane < qn - 64) q[lane] = q[64 + lane];
      qn -= 64;
      __syncwarp();
    }
  }
  if (lane < qn) eval_site(q[lane]);
  if (lane + 32 < qn) eval_site(q[lane + 32]);
  long long *rd_l = reinterpret_cast<long long *>(red);
  for (int off = 16; off; off >>= 1) {
    n1 += __shfl_xor_sync(0xffffffffu, n1, off);
    for (int g = 0; g < MAX_ORBITS; ++g) cnt[g] += __shfl_xor_sync(0xffffffffu, cnt[g], off);
    for (int k = 0; k < 4; ++k) sub[k] += __shfl_xor_sync(0xffffffffu, sub[k], off);
  }
  if (lane == 0) {
    for (int g = 0; g < MAX_ORBITS; ++g) rd_l[warp * 16 + g] = cnt[g];
    rd_l[warp * 16 + 8] = n1;
    for (int k = 0; k < 4; ++k) rd_l[warp * 16 + 9 + k] = sub[k];
  }
  __syncthreads();
  if (tid == 0) {
    long long tot[13] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int w = 0; w < NW; ++w)
      for (int k = 0; k < 13; ++k) tot[k] += rd_l[w * 16 + k];
    double e = T.w[0] * n_uc;
    for (int g = 0; g < T.n_orbits; ++g)
      e += T.w[T.orb_func_base[g]] * (double)(tot[g] / T.orb_size[g]);
    const long long pass = S.pass, np = S.n_proposed, na = S.n_accepted;
    unsigned char *raw = reinterpret_cast<unsigned char *>(&S);
    for (int q = 0; q < (int)sizeof(ReplicaStats); ++q) raw[q] = 0;
    S.energy = e;
    S.n_species[0] = n_sites - tot[8];
    S.n_species[1] = tot[8];
    for (int k = 0; k < 4; ++k) S.n_sub[k] = tot[9 + k];
    S.pass = pass;
    S.n_proposed = np;
    S.n_accepted = na;
  }
  __syncthreads();
}

template <int NOCC, int PITCH, int THREADS = SWEEP_THREADS, bool CLUSTERED = false>
__global__ void __launch_bounds__(THREADS, 512 / THREADS)
    k_sweep(const __grid_constant__ CeTables T, const __grid_constant__ SweepParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  // a replica per CTA, or per thread-block cluster of CL CTAs (generated
  // binary evaluator): every CTA keeps a whole copy of the replica, takes
  // its share of each sub-step's candidates and writes each accepted change
  // into every copy (distributed shared memory); a cluster barrier ends each
  // sub-step, and rank 0 keeps the statistics and writes the replica back
  namespace cg = cooperative_groups;
  static_assert(!CLUSTERED || PITCH > 0, "clusters share the generated binary evaluator's sweep");
  const int CL = CLUSTERED ? P.cluster : 1;  // a compile-time 1 for the one-CTA kernel
  const int crank = CLUSTERED ? (int)cg::this_cluster().block_rank() : 0;
  const int cta = (int)blockIdx.x / CL;
  const int rep = P.cta_rep ? P.cta_rep[cta] : cta;
  const Replica &R = P.reps[rep];
  ReplicaStats &Sg = P.stats[rep];
  constexpr int NW = THREADS / 32;
  __shared__ long long s_part[CLUSTERED ? 8 : 1][16];  // per-rank pass totals, gathered in rank 0
  const int tid = threadIdx.x, nth = THREADS;
  Geo G;
  G.L0 = R.L[0];
  G.L1 = R.L[1];
  G.L2 = R.L[2];
  G.R = T.reach;
  G.W = PITCH > 0 ? PITCH : G.L0 + 2 * G.R;
  G.H = PITCH > 0 ? PITCH : G.L1 + 2 * G.R;
  // a non-diagonal supercell (run-time tables only): halo cells are twisted
  // periodic images of the core
  const Cells Ctw = R.cells();
  const bool twisted = PITCH == 0 && (Ctw.t10 | Ctw.t20 | Ctw.t21) != 0;
  auto put1 = [&](int8_t *o, int b, int x, int y, int z, int8_t v) {
    if constexpr (PITCH == 0) {
      if (twisted) {
        put_site_cells(o, G, Ctw, b, x, y, z, v);
        return;
      }
    }
    put_site(o, G, b, x, y, z, v);
  };
  // binary systems with generated or register-accumulated tables keep exact
  // integer delta correlations per orbit for the running energy
  constexpr bool EXACT = (NOCC == 2 && PITCH >= 0);
  static_assert(PITCH != -2 || NOCC == 2, "the warp-cooperative evaluator is binary");
  G.V = G.W * G.H * (G.L2 + 2 * G.R);
  const int n_uc = G.L0 * G.L1 * G.L2;
  const int nsl = T.n_sublat;
  const int ncol0 = R.n_col[0], ncol1 = R.n_col[1];
  const int ncol_all = ncol0 * ncol1 * R.n_col[2];
  const int n_classes = nsl * ncol_all;
  const int ensemble = R.ensemble;
  const float beta_f = R.beta_f;
  SweepSmem lay;
  sweep_layout(T, G.L0, G.L1, G.L2, P.max_sub, PITCH, lay);
  int8_t *occ = reinterpret_cast<int8_t *>(smem + lay.occ);
  int *cl_off = reinterpret_cast<int *>(smem + lay.cl_off);
  int *lutoff = reinterpret_cast<int *>(smem + lay.lutoff);
  uint8_t *lut = reinterpret_cast<uint8_t *>(smem + lay.lut);
  float *whi = reinterpret_cast<float *>(smem + lay.whi);
  float *wlo = reinterpret_cast<float *>(smem + lay.wlo);
  float *dmu_hi = reinterpret_cast<float *>(smem + lay.dmu);
  float *dmu_lo = dmu_hi + 16;
  int *ax = reinterpret_cast<int *>(smem + lay.ax);
  uint32_t *sched = reinterpret_cast<uint32_t *>(smem + lay.sched);
  unsigned char *red = smem + lay.red;
  uint16_t *clist = reinterpret_cast<uint16_t *>(smem + lay.clist);
  int *wkept = reinterpret_cast<int *>(smem + lay.wkept);
  const int clist_cap = align16(2 * clist_capacity(G.L0, G.L1, G.L2)) / 2;
  ReplicaStats &S = *reinterpret_cast<ReplicaStats *>(smem + lay.stats);
  SubDesc *sdesc = reinterpret_cast<SubDesc *>(smem + lay.desc);
  {  // running statistics: global -> shared for the launch
    const long long *src = reinterpret_cast<const long long *>(&Sg);
    long long *dst = reinterpret_cast<long long *>(&S);
    for (int q = tid; q < (int)(sizeof(ReplicaStats) / 8); q += nth) dst[q] = src[q];
  }
  int *ax_begin[3], *ax_cnt[3], *ax_coord[3];
  for (int a = 0; a < 3; ++a) {
    ax_begin[a] = ax + a * (2 * MAX_COLOURS + MAX_L);
    ax_cnt[a] = ax_begin[a] + MAX_COLOURS;
    ax_coord[a] = ax_cnt[a] + MAX_COLOURS;
  }
  // ---- stage tables
  int *seg = reinterpret_cast<int *>(smem + lay.initq);  // PITCH -2: [n_sublat][5]
  if constexpr (PITCH <= 0) {
    for (int c = tid; c < T.n_fl; c += nth) {
      int cb = 0;
      for (int b = 0; b < nsl; ++b)
        if (c >= T.fl_begin[b][0]) cb = b;
      int off[3];
      for (int q = 0; q < 3; ++q) {
        const int pb = T.cl_pb[c * 3 + q];
        const int *du = T.cl_du + c * 9 + q * 3;
        off[q] = (pb < 0) ? 0 : (pb - cb) * G.V + du[0] + G.W * (du[1] + G.H * du[2]);
        if (PITCH != -2) cl_off[c * 3 + q] = off[q];
      }
      if constexpr (PITCH == -2) {
        int g = 0;  // the cluster's orbit: fl_begin[cb][g] <= c < fl_begin[cb][g + 1]
        while (g + 1 < T.n_orbits && c >= T.fl_begin[cb][g + 1]) ++g;
        if (P.pack16) {  // the host checked that offsets and weights fit in int16
          cl_off[c] = pack16(off[0], off[1]);
          cl_off[T.n_fl + c] = pack16(off[2], T.wq_all[g]);
        } else {  // partner-major 32-bit offsets
          for (int q = 0; q < 3; ++q) cl_off[q * T.n_fl + c] = off[q];
          lutoff[c] = T.wq_all[g];
        }
        reinterpret_cast<float *>(lut)[c] = T.wr_all[g];
      } else {
        lutoff[c] = T.cl_lut[c];
      }
    }
    if constexpr (PITCH != -2) {
      const int lut_n = T.n_fl * (T.n_sf * T.n_sf * T.n_sf * T.n_sf);
      for (int i = tid; i < lut_n; i += nth) lut[i] = T.lut[i];
    }
  }
  for (int f = tid; f < T.n_funcs; f += nth) {
    whi[f] = T.w_hi[f];
    wlo[f] = T.w_lo[f];
  }
  if (tid < 16) {
    dmu_hi[tid] = R.dmu_hi[tid];
    dmu_lo[tid] = R.dmu_lo[tid];
  }
  // colour lists per axis: L = q blocks, the first r = (L - q p) mod q of
  // size big = small + 1, the others of size small = p + (L - q p) / q;
  // colour = offset inside the block, list order = block order
  for (int i = tid; i < 3 * MAX_L; i += nth) {
    const int a = i / MAX_L, x = i - a * MAX_L;
    const int L = R.L[a], p = R.p, q = L / p, e = L - q * p, r = e % q;
    const int small = p + e / q, big = small + 1;
    if (x < R.n_col[a]) {
      ax_cnt[a][x] = x < small ? q : r;
      ax_begin[a][x] = x * q;
    }
    if (x < L) {
      int blk, off;
      if (x < r * big) {
        blk = x / big;
        off = x - blk * big;
      } else {
        const int y = x - r * big;
        blk = r + y / small;
        off = y - (blk - r) * small;
      }
      ax_coord[a][off * q + blk] = x;
    }
  }
  // ---- occupation: global -> shared core and its periodic halo images
  const int8_t *gocc = P.occ + R.occ_offset;
  const int n_sites = n_uc * nsl;
  const SiteIndex site_of(n_uc, G.L0, G.L1);
  // bulk (TMA) copies when the replica's occupations are 16-byte aligned,
  // byte loads otherwise
  const bool vec16 = !CLUSTERED && !twisted && ((R.occ_offset | n_sites) & 15) == 0;
  uint8_t *stg = smem + lay.clist;
  const int stg_cap = ((lay.bar - lay.clist) / 16) * 16;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + lay.bar);
  if (vec16) {
    const int st = stage_replica_bulk(gocc, n_sites, occ, G, site_of, stg, stg_cap, bar);
    if (st) {
      // a staging copy did not complete: the replica is left unchanged
      // (STAGE_IN_FLIGHT: its copies may also still have been in flight)
      if (tid == 0) Sg.status = st;
      return;
    }
  } else {
    for (int l = tid; l < n_sites; l += nth) {
      int b, x, y, z;
      site_of(l, b, x, y, z);
      put1(occ, b, x, y, z, gocc[l]);
    }
  }
  __syncthreads();  // core and periodic halo images (every halo cell is the
                    // image of one core site)
  if constexpr (PITCH == -2) {
    // flower bounds by cluster size (orbits are sorted by size), written after
    // the staging copies, which pass through this area; the schedule's
    // barriers order them before the first sub-step
    for (int i = tid; i < nsl * 5; i += nth) {
      const int b = i / 5, sz = i - 5 * b;  // sz = 0..4: first cluster of size > sz
      int g = 0;
      while (g < T.n_orbits && T.orb_size[g] <= sz) ++g;
      seg[i] = T.fl_begin[b][g];
    }
  }

  const SiteEval<NOCC, PITCH> ev{&T, cl_off, lutoff, lut};
  const int lane = tid & 31, warp = tid >> 5;
  // an accepted change reaches every copy of the replica
  auto put_all = [&](int b, int x, int y, int z, int8_t v) {
    if constexpr (!CLUSTERED) {
      put1(occ, b, x, y, z, v);
    } else {
      cg::cluster_group cluster = cg::this_cluster();
      for (int r = 0; r < CL; ++r) put_site(cluster.map_shared_rank(occ, r), G, b, x, y, z, v);
    }
  };
  auto sub_barrier = [&]() {
    if constexpr (!CLUSTERED) __syncthreads();
    else cg::this_cluster().sync();
  };
  if constexpr (EXACT) {
    if (P.init)
      init_binary_stats<PITCH, NW>(T, occ, G, site_of, ev, n_sites, n_uc,
                                   reinterpret_cast<int *>(smem + lay.initq), red, S);
  }
  double energy = S.energy;
  long long nspec[8], nsub[4];
  for (int a = 0; a < 8; ++a) nspec[a] = S.n_species[a];
  for (int k = 0; k < 4; ++k) nsub[k] = S.n_sub[k];
  long long pass_global = S.pass;
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const int n_pair_sw = P.n_pair_sweeps, n_local_sw = P.n_local_sweeps;
  const int n_sweeps = (ensemble == 1) ? n_pair_sw + n_local_sw : 1;
  const int n_sub = n_sweeps * n_classes;
  uint32_t *skey = sched, *spar = sched + n_sub;

  // stop requests of the host (a flag in host-mapped memory): thread 0 reads
  // it at the start of a pass and publishes it at the end of that pass, so
  // the read's latency is hidden by the pass; the block leaves at the next
  // pass boundary with a consistent state
  __shared__ int s_stop;
  if (tid == 0) s_stop = 0;
  for (long long ip = 0; ip < P.n_passes; ++ip, ++pass_global) {
    const uint32_t plo = (uint32_t)pass_global, phi = (uint32_t)(pass_global >> 32) & 0xFFFFu;
    const int stop_seen = (tid == 0 && P.stop) ? *P.stop : 0;
    // schedule: per sweep a random order of the classes, plus parameters
    for (int e = tid; e < n_sub; e += nth) {
      const int c = e % n_classes;
      const U4 r =
          philox4x32_10(U4{0xFFFFFFFFu - (uint32_t)e, 0u, plo, phi | (TAG_SCHED << 16)}, k0, k1);
      skey[e] = r.x;
      const int cb = c / ncol_all, cr = c - cb * ncol_all;
      const int cc[3] = {cr % ncol0, (cr / ncol0) % ncol1, cr / (ncol0 * ncol1)};
      int dims[3];
      for (int a = 0; a < 3; ++a) dims[a] = ax_cnt[a][cc[a]];
      const int sweep = e / n_classes;
      const uint32_t par = sched_param(r, ensemble, sweep, n_pair_sw, dims, T.n_nb[cb]);
      spar[e] = par;
    }
    __syncthreads();
    if (s_stop) break;  // the host asked the run to stop
    // rank each class inside its sweep and decode its sub-step into that slot
    for (int e = tid; e < n_sub; e += nth) {
      const int sw = e / n_classes, c = e - sw * n_classes;
      const uint32_t key = skey[e];
      int rank = 0;
      for (int c2 = 0; c2 < n_classes; ++c2) {
        const uint32_t k2 = skey[sw * n_classes + c2];
        rank += (k2 < key) || (k2 == key && c2 < c);
      }
      const uint32_t par = spar[e];
      SubDesc D;
      const int cb = c / ncol_all, cr = c - cb * ncol_all;
      const int c0 = cr % ncol0, c1 = (cr / ncol0) % ncol1, c2 = cr / (ncol0 * ncol1);
      D.cb = cb;
      D.d0 = ax_cnt[0][c0];
      D.d1 = ax_cnt[1][c1];
      D.d2 = ax_cnt[2][c2];
      D.cxo = ax_begin[0][c0];
      D.cyo = ax_begin[1][c1];
      D.czo = ax_begin[2][c2];
      D.bb = cb;
      D.par = (int)par;
      D.du0 = D.du1 = D.du2 = 0;
      int g0 = 1, g1 = 1, n = 0, pm = 1;
      if (ensemble == 0) {
        D.mode = 0;
        g0 = D.d0;
        g1 = D.d1;
        n = D.d0 * D.d1 * D.d2;
      } else if (sw < n_pair_sw) {
        // pairs along axis pa at class distance pm: candidate grid with the
        // pair axis halved
        D.mode = 1;
        if (par != 0xFFFFFFFFu) {
          const int pa = par & 3;
          pm = (par >> 2) & 255;
          const int pna = pa == 0 ? D.d0 : (pa == 1 ? D.d1 : D.d2);
          const int half = (pna / (2 * pm)) * pm;
          g0 = pa == 0 ? half : D.d0;
          g1 = pa == 1 ? half : D.d1;
          n = g0 * g1 * (pa == 2 ? half : D.d2);
        }
      } else {
        // every other class coordinate (parity bits) along each axis, paired
        // with neighbour dlt
        D.mode = 2;
        if (T.n_nb[cb] > 0) {
          const int parity = par & 7, dlt = (par >> 3) & 15;
          D.bb = T.nb_b[cb][dlt];
          D.du0 = T.nb_du[cb][dlt][0];
          D.du1 = T.nb_du[cb][dlt][1];
          D.du2 = T.nb_du[cb][dlt][2];
          const int h0 = D.d0 >= 2 ? D.d0 / 2 : 1, h1 = D.d1 >= 2 ? D.d1 / 2 : 1,
                    h2 = D.d2 >= 2 ? D.d2 / 2 : 1;
          const bool empty = (D.d0 < 2 && (parity & 1)) || (D.d1 < 2 && (parity & 2)) ||
                             (D.d2 < 2 && (parity & 4));
          g0 = h0;
          g1 = h1;
          n = empty ? 0 : h0 * h1 * h2;
        }
      }
      D.n = n;
      D.chunk = (n + NW - 1) / NW;
      D.g0 = g0;
      D.g1 = g1;
      D.m0 = (int)FastDiv::magic(g0);
      D.m1 = (int)FastDiv::magic(g1);
      D.mpm = (int)FastDiv::magic(pm);
      sdesc[sw * n_classes + rank] = D;
    }
    __syncthreads();

    std::conditional_t<EXACT, EnergyAcc<NOCC>, EnergyAccF64> eacc;
    RegCounts<NOCC> dspec;
    RegCounts<4> dsub;  // binary FCC only (PITCH > 0)
    int n_prop = 0, n_acc = 0;
    int a_buf = -1;  // clist buffer already holding this sub-step's phase A

    for (int sub = 0; sub < n_sub; ++sub) {
      const SubDesc D = sdesc[sub];
      const int cb = D.cb, d0 = D.d0, d1 = D.d1;
      const int *cx = ax_coord[0] + D.cxo;
      const int *cy = ax_coord[1] + D.cyo;
      const int *cz = ax_coord[2] + D.czo;
      const uint32_t ctr_sub = (uint32_t)sub;
      const FastDiv fe0(D.g0, (uint32_t)D.m0), fe1(D.g1, (uint32_t)D.m1);
      if (D.mode == 0) {
       if constexpr (PITCH == -2) {
        // ---------------- flips, one warp per site (binary, any size)
        const int *sg = seg + 5 * cb;
        const int *cw_a = lutoff;
        const float *cw_r = reinterpret_cast<const float *>(lut);
        for (int q = warp; q < D.n; q += NW) {
          const int t = fe0.div(q), iz = fe1.div(t);
          const int ix = q - t * d0, iy = t - iz * d1;
          const int x = cx[ix], y = cy[iy], z = cz[iz];
          const int ad = G.addr(cb, x, y, z);
          const int o_i = occ[ad], o_f = 1 - o_i;
          const int l = cb * n_uc + x + G.L0 * (y + G.L1 * z);
          const U4 r = philox4x32_10(U4{(uint32_t)l, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
          int nq = 0;
          float rr = 0.f;
          if (P.pack16)
            coop_site16(occ, ad, cl_off, cl_off + T.n_fl, cw_r, sg, lane, nq, rr);
          else
            coop_site(occ, ad, cl_off, T.n_fl, cw_a, cw_r, sg, lane, nq, rr);
          warp_sum_nr(nq, rr);
          const int dd = o_f - o_i;
          nq *= dd;
          rr = dd > 0 ? rr : -rr;
          const float de = FADD(FADD(FFMA((float)nq, T.wq_scale, rr), -dmu_hi[o_i * NOCC + o_f]),
                                -dmu_lo[o_i * NOCC + o_f]);
          if (lane == 0) {
            ++n_prop;
            if (accept_de(de, beta_f, u24(r.x))) {
              ++n_acc;
              put_site(occ, G, cb, x, y, z, (int8_t)o_f);
              eacc.de += (double)nq * (double)T.wq_scale + (double)rr;
              dspec.add(o_i, -1);
              dspec.add(o_f, 1);
            }
          }
        }
       } else {
        // ---------------- flips of every site of the class (this CTA's share)
        for (int q = crank * nth + tid; q < D.n; q += CL * nth) {
          const int t = fe0.div(q), iz = fe1.div(t);
          const int ix = q - t * d0, iy = t - iz * d1;
          const int x = cx[ix], y = cy[iy], z = cz[iz];
          const int ad = G.addr(cb, x, y, z);
          const int o_i = occ[ad];
          const int l = cb * n_uc + x + G.L0 * (y + G.L1 * z);
          const U4 r = philox4x32_10(U4{(uint32_t)l, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
          int o_f;
          if constexpr (NOCC == 2) {
            o_f = 1 - o_i;
          } else {
            const int alt = (int)(r.y % (uint32_t)(NOCC - 1));
            o_f = alt < o_i ? alt : alt + 1;
          }
          Acc<NOCC> acc;
          FF d;
          float de;
          if constexpr (PITCH >= 0) {
            acc.zero();
            ev.add(cb, o_i, o_f, occ, ad, acc);
            de = sweep_de<NOCC>(T, acc, whi, wlo, dmu_hi[o_i * NOCC + o_f],
                                dmu_lo[o_i * NOCC + o_f], d);
          } else {
            d = FF{0.f, 0.f};
            for (int g = 0; g < T.n_orbits; ++g) {
              OrbAcc<NOCC> a;
              ev.orbit(cb, g, o_i, o_f, occ, ad, a);
              orbit_fold<NOCC>(T, g, a, whi, wlo, d);
            }
            ff_add_ff(d, -dmu_hi[o_i * NOCC + o_f], -dmu_lo[o_i * NOCC + o_f]);
            de = FADD(d.s, d.e);
          }
          ++n_prop;
          if (accept_de(de, beta_f, u24(r.x))) {
            ++n_acc;
            put_all(cb, x, y, z, (int8_t)o_f);
            eacc.add(acc, d, R.dmu[o_i * NOCC + o_f]);
            dspec.add(o_i, -1);
            dspec.add(o_f, 1);
            if constexpr (PITCH > 0) dsub.add(sc_sublattice(x, y, z), o_f - o_i);
          }
        }
       }
      } else {
        // ---------------- canonical swaps: pairs inside the class (mode 1)
        // or a site with a neighbour (mode 2, sequential dE).
        // Phase A compacts the candidate pairs whose occupants differ (the
        // only proposals); phase B spreads them evenly over the block. The
        // kept order and the pair -> thread map depend only on the
        // occupations, so runs stay deterministic. Phase A of a pair sub-step
        // that follows a pair sub-step on another class runs at the end of
        // the previous phase B: it reads only its own class's sites, which
        // that phase B does not write.
        const PairGeom pg(D, ax_coord);
        const int buf = sub & 1, chunk = !CLUSTERED ? D.chunk : (D.n + CL * NW - 1) / (CL * NW);
        uint16_t *cl = clist + buf * clist_cap;
        int *wk = wkept + buf * 32;
        if (a_buf != buf) {
          compact_pairs(pg, G, occ, D.n, chunk, warp, crank * NW + warp, lane, cl, wk);
          __syncthreads();
        }
        const bool local = pg.local;
        const int bb = pg.bb;
        int total = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) total += wk[w];
        if constexpr (PITCH == -2) {
          // one warp per pair (binary, any size); the first change is applied
          // before any cluster is read (a site's own flower never contains
          // it): a sees the original state, b sees a changed
          const int *cw_a = lutoff;
          const float *cw_r = reinterpret_cast<const float *>(lut);
          for (int i = warp; i < total; i += NW) {
            int wsel = 0, bsel = 0, run = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
              const int k = wk[w];
              if (i >= run) {
                wsel = w;
                bsel = run;
              }
              run += k;
            }
            const int q = cl[wsel * chunk + (i - bsel)];
            int xa, ya, za, xb, yb, zb;
            pg.sites(q, G, xa, ya, za, xb, yb, zb);
            const int ada = G.addr(cb, xa, ya, za), adb = G.addr(bb, xb, yb, zb);
            const int oa = occ[ada], ob = occ[adb];
            const int la = cb * n_uc + xa + G.L0 * (ya + G.L1 * za);
            const U4 r =
                philox4x32_10(U4{(uint32_t)la, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
            __syncwarp();
            if (local && lane == 0) put_site(occ, G, cb, xa, ya, za, (int8_t)ob);
            __syncwarp();
            int na = 0, nb = 0;
            float ra = 0.f, rb = 0.f;
            if (P.pack16) {
              coop_site16(occ, ada, cl_off, cl_off + T.n_fl, cw_r, seg + 5 * cb, lane, na, ra);
              coop_site16(occ, adb, cl_off, cl_off + T.n_fl, cw_r, seg + 5 * bb, lane, nb, rb);
            } else {
              coop_site(occ, ada, cl_off, T.n_fl, cw_a, cw_r, seg + 5 * cb, lane, na, ra);
              coop_site(occ, adb, cl_off, T.n_fl, cw_a, cw_r, seg + 5 * bb, lane, nb, rb);
            }
            int nq = na - nb;
            float rr = FADD(ra, -rb);
            warp_sum_nr(nq, rr);
            const int dd = ob - oa;  // a: oa -> ob, b: ob -> oa
            nq *= dd;
            rr = dd > 0 ? rr : -rr;
            const float de = FFMA((float)nq, T.wq_scale, rr);
            __syncwarp();
            if (lane == 0) {
              ++n_prop;
              if (accept_de(de, beta_f, u24(r.x))) {
                ++n_acc;
                if (!local) put_site(occ, G, cb, xa, ya, za, (int8_t)ob);
                put_site(occ, G, bb, xb, yb, zb, (int8_t)oa);
                eacc.de += (double)nq * (double)T.wq_scale + (double)rr;
              } else if (local) {
                put_site(occ, G, cb, xa, ya, za, (int8_t)oa);
              }
            }
          }
        }
        for (int i = tid; PITCH != -2 && i < total; i += nth) {
          int wsel = 0, bsel = 0, run = 0;
#pragma unroll
          for (int w = 0; w < NW; ++w) {  // last warp whose kept range starts at or before i
            const int k = wk[w];
            if (i >= run) {
              wsel = w;
              bsel = run;
            }
            run += k;
          }
          const int q = cl[wsel * chunk + (i - bsel)];
          int xa, ya, za, xb, yb, zb;
          pg.sites(q, G, xa, ya, za, xb, yb, zb);
          const int ada = G.addr(cb, xa, ya, za), adb = G.addr(bb, xb, yb, zb);
          const int oa = occ[ada], ob = occ[adb];
          const int la = cb * n_uc + xa + G.L0 * (ya + G.L1 * za);
          const U4 r = philox4x32_10(U4{(uint32_t)la, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
          Acc<NOCC> acc;
          FF d;
          float de;
          if constexpr (PITCH >= 0) {
            // the first change is applied before either flower is read (a
            // site's own flower never contains it, so a sees the original
            // state and b sees a changed); the two gathers can then overlap
            acc.zero();
            if (local) put_site(occ, G, cb, xa, ya, za, (int8_t)ob);
            ev.add(cb, oa, ob, occ, ada, acc);
            ev.add(bb, ob, oa, occ, adb, acc);
            de = sweep_de<NOCC>(T, acc, whi, wlo, 0.f, 0.f, d);
          } else {
            // the first change is applied before any cluster is read: a
            // site's own flower never contains it, so a sees the original
            // state and b sees a changed
            if (local) put_site(occ, G, cb, xa, ya, za, (int8_t)ob);
            d = FF{0.f, 0.f};
            for (int g = 0; g < T.n_orbits; ++g) {
              OrbAcc<NOCC> a;
              ev.orbit(cb, g, oa, ob, occ, ada, a);
              ev.orbit(bb, g, ob, oa, occ, adb, a);
              orbit_fold<NOCC>(T, g, a, whi, wlo, d);
            }
            de = FADD(d.s, d.e);
          }
          ++n_prop;
          if (accept_de(de, beta_f, u24(r.x))) {
            ++n_acc;
            // (a neighbour swap's first change is already in this copy; the
            // other copies receive it now)
            if (!local || CLUSTERED) put_all(cb, xa, ya, za, (int8_t)ob);
            put_all(bb, xb, yb, zb, (int8_t)oa);
            eacc.add(acc, d, 0.0);
            if constexpr (PITCH > 0) {
              dsub.add(sc_sublattice(xa, ya, za), ob - oa);
              dsub.add(sc_sublattice(xb, yb, zb), oa - ob);
            }
          } else if (local) {
            put_site(occ, G, cb, xa, ya, za, (int8_t)oa);
          }
        }
        a_buf = -1;
        if (D.mode == 1 && sub + 1 < n_sub) {
          const SubDesc Dn = sdesc[sub + 1];
          if (Dn.mode == 1 &&
              (Dn.cb != D.cb || Dn.cxo != D.cxo || Dn.cyo != D.cyo || Dn.czo != D.czo)) {
            const PairGeom pn(Dn, ax_coord);
            const int chunk_n = !CLUSTERED ? Dn.chunk : (Dn.n + CL * NW - 1) / (CL * NW);
            compact_pairs(pn, G, occ, Dn.n, chunk_n, warp, crank * NW + warp, lane,
                          clist + (buf ^ 1) * clist_cap, wkept + (buf ^ 1) * 32);
            a_buf = buf ^ 1;
          }
        }
      }
      sub_barrier();  // every copy holds the sub-step's changes
    }

    // ---- end of pass: reduce (32-bit per-pass counters), sample
    {
      // slots: 0 proposals, 1 accepts, 2..2+NOCC species, 4..7 sublattice
      // counts (binary FCC), 8..15 energy terms (binary); double slot: dE sum
      int vals[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) vals[k] = 0;
      vals[0] = n_prop;
      vals[1] = n_acc;
#pragma unroll
      for (int a = 0; a < NOCC; ++a) vals[2 + a] = dspec.v[a];
      if constexpr (PITCH > 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) vals[4 + k] = dsub.v[k];
      }
      double dsum = 0.0;
      if constexpr (EXACT) {
#pragma unroll
        for (int g = 0; g < MAX_ORBITS; ++g) vals[8 + g] = eacc.dc[g];
      } else {
        dsum = eacc.de;
      }
#pragma unroll
      for (int k = 0; k < 16; ++k)
        for (int off = 16; off; off >>= 1) vals[k] += __shfl_xor_sync(0xffffffffu, vals[k], off);
      if constexpr (!EXACT)
        for (int off = 16; off; off >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, off);
      int *rd_i = reinterpret_cast<int *>(red);                   // [NW][16]
      double *rd_d = reinterpret_cast<double *>(red + NW * 64);  // [NW]
      if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 16; ++k) rd_i[warp * 16 + k] = vals[k];
        rd_d[warp] = dsum;
      }
      __syncthreads();
      // lane k < 16 of warp 0 sums slot k over the warps; lane 16 sums the dE
      // slot in warp order
      long long v = 0;
      double dv = 0.0;
      if (warp == 0) {
        if (lane < 16)
          for (int w = 0; w < NW; ++w) v += rd_i[w * 16 + lane];
        if (lane == 16)
          for (int w = 0; w < NW; ++w) dv += rd_d[w];
      }
      if constexpr (CLUSTERED) {
        // a cluster's pass totals (binary: integers only) gather in rank 0
        cg::cluster_group cluster = cg::this_cluster();
        if (warp == 0 && lane < 16) *cluster.map_shared_rank(&s_part[crank][lane], 0) = v;
        cluster.sync();
        if (warp == 0 && crank == 0 && lane < 16) {
          v = 0;
          for (int r = 0; r < CL; ++r) v += s_part[r][lane];
        }
      }
      if (warp == 0 && crank == 0) {
        long long tot[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) tot[k] = __shfl_sync(0xffffffffu, v, k);
        double dtot = __shfl_sync(0xffffffffu, dv, 16);
        if (lane == 0) {
          s_stop = stop_seen;
          if constexpr (CLUSTERED) {  // every rank leaves at the same pass boundary
            cg::cluster_group cluster = cg::this_cluster();
            for (int r = 1; r < CL; ++r) *cluster.map_shared_rank(&s_stop, r) = stop_seen;
          }
          if constexpr (EXACT) {
            dtot = 0.0;
            for (int g = 0; g < T.n_orbits; ++g)
              dtot += T.w[T.orb_func_base[g]] * (double)tot[8 + g];
          }
          energy += dtot;
          S.n_proposed += tot[0];
          S.n_accepted += tot[1];
          for (int a = 0; a < NOCC; ++a) nspec[a] += tot[2 + a];
          double op = 0.0;
          if constexpr (PITCH > 0) {
            for (int k = 0; k < 4; ++k) nsub[k] += tot[4 + k];
            const double xb = (double)nspec[1] / n_sites;
            for (int k = 0; k < 4; ++k) {
              const double c = (double)nsub[k] / (0.25 * n_sites) - xb;
              op += c * c;
            }
            op = sqrt(op);
          }
          // param composition per unit cell and potential per unit cell
          double x[3] = {0.0, 0.0, 0.0}, ef, ep;
          sample_values<NOCC>(P.RT, R.mu, nspec, n_sites, n_uc, energy, x, ef, ep);
          if (ip >= P.n_equil) {
            S.n_samples += 1.0;
            S.sum_e += ep;
            S.sum_e2 += ep * ep;
            S.sum_f += ef;
            for (int k = 0; k < NOCC - 1; ++k) {
              S.sum_x[k] += x[k];
              S.sum_ex[k] += ep * x[k];
              for (int k2 = 0; k2 < NOCC - 1; ++k2) S.sum_xx[k * 3 + k2] += x[k] * x[k2];
            }
            if (P.samples) {
              const long long si = (long long)(S.n_samples) - 1;
              if (si < P.sample_capacity) {
                double *out = P.samples + (long long)rep * P.sample_capacity * P.sample_width +
                              si * P.sample_width;
                out[0] = ep;
                for (int k = 0; k < NOCC - 1; ++k) out[1 + k] = x[k];
                out[NOCC] = op;
              }
            }
          }
        }
      }
      if constexpr (CLUSTERED) cg::this_cluster().sync();  // the stop decision reached every rank
    }
  }
  if constexpr (CLUSTERED) {
    cg::this_cluster().sync();  // no peer writes into this copy any more
    if (crank != 0) return;     // rank 0 writes the replica and its statistics back
  }
  // ---- write back
  if (vec16) {
    writeback_replica_bulk(P.occ + R.occ_offset, n_sites, occ, G, site_of, stg, stg_cap);
  } else {
    for (int l = tid; l < n_sites; l += nth) {
      int b, x, y, z;
      site_of(l, b, x, y, z);
      P.occ[R.occ_offset + l] = occ[G.addr(b, x, y, z)];
    }
  }
  if (tid == 0) {
    S.energy = energy;
    for (int a = 0; a < NOCC; ++a) S.n_species[a] = nspec[a];
    for (int k = 0; k < 4; ++k) S.n_sub[k] = nsub[k];
    S.pass = pass_global;
  }
  __syncthreads();
  {
    const long long *src = reinterpret_cast<const long long *>(&S);
    long long *dst = reinterpret_cast<long long *>(&Sg);
    for (int q = tid; q < (int)(sizeof(ReplicaStats) / 8); q += nth) dst[q] = src[q];
  }
}

// ------------------------------------------------------------ launchers
template <int NOCC>
cudaError_t launch_energy_t(const CeTables &T, const int8_t *occ, const Cells &C,
                            unsigned long long *counts, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * T.n_funcs, st);
  if (e != cudaSuccess) return e;
  const int n = C.L0 * C.L1 * C.L2 * T.n_sublat;
  int grid = (n + 255) / 256;
  if (grid > 4096) grid = 4096;
  k_energy<NOCC><<<grid, 256, 0, st>>>(T, occ, C, counts);
  return cudaGetLastError();
}

template <int NOCC>
cudaError_t launch_delta_t(const CeTables &T, const int8_t *occ, const Cells &C,
                           int n_events, int k_sites, const long long *sites, const int *new_occ,
                           const double *dmu, double *dE, long long *dcount, cudaStream_t st) {
  const int grid = (n_events + 127) / 128;
  if (grid == 0) return cudaSuccess;
  k_delta<NOCC><<<grid, 128, 0, st>>>(T, occ, C, n_events, k_sites, sites, new_occ, dmu, dE,
                                      dcount);
  return cudaGetLastError();
}

template <int NOCC>
cudaError_t launch_init_stats_t(const CeTables &T, const Replica *reps, ReplicaStats *stats,
                                const int8_t *occ, int n_replicas, int max_sites, cudaStream_t st) {
  const int cap = max_sites <= 160 * 1024 ? ((max_sites + 15) & ~15) : 0;
  cudaError_t e =
      cudaFuncSetAttribute(k_init_stats<NOCC>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  if (e != cudaSuccess) return e;
  k_init_stats<NOCC><<<n_replicas, 512, cap, st>>>(T, reps, stats, occ, cap);
  return cudaGetLastError();
}

inline int replay_smem_bytes_impl(int n_sites, int n_occ) {
  return (int)sizeof(MtState) + ((n_sites + 15) & ~15) + 4 * n_sites * (1 + n_occ);
}

template <int NOCC>
cudaError_t launch_replay_t(const CeTables &T, const ReplayParams &P, cudaStream_t st) {
  const int smem = replay_smem_bytes_impl(P.n_sites, T.n_occ);
  cudaError_t e =
      cudaFuncSetAttribute(k_replay<NOCC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_replay<NOCC><<<1, 32, smem, st>>>(T, P);
  return cudaGetLastError();
}

template <int NOCC, int PITCH, int THREADS = SWEEP_THREADS>
cudaError_t launch_sweep_t(const CeTables &T, const SweepParams &P, int n_replicas, int smem,
                           cudaStream_t st) {
  if constexpr (PITCH > 0 && THREADS == SWEEP_THREADS) {
    if (P.cluster > 1) {
      // one thread-block cluster of P.cluster CTAs per replica
      cudaError_t e = cudaFuncSetAttribute(k_sweep<NOCC, PITCH, THREADS, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)(n_replicas * P.cluster));
      cfg.blockDim = dim3(THREADS);
      cfg.dynamicSmemBytes = (size_t)smem;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)P.cluster;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      return cudaLaunchKernelEx(&cfg, k_sweep<NOCC, PITCH, THREADS, true>, T, P);
    }
  }
  cudaError_t e = cudaFuncSetAttribute(k_sweep<NOCC, PITCH, THREADS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_sweep<NOCC, PITCH, THREADS><<<n_replicas, THREADS, smem, st>>>(T, P);
  return cudaGetLastError();
}

#define CEM_INSTANTIATE(N)                                                                     \
  template cudaError_t launch_energy_t<N>(const CeTables &, const int8_t *, const Cells &,     \
                                          unsigned long long *, cudaStream_t);                 \
  template cudaError_t launch_delta_t<N>(const CeTables &, const int8_t *, const Cells &, int, \
                                         int, const long long *, const int *, const double *,  \
                                         double *, long long *, cudaStream_t);                 \
  template cudaError_t launch_replay_t<N>(const CeTables &, const ReplayParams &, cudaStream_t); \
  template cudaError_t launch_init_stats_t<N>(const CeTables &, const Replica *, ReplicaStats *, \
                                              const int8_t *, int, int, cudaStream_t);         \
  template cudaError_t launch_sweep_t<N, 0, SWEEP_THREADS>(const CeTables &, const SweepParams &, \
                                                           int, int, cudaStream_t);

}  // namespace cem
