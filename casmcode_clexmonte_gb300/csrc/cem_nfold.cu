// n-fold way: rejection-free semi-grand canonical Monte Carlo (Bortz, Kalos
// and Lebowitz, J. Comput. Phys. 17, 10 (1975)), the method of
// clexmonte::nfold::Nfold::run (include/casm/clexmonte/nfold/nfold_impl.hh:20-108).
//
// Events are all single-site occupant changes (site l to each other occupant);
// an event's rate is its Metropolis acceptance, 1 if dE <= 0 else
// exp(-beta dE), with dE the semi-grand canonical potential change
// (CompleteEventCalculator::calculate_rate, src/casm/clexmonte/nfold/nfold_events.cc:24-60).
// Each step draws one event with probability rate / total from a 32-ary
// FP64 sum tree over all events of the replica (a node is the pairwise sum of
// its 32 children, zero-padded: (c0 + c1) + (c2 + c3), ...; a descent walks
// down the same binary tree inside each node), applies it and recomputes the
// rates of the events whose site shares a cluster with the changed site. The
// state before the step is weighted by its expected residence time in
// Metropolis trials, n_possible / total, with n_possible = sites x n_occ x
// (n_occ - 1) (the reference's n_events_possible: semi-grand canonical swaps
// per unit cell x unit cells).
//
// One CTA per replica; the replica's occupation stays in shared memory (the
// sweep kernel's halo'd layout), and so does the tree when it fits beside it
// (24^3 binary: 14 271 doubles, 114 KB), else it lives in global memory (L2
// resident). Pairwise sums keep the dependent chain of a node short (depth 5
// instead of 31 sequential additions on the narrow FP64 pipe); warp 0
// descends with one child per lane.
// Every floating-point operation that decides the trajectory (energy change,
// rate, tree sums, descent) is explicitly rounded, so the oracle's sequential
// restatement reproduces the event sequence bit for bit.
#include "cem_kernels.cuh"

namespace cem {

namespace {

constexpr int NF_THREADS = 128;
constexpr uint32_t TAG_NFOLD = 0x3u;

// FP64 energy change of the formation energy from integer delta counts, in
// function-index order, one fused multiply-add per function.
template <int NOCC>
__device__ __forceinline__ double de_fp64(const CeTables &T, const Acc<NOCC> &acc) {
  double d = 0.0;
#pragma unroll
  for (int g = 0; g < MAX_ORBITS; ++g) {
    if (g < T.n_orbits) {
      const int base = T.orb_func_base[g];
      if constexpr (NOCC == 2) {
        d = DFMA(T.w[base], (double)acc.c[g], d);
      } else {
        const int nf = T.orb_n_funcs[g];
        for (int fl = 0; fl < nf; ++fl) d = DFMA(T.w[base + fl], (double)acc_dc<NOCC>(acc, g, fl), d);
      }
    }
  }
  return d;
}

// The same sum one orbit at a time (any number of orbits): adds orbit g's
// terms to d in function-index order.
template <int NOCC>
__device__ __forceinline__ double orbit_fold_fp64(const CeTables &T, int g, const OrbAcc<NOCC> &a,
                                                  double d) {
  const int base = T.orb_func_base[g];
  if constexpr (NOCC == 2) {
    return DFMA(T.w[base], (double)a.c, d);
  } else {
    const int nf = T.orb_n_funcs[g];
    for (int fl = 0; fl < nf; ++fl) {
      const int dc = (int)((a.p >> (8 * fl)) & 255ull) - (int)((a.m >> (8 * fl)) & 255ull);
      d = DFMA(T.w[base + fl], (double)dc, d);
    }
    return d;
  }
}

struct NfoldLayout {
  int occ, cl_off, lutoff, lut, stats, imp, misc, tree, total;
};

inline __host__ __device__ void nfold_layout(const CeTables &T, int L0, int L1, int L2, int pitch,
                                             int tree_smem, NfoldLayout &s) {
  const int R = T.reach;
  const int W = pitch ? pitch : L0 + 2 * R, H = pitch ? pitch : L1 + 2 * R;
  const int V = W * H * (L2 + 2 * R);
  const bool tables = pitch == 0;
  int o = 0;
  s.occ = o;
  o += align16(T.n_sublat * V);
  s.cl_off = o;
  o += tables ? align16(T.n_fl * 3 * 4) : 0;
  s.lutoff = o;
  o += tables ? align16(T.n_fl * 4) : 0;
  s.lut = o;
  o += tables ? align16(T.n_fl * (T.n_sf * T.n_sf * T.n_sf * T.n_sf)) : 0;
  s.stats = o;
  o += align16((int)sizeof(ReplicaStats));
  s.imp = o;  // impacted sites of the current step
  o += align16((MAX_FP + 1) * 4);
  s.misc = o;  // selected event
  o += 16;
  s.tree = o;  // the rate tree (tree_smem)
  if (tree_smem)
    o += align16((int)(8 * rate_tree_size((long long)L0 * L1 * L2 * T.n_sublat * (T.n_occ - 1))));
  s.total = o;
}

template <int NOCC, int PITCH>
__global__ void __launch_bounds__(NF_THREADS)
    k_nfold(const __grid_constant__ CeTables T, const __grid_constant__ NfoldParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int rep = blockIdx.x, tid = threadIdx.x, nth = NF_THREADS;
  const Replica &R = P.reps[rep];
  ReplicaStats &Sg = P.stats[rep];
  Geo G;
  G.L0 = R.L[0];
  G.L1 = R.L[1];
  G.L2 = R.L[2];
  G.R = T.reach;
  G.W = PITCH ? PITCH : G.L0 + 2 * G.R;
  G.H = PITCH ? PITCH : G.L1 + 2 * G.R;
  G.V = G.W * G.H * (G.L2 + 2 * G.R);
  const int n_uc = G.L0 * G.L1 * G.L2, nsl = T.n_sublat, n_sites = n_uc * nsl;
  NfoldLayout lay;
  nfold_layout(T, G.L0, G.L1, G.L2, PITCH, P.tree_smem, lay);
  int8_t *occ = reinterpret_cast<int8_t *>(smem + lay.occ);
  int *cl_off = reinterpret_cast<int *>(smem + lay.cl_off);
  int *lutoff = reinterpret_cast<int *>(smem + lay.lutoff);
  uint8_t *lut = reinterpret_cast<uint8_t *>(smem + lay.lut);
  ReplicaStats &S = *reinterpret_cast<ReplicaStats *>(smem + lay.stats);
  int *imp = reinterpret_cast<int *>(smem + lay.imp);
  long long *sel = reinterpret_cast<long long *>(smem + lay.misc);

  if constexpr (PITCH == 0) {
    for (int c = tid; c < T.n_fl; c += nth) {
      int cb = 0;
      for (int b = 0; b < nsl; ++b)
        if (c >= T.fl_begin[b][0]) cb = b;
      for (int q = 0; q < 3; ++q) {
        const int pb = T.cl_pb[c * 3 + q];
        const int *du = T.cl_du + c * 9 + q * 3;
        cl_off[c * 3 + q] = (pb < 0) ? 0 : (pb - cb) * G.V + du[0] + G.W * (du[1] + G.H * du[2]);
      }
      lutoff[c] = T.cl_lut[c];
    }
    const int lut_n = T.n_fl * (T.n_sf * T.n_sf * T.n_sf * T.n_sf);
    for (int i = tid; i < lut_n; i += nth) lut[i] = T.lut[i];
  }
  {
    const long long *src = reinterpret_cast<const long long *>(&Sg);
    long long *dst = reinterpret_cast<long long *>(&S);
    for (int q = tid; q < (int)(sizeof(ReplicaStats) / 8); q += nth) dst[q] = src[q];
  }
  const int8_t *gocc = P.occ + R.occ_offset;
  const SiteIndex site_of(n_uc, G.L0, G.L1);
  // non-diagonal supercells: twisted periodic images
  const Cells C = R.cells();
  const bool twisted = (C.t10 | C.t20 | C.t21) != 0;
  auto put = [&](int b, int x, int y, int z, int8_t v) {
    if (twisted)
      put_site_cells(occ, G, C, b, x, y, z, v);
    else
      put_site(occ, G, b, x, y, z, v);
  };
  for (int l = tid; l < n_sites; l += nth) {
    int b, x, y, z;
    site_of(l, b, x, y, z);
    put(b, x, y, z, gocc[l]);
  }
  __syncthreads();

  const SiteEval<NOCC, PITCH> ev{&T, cl_off, lutoff, lut};
  const double beta = R.beta;
  // FP64 formation-energy change of one site change: the generated evaluator
  // with register counts, or the run-time tables one orbit at a time (the
  // same terms in the same order, for expansions of any size)
  auto site_de = [&](int b, int o_i, int o_f, int ad) -> double {
    if constexpr (PITCH > 0) {
      Acc<NOCC> acc;
      acc.zero();
      ev.add(b, o_i, o_f, occ, ad, acc);
      return de_fp64<NOCC>(T, acc);
    } else {
      double d = 0.0;
      for (int g = 0; g < T.n_orbits; ++g) {
        OrbAcc<NOCC> a;
        ev.orbit(b, g, o_i, o_f, occ, ad, a);
        d = orbit_fold_fp64<NOCC>(T, g, a, d);
      }
      return d;
    }
  };
  // rate of event e = l (n_occ - 1) + k: site l to its k-th other occupant
  auto rate_of = [&](long long e) -> double {
    const int l = (int)(e / (NOCC - 1)), k = (int)(e - (long long)l * (NOCC - 1));
    int b, x, y, z;
    site_of(l, b, x, y, z);
    const int ad = G.addr(b, x, y, z);
    const int o_i = occ[ad];
    const int o_f = k < o_i ? k : k + 1;
    const double de = DSUB(site_de(b, o_i, o_f, ad), R.dmu[o_i * NOCC + o_f]);
    return de <= 0.0 ? 1.0 : cem_exp_neg(DMUL(-beta, de));
  };
  // sum tree over the events: level 0 = rates, node = sum of its 32 children
  const long long n_ev = (long long)n_sites * (NOCC - 1);
  RateTree tg;
  rate_tree_geo(n_ev, tg);
  double *tr = P.tree_smem ? reinterpret_cast<double *>(smem + lay.tree) : P.tree + P.tree_off[rep];
  auto node_sum = [&](int lev, long long node) {
    const double *ch = tr + tg.off[lev - 1];
    const long long c0 = node * 32;
    const int cnt = (int)(min(c0 + 32, tg.n[lev - 1]) - c0);
    double v[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = c < cnt ? ch[c0 + c] : 0.0;
#pragma unroll
    for (int w = 1; w < 32; w *= 2)
#pragma unroll
      for (int i = 0; i < 32; i += 2 * w) v[i] = DADD(v[i], v[i + w]);
    tr[tg.off[lev] + node] = v[0];
  };
  for (long long e = tid; e < n_ev; e += nth) tr[e] = rate_of(e);
  __syncthreads();
  for (int lev = 1; lev < tg.n_lev; ++lev) {
    for (long long node = tid; node < tg.n[lev]; node += nth) node_sum(lev, node);
    __syncthreads();
  }

  // the running energy and species counts live in S (shared memory): thread
  // 0 applies each event to them, warp 1 samples them while warp 0 descends
  long long counter = S.pass;  // events drawn by this replica so far
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const double n_possible = (double)n_sites * (double)(NOCC * (NOCC - 1));
  int status = 0;
  const long long n_total = P.n_equil + P.n_events;
  const int lane = tid & 31;
  for (long long it = 0; it < n_total; ++it, ++counter) {
    if (tid == 32 && it >= P.n_equil) {
      // the state before this step, weighted by its residence time
      const double total = tr[tg.off[tg.n_lev - 1]];
      if (total > 0.0) {
        const double dt = DDIV(n_possible, total);
        {
          double x[3] = {0.0, 0.0, 0.0}, ef, ep;
          sample_values<NOCC>(P.RT, R.mu, reinterpret_cast<const long long *>(S.n_species), n_sites, n_uc,
                              S.energy, x, ef, ep);
          S.n_samples = DADD(S.n_samples, dt);
          S.sum_e = DADD(S.sum_e, DMUL(dt, ep));
          S.sum_e2 = DADD(S.sum_e2, DMUL(dt, DMUL(ep, ep)));
          S.sum_f = DADD(S.sum_f, DMUL(dt, ef));
          for (int k = 0; k < NOCC - 1; ++k) {
            S.sum_x[k] = DADD(S.sum_x[k], DMUL(dt, x[k]));
            S.sum_ex[k] = DADD(S.sum_ex[k], DMUL(dt, DMUL(ep, x[k])));
            for (int k2 = 0; k2 < NOCC - 1; ++k2)
              S.sum_xx[k * 3 + k2] = DADD(S.sum_xx[k * 3 + k2], DMUL(dt, DMUL(x[k], x[k2])));
          }
        }
      }
    }
    if (tid < 32) {
      const double total = tr[tg.off[tg.n_lev - 1]];
      long long leaf = -1;
      if (total > 0.0) {
        const double dt = DDIV(n_possible, total);
        const U4 r = philox4x32_10(
            U4{(uint32_t)counter, (uint32_t)(counter >> 32), 0u, TAG_NFOLD << 16}, k0, k1);
        double tgt = DMUL(u53(r.x, r.y), total);
        long long node = 0;
        const unsigned full = 0xffffffffu;
        for (int lev = tg.n_lev - 1; lev >= 1; --lev) {
          const long long c0 = node * 32;
          const int cnt = (int)(min(c0 + 32, tg.n[lev - 1]) - c0);
          // one child per lane; p_k on lanes i 2^k holds the sum of children
          // i 2^k .. (i + 1) 2^k - 1 (the node's binary tree)
          const double p0 = lane < cnt ? tr[tg.off[lev - 1] + c0 + lane] : 0.0;
          const double p1 = DADD(p0, __shfl_down_sync(full, p0, 1));
          const double p2 = DADD(p1, __shfl_down_sync(full, p1, 2));
          const double p3 = DADD(p2, __shfl_down_sync(full, p2, 4));
          const double p4 = DADD(p3, __shfl_down_sync(full, p3, 8));
          // down the binary tree: left when the right half is empty or the
          // target lies below the left half's sum, else right
          int base = 0;
          auto step = [&](double p, int half) {
            const double left = __shfl_sync(full, p, base), right = __shfl_sync(full, p, base + half);
            if (!(right == 0.0 || (left > 0.0 && tgt < left))) {
              tgt = DSUB(tgt, left);
              base += half;
            }
          };
          step(p4, 16);
          step(p3, 8);
          step(p2, 4);
          step(p1, 2);
          step(p0, 1);
          node = c0 + base;
        }
        leaf = node;
        if (lane == 0) {
          if (it < P.rec_cap) {
            const long long ri = (long long)rep * P.rec_cap + it;
            const int l = (int)(leaf / (NOCC - 1)), k = (int)(leaf - (long long)l * (NOCC - 1));
            int b, x, y, z;
            site_of(l, b, x, y, z);
            const int o_i = occ[G.addr(b, x, y, z)];
            P.rec_site[ri] = l;
            P.rec_occ[ri] = k < o_i ? k : k + 1;
            P.rec_dt[ri] = dt;
          }
          S.n_proposed += 1;
          S.n_accepted += 1;
        }
      }
      if (lane == 0) sel[0] = leaf;
    }
    __syncthreads();
    const long long leaf = sel[0];
    if (leaf < 0) {
      status = 1;  // no event has a non-zero rate
      break;
    }
    const int l = (int)(leaf / (NOCC - 1)), kk = (int)(leaf - (long long)l * (NOCC - 1));
    int b, x, y, z;
    site_of(l, b, x, y, z);
    const int ad_l = G.addr(b, x, y, z);
    if (tid == 0) {
      const int o_i = occ[ad_l];
      const int o_f = kk < o_i ? kk : kk + 1;
      sel[1] = o_i;
      S.n_species[o_i] -= 1;
      S.n_species[o_f] += 1;
      put(b, x, y, z, (int8_t)o_f);
    }
    // impacted sites: the changed site and its flower partners
    const int n_imp = 1 + T.n_fp[b];
    for (int t = tid; t < n_imp; t += nth) {
      int s = l;
      if (t > 0) {
        const int *e = T.fp + ((size_t)b * MAX_FP + (t - 1)) * 4;
        s = e[0] * n_uc + C.index(x + e[1], y + e[2], z + e[3]);
      }
      imp[t] = s;
    }
    __syncthreads();
    if (tid == 96) {
      // the applied change's energy, from the reverse change on the new state:
      // its delta counts are the exact negatives (the flower excludes the
      // site), so E - dE_reverse equals E + dE bit for bit; off the critical
      // path of the rate updates
      const int o_f = occ[ad_l], o_i = (int)sel[1];
      S.energy = DSUB(S.energy, site_de(b, o_f, o_i, ad_l));
    }
    for (int t = tid; t < n_imp * (NOCC - 1); t += nth) {
      const long long e = (long long)imp[t / (NOCC - 1)] * (NOCC - 1) + t % (NOCC - 1);
      tr[e] = rate_of(e);
    }
    __syncthreads();
    for (int lev = 1; lev < tg.n_lev; ++lev) {
      for (int t = tid; t < n_imp * (NOCC - 1); t += nth) {
        const long long e = (long long)imp[t / (NOCC - 1)] * (NOCC - 1) + t % (NOCC - 1);
        node_sum(lev, e >> (5 * lev));
      }
      __syncthreads();
    }
  }
  for (int l = tid; l < n_sites; l += nth) {
    int b, x, y, z;
    site_of(l, b, x, y, z);
    P.occ[R.occ_offset + l] = occ[G.addr(b, x, y, z)];
  }
  if (tid == 0) {
    S.pass = counter;
    S.status = status;
  }
  __syncthreads();
  {
    const long long *src = reinterpret_cast<const long long *>(&S);
    long long *dst = reinterpret_cast<long long *>(&Sg);
    for (int q = tid; q < (int)(sizeof(ReplicaStats) / 8); q += nth) dst[q] = src[q];
  }
}

template <int NOCC, int PITCH>
cudaError_t launch_nfold_t(const CeTables &T, const NfoldParams &P, int n_replicas, int smem,
                           cudaStream_t st) {
  cudaError_t e =
      cudaFuncSetAttribute(k_nfold<NOCC, PITCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_nfold<NOCC, PITCH><<<n_replicas, NF_THREADS, smem, st>>>(T, P);
  return cudaGetLastError();
}

}  // namespace

int nfold_smem_bytes(const CeTables &T, int L0, int L1, int L2, int pitch, int tree_smem) {
  NfoldLayout s;
  nfold_layout(T, L0, L1, L2, pitch, tree_smem, s);
  return s.total;
}

cudaError_t launch_nfold(const CeTables &T, const NfoldParams &P, int n_replicas, int smem,
                         int pitch, cudaStream_t st) {
  if (pitch == 28) return launch_nfold_t<2, 28>(T, P, n_replicas, smem, st);
  if (pitch == 14) return launch_nfold_t<2, 14>(T, P, n_replicas, smem, st);
  if (pitch != 0) return cudaErrorInvalidValue;
  if (T.n_occ == 2) return launch_nfold_t<2, 0>(T, P, n_replicas, smem, st);
  if (T.n_occ == 3) return launch_nfold_t<3, 0>(T, P, n_replicas, smem, st);
  return cudaErrorInvalidValue;
}

}  // namespace cem
