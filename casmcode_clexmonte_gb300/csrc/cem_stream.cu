// HBM-streamed parallel Metropolis for replicas too large for shared memory
// (binary FCC of the generated topology, even supercell lengths).
//
// Each replica's occupation lives in a halo'd global-memory block (x/y pitch
// P = L + 4). One pass is a sequence of sub-step kernels, each updating one
// colour class of every replica at once over many CTAs, followed by an
// end-of-pass kernel that folds the per-replica accumulators into the running
// energy, moments and samples. The sub-step schedule, the site/pair mapping
// and the random numbers are those of the shared-memory sweep, so a replica
// gives the same chain through either path. One pass is captured once into a
// CUDA graph and replayed pass after pass.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "cem_kernels.cuh"

namespace cem {

struct StreamParams {
  const Replica *reps;
  ReplicaStats *stats;
  int8_t *halo;            // [n_rep][halo_stride]
  long long halo_stride;
  long long *acc;          // [n_rep][16] pass accumulators
  const StreamRun *run;
  int sub, n_classes, n_pair_sw, n_local_sw;
  double RT[16];
};

// Class and parameters of sub-step `sub` of the pass (the schedule of the
// shared-memory sweep: rank of the class key within its sweep).
__device__ __forceinline__ void stream_schedule(const Replica &R, const CeTables &T, int ensemble,
                                                long long pass, int sub, int n_classes,
                                                int n_pair_sw, int &cls, uint32_t &par) {
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const uint32_t plo = (uint32_t)pass, phi = (uint32_t)(pass >> 32) & 0xFFFFu;
  const int sw = sub / n_classes, want = sub - sw * n_classes;
  uint32_t keys[64];
  for (int c = 0; c < n_classes; ++c) {
    const int e = sw * n_classes + c;
    keys[c] = philox4x32_10(U4{0xFFFFFFFFu - (uint32_t)e, 0u, plo, phi | (TAG_SCHED << 16)}, k0, k1).x;
  }
  cls = 0;
  for (int c = 0; c < n_classes; ++c) {
    int rank = 0;
    for (int c2 = 0; c2 < n_classes; ++c2)
      rank += (keys[c2] < keys[c]) || (keys[c2] == keys[c] && c2 < c);
    if (rank == want) cls = c;
  }
  const int e = sw * n_classes + cls;
  const U4 r = philox4x32_10(U4{0xFFFFFFFFu - (uint32_t)e, 0u, plo, phi | (TAG_SCHED << 16)}, k0, k1);
  const int half = R.L[0] / 2;
  const int dims[3] = {half, R.L[1] / 2, R.L[2] / 2};
  par = sched_param(r, ensemble, sw, n_pair_sw, dims, T.n_nb[0]);
}

template <int PITCH>
__global__ void __launch_bounds__(256) k_stream_sub(const __grid_constant__ CeTables T,
                                                    const __grid_constant__ StreamParams SP) {
  const int rep = blockIdx.y;
  const Replica &R = SP.reps[rep];
  __shared__ int s_cls;
  __shared__ uint32_t s_par;
  __shared__ long long s_red[8][16];
  __shared__ float whi[MAX_FUNCS], wlo[MAX_FUNCS];
  const long long pass = SP.stats[rep].pass;
  const int ensemble = R.ensemble;
  if (threadIdx.x == 0) {
    int c;
    uint32_t par;
    stream_schedule(R, T, ensemble, pass, SP.sub, SP.n_classes, SP.n_pair_sw, c, par);
    s_cls = c;
    s_par = par;
  }
  for (int f = threadIdx.x; f < T.n_funcs; f += blockDim.x) {
    whi[f] = T.w_hi[f];
    wlo[f] = T.w_lo[f];
  }
  __syncthreads();
  Geo G;
  G.L0 = R.L[0];
  G.L1 = R.L[1];
  G.L2 = R.L[2];
  G.R = 2;
  G.W = G.H = PITCH;
  G.V = PITCH * PITCH * (G.L2 + 4);
  int8_t *occ = SP.halo + (long long)rep * SP.halo_stride;
  const int n_uc = G.L0 * G.L1 * G.L2;
  const int c = s_cls;
  const uint32_t par = s_par;
  const int cc[3] = {c & 1, (c >> 1) & 1, (c >> 2) & 1};  // class = parities (p = 2, even L)
  const int dims[3] = {G.L0 / 2, G.L1 / 2, G.L2 / 2};
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const uint32_t plo = (uint32_t)pass, phi = (uint32_t)(pass >> 32) & 0xFFFFu;
  const uint32_t ctr_sub = (uint32_t)SP.sub;
  const float beta_f = R.beta_f;
  const int sw = SP.sub / SP.n_classes;
  const SiteEval<2, PITCH> ev{&T, nullptr, nullptr, nullptr};
  EnergyAcc<2> eacc;
  int n_prop = 0, n_acc = 0, d1 = 0;
  int dsub[4] = {0, 0, 0, 0};
  auto cxf = [&](int a, int i) { return 2 * i + cc[a]; };
  const int nthreads = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (ensemble == 0) {
    const int n = dims[0] * dims[1] * dims[2];
    for (int q = t0; q < n; q += nthreads) {
      const int ix = q % dims[0], iy = (q / dims[0]) % dims[1], iz = q / (dims[0] * dims[1]);
      const int x = cxf(0, ix), y = cxf(1, iy), z = cxf(2, iz);
      const int ad = G.addr(0, x, y, z);
      const int o_i = occ[ad];
      const int l = x + G.L0 * (y + G.L1 * z);
      const U4 r = philox4x32_10(U4{(uint32_t)l, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
      const int o_f = 1 - o_i;
      Acc<2> acc;
      acc.zero();
      ev.add(0, o_i, o_f, occ, ad, acc);
      FF d;
      const float de = sweep_de<2>(T, acc, whi, wlo, R.dmu_hi[o_i * 2 + o_f], R.dmu_lo[o_i * 2 + o_f], d);
      ++n_prop;
      if (accept_de(de, beta_f, u24(r.x))) {
        ++n_acc;
        put_site(occ, G, 0, x, y, z, (int8_t)o_f);
        eacc.add(acc, d, 0.0);
        d1 += o_f - o_i;
        dsub[sc_sublattice(x, y, z)] += o_f - o_i;
      }
    }
  } else if (sw < SP.n_pair_sw) {
    if (par != 0xFFFFFFFFu) {
      const int a = par & 3, m = (par >> 2) & 255, rot = par >> 10;
      const int na = dims[a];
      const int half = (na / (2 * m)) * m;
      int e3[3] = {dims[0], dims[1], dims[2]};
      e3[a] = half;
      const int n = e3[0] * e3[1] * e3[2];
      for (int q = t0; q < n; q += nthreads) {
        int ia[3] = {q % e3[0], (q / e3[0]) % e3[1], q / (e3[0] * e3[1])};
        int ib[3] = {ia[0], ia[1], ia[2]};
        const int jj = ia[a];
        const int u = 2 * m * (jj / m) + (jj % m);
        ia[a] = (u + rot) % na;
        ib[a] = (u + m + rot) % na;
        const int xa = cxf(0, ia[0]), ya = cxf(1, ia[1]), za = cxf(2, ia[2]);
        const int xb = cxf(0, ib[0]), yb = cxf(1, ib[1]), zb = cxf(2, ib[2]);
        const int ada = G.addr(0, xa, ya, za), adb = G.addr(0, xb, yb, zb);
        const int oa = occ[ada], ob = occ[adb];
        if (oa == ob) continue;
        const int la = xa + G.L0 * (ya + G.L1 * za);
        const U4 r = philox4x32_10(U4{(uint32_t)la, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
        Acc<2> acc;
        acc.zero();
        ev.add(0, oa, ob, occ, ada, acc);
        ev.add(0, ob, oa, occ, adb, acc);
        FF d;
        const float de = sweep_de<2>(T, acc, whi, wlo, 0.f, 0.f, d);
        ++n_prop;
        if (accept_de(de, beta_f, u24(r.x))) {
          ++n_acc;
          put_site(occ, G, 0, xa, ya, za, (int8_t)ob);
          put_site(occ, G, 0, xb, yb, zb, (int8_t)oa);
          eacc.add(acc, d, 0.0);
        }
      }
    }
  } else {
    const int parity = par & 7, dlt = (par >> 3) & 15;
    const int rots[3] = {(int)((par >> 7) & 127), (int)((par >> 14) & 127), (int)((par >> 21) & 127)};
    if (T.n_nb[0] > 0) {
      const int *du = T.nb_du[0][dlt];
      int h[3];
      for (int a = 0; a < 3; ++a) h[a] = dims[a] / 2;
      const int n = h[0] * h[1] * h[2];
      for (int q = t0; q < n; q += nthreads) {
        const int t[3] = {q % h[0], (q / h[0]) % h[1], q / (h[0] * h[1])};
        int ii[3];
        for (int a = 0; a < 3; ++a) ii[a] = (rots[a] + ((parity >> a) & 1) + 2 * t[a]) % dims[a];
        const int xa = cxf(0, ii[0]), ya = cxf(1, ii[1]), za = cxf(2, ii[2]);
        const int xb = wrapc(xa + du[0], G.L0), yb = wrapc(ya + du[1], G.L1), zb = wrapc(za + du[2], G.L2);
        const int ada = G.addr(0, xa, ya, za), adb = G.addr(0, xb, yb, zb);
        const int oa = occ[ada], ob = occ[adb];
        if (oa == ob) continue;
        const int la = xa + G.L0 * (ya + G.L1 * za);
        const U4 r = philox4x32_10(U4{(uint32_t)la, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
        Acc<2> acc;
        acc.zero();
        ev.add(0, oa, ob, occ, ada, acc);
        put_site(occ, G, 0, xa, ya, za, (int8_t)ob);
        ev.add(0, ob, oa, occ, adb, acc);
        FF d;
        const float de = sweep_de<2>(T, acc, whi, wlo, 0.f, 0.f, d);
        ++n_prop;
        if (accept_de(de, beta_f, u24(r.x))) {
          ++n_acc;
          put_site(occ, G, 0, xb, yb, zb, (int8_t)oa);
          eacc.add(acc, d, 0.0);
          dsub[sc_sublattice(xa, ya, za)] += ob - oa;
          dsub[sc_sublattice(xb, yb, zb)] += oa - ob;
        } else {
          put_site(occ, G, 0, xa, ya, za, (int8_t)oa);
        }
      }
    }
  }
  // block reduce -> per-replica accumulators
  long long vals[16];
  for (int k = 0; k < 16; ++k) vals[k] = 0;
  vals[0] = n_prop;
  vals[1] = n_acc;
  vals[2] = d1;
  for (int k = 0; k < 4; ++k) vals[4 + k] = dsub[k];
  for (int g = 0; g < MAX_ORBITS; ++g) vals[8 + g] = eacc.dc[g];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 16; ++k)
    for (int off = 16; off; off >>= 1) vals[k] += __shfl_xor_sync(0xffffffffu, vals[k], off);
  if (lane == 0)
    for (int k = 0; k < 16; ++k) s_red[warp][k] = vals[k];
  __syncthreads();
  if (threadIdx.x < 16) {
    long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w][threadIdx.x];
    if (t) atomicAdd((unsigned long long *)&SP.acc[rep * 16 + threadIdx.x], (unsigned long long)t);
  }
  (void)n_uc;
}

// End of pass: one thread per replica.
__global__ void k_stream_end(const __grid_constant__ CeTables T, const __grid_constant__ StreamParams SP,
                             int n_rep) {
  const int rep = blockIdx.x * blockDim.x + threadIdx.x;
  if (rep >= n_rep) return;
  const Replica &R = SP.reps[rep];
  ReplicaStats &S = SP.stats[rep];
  long long *a = SP.acc + rep * 16;
  const int n_sites = R.n_sites, n_uc = R.L[0] * R.L[1] * R.L[2];
  double de = 0.0;
  for (int g = 0; g < T.n_orbits; ++g) de += T.w[T.orb_func_base[g]] * (double)a[8 + g];
  S.energy += de;
  S.n_proposed += a[0];
  S.n_accepted += a[1];
  S.n_species[1] += a[2];
  S.n_species[0] -= a[2];
  for (int k = 0; k < 4; ++k) S.n_sub[k] += a[4 + k];
  for (int k = 0; k < 16; ++k) a[k] = 0;
  const StreamRun &run = *SP.run;
  const long long ip = S.pass - run.start_pass;
  double xs[3] = {0.0, 0.0, 0.0}, ef, ep;
  const long long nspec[2] = {S.n_species[0], S.n_species[1]};
  sample_values<2>(SP.RT, R.mu, nspec, n_sites, n_uc, S.energy, xs, ef, ep);
  const double xu = xs[0];
  double op = 0.0;
  const double xb = (double)S.n_species[1] / n_sites;
  for (int k = 0; k < 4; ++k) {
    const double c = (double)S.n_sub[k] / (0.25 * n_sites) - xb;
    op += c * c;
  }
  op = sqrt(op);
  if (ip >= run.n_equil) {
    S.n_samples += 1.0;
    S.sum_e += ep;
    S.sum_e2 += ep * ep;
    S.sum_f += ef;
    S.sum_x[0] += xu;
    S.sum_xx[0] += xu * xu;
    S.sum_ex[0] += ep * xu;
    if (run.samples) {
      const long long si = (long long)S.n_samples - 1;
      if (si < run.sample_capacity) {
        double *out = run.samples + ((long long)rep * run.sample_capacity + si) * run.sample_width;
        out[0] = ep;
        out[1] = xu;
        out[2] = op;
      }
    }
  }
  S.pass += 1;
}

// packed occupations <-> halo blocks; sublattice counts on the way in
template <int PITCH>
__global__ void k_halo_fill(const Replica *reps, const int8_t *occ_all, int8_t *halo,
                            long long stride, ReplicaStats *stats, int count_sub) {
  const int rep = blockIdx.y;
  const Replica &R = reps[rep];
  const int L0 = R.L[0], L1 = R.L[1], L2 = R.L[2];
  const int D = L2 + 4;
  const long long V = (long long)PITCH * PITCH * D;
  int8_t *h = halo + rep * stride;
  const int8_t *o = occ_all + R.occ_offset;
  __shared__ unsigned long long sub[4];
  if (threadIdx.x < 4) sub[threadIdx.x] = 0;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < V;
       i += (long long)gridDim.x * blockDim.x) {
    const int xh = (int)(i % PITCH), yh = (int)((i / PITCH) % PITCH), zh = (int)(i / ((long long)PITCH * PITCH));
    const int x = xh - 2, y = yh - 2, z = zh - 2;
    if (x >= L0 + 2 || y >= L1 + 2) continue;
    const int v = o[wrapc(x, L0) + L0 * (wrapc(y, L1) + L1 * wrapc(z, L2))];
    h[i] = (int8_t)v;
    if (count_sub && v && x >= 0 && x < L0 && y >= 0 && y < L1 && z >= 0 && z < L2)
      atomicAdd(&sub[sc_sublattice(x, y, z)], 1ull);
  }
  __syncthreads();
  if (count_sub && threadIdx.x < 4)
    atomicAdd((unsigned long long *)&stats[rep].n_sub[threadIdx.x], sub[threadIdx.x]);
}

template <int PITCH>
__global__ void k_halo_store(const Replica *reps, int8_t *occ_all, const int8_t *halo,
                             long long stride) {
  const int rep = blockIdx.y;
  const Replica &R = reps[rep];
  const int L0 = R.L[0], L1 = R.L[1], L2 = R.L[2];
  const int n = L0 * L1 * L2;
  const int8_t *h = halo + rep * stride;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x) {
    const int x = l % L0, y = (l / L0) % L1, z = l / (L0 * L1);
    occ_all[R.occ_offset + l] = h[(x + 2) + PITCH * ((y + 2) + PITCH * (z + 2))];
  }
}

// ----------------------------------------------------------------- host side
long long stream_halo_bytes(int L2, int pitch) { return (long long)pitch * pitch * (L2 + 4); }

template <int PITCH>
static cudaError_t stream_run_t(const CeTables &T, StreamState &st, const Replica *reps,
                                ReplicaStats *stats, int8_t *occ_all, int n_rep, int L2,
                                int n_classes, int n_pair_sw, int n_local_sw, const double *RT,
                                long long n_passes, long long n_equil, long long start_pass,
                                double *samples, long long capacity, int width, int count_sub,
                                cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1) {
  cudaError_t e;
  const long long stride = stream_halo_bytes(L2, PITCH);
  // run parameters (device)
  StreamRun run{n_equil, start_pass, samples, capacity, width, 0};
  if ((e = cudaMemcpyAsync(st.run, &run, sizeof(run), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(st.acc, 0, sizeof(long long) * 16 * n_rep, s)) != cudaSuccess) return e;
  dim3 g2(1024, n_rep);
  k_halo_fill<PITCH><<<g2, 256, 0, s>>>(reps, occ_all, st.halo, stride, stats, count_sub);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int n_sub = (n_pair_sw + n_local_sw) * n_classes;
  const int key = n_sub * 1000 + n_classes * 10 + n_pair_sw;
  if (!st.exec || st.key != key) {
    if (st.exec) cudaGraphExecDestroy(st.exec);
    st.exec = nullptr;
    StreamParams SP{};
    SP.reps = reps;
    SP.stats = stats;
    SP.halo = st.halo;
    SP.halo_stride = stride;
    SP.acc = st.acc;
    SP.run = st.run;
    SP.n_classes = n_classes;
    SP.n_pair_sw = n_pair_sw;
    SP.n_local_sw = n_local_sw;
    for (int k = 0; k < 16; ++k) SP.RT[k] = RT[k];
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    const int blocks = 304;  // 2 x 152 SMs of CTAs per replica and sub-step
    for (int sub = 0; sub < n_sub; ++sub) {
      SP.sub = sub;
      k_stream_sub<PITCH><<<dim3(blocks / n_rep > 0 ? blocks / n_rep : 1, n_rep), 256, 0, s>>>(T, SP);
    }
    k_stream_end<<<(n_rep + 63) / 64, 64, 0, s>>>(T, SP, n_rep);
    if ((e = cudaStreamEndCapture(s, &graph)) != cudaSuccess) return e;
    e = cudaGraphInstantiate(&st.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    st.key = key;
  }
  if ((e = cudaEventRecord(ev0, s)) != cudaSuccess) return e;
  for (long long p = 0; p < n_passes; ++p)
    if ((e = cudaGraphLaunch(st.exec, s)) != cudaSuccess) return e;
  if ((e = cudaEventRecord(ev1, s)) != cudaSuccess) return e;
  k_halo_store<PITCH><<<g2, 256, 0, s>>>(reps, occ_all, st.halo, stride);
  return cudaGetLastError();
}

cudaError_t stream_run(const CeTables &T, StreamState &st, const Replica *reps, ReplicaStats *stats,
                       int8_t *occ_all, int n_rep, int L2, int pitch, int n_classes, int n_pair_sw,
                       int n_local_sw, const double *RT, long long n_passes, long long n_equil,
                       long long start_pass, double *samples, long long capacity, int width,
                       int count_sub, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1) {
  switch (pitch) {
    case 100:
      return stream_run_t<100>(T, st, reps, stats, occ_all, n_rep, L2, n_classes, n_pair_sw,
                               n_local_sw, RT, n_passes, n_equil, start_pass, samples, capacity,
                               width, count_sub, s, ev0, ev1);
    case 28:
      return stream_run_t<28>(T, st, reps, stats, occ_all, n_rep, L2, n_classes, n_pair_sw,
                              n_local_sw, RT, n_passes, n_equil, start_pass, samples, capacity,
                              width, count_sub, s, ev0, ev1);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace cem
