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
  int2 *sched;             // [n_rep][n_sub]: (class, parameters) of each sub-step
  int sub, n_sub, n_classes, n_pair_sw, n_local_sw;
  double RT[16];
};

// A CTA's share of a sub-step's candidate grid (g0 x g1 x g2, x fastest):
// full x rows over a (y, z) tile of a grid of ny x nz tiles, ny nz <= the
// CTAs per replica. A box of rows keeps the neighbour reads of a CTA local
// (a slab of contiguous candidates would span whole planes and read each
// plane's halo rows again in the next CTA). Candidate ql of the tile, ql <
// count, is cell (ql mod g0, y0 + (ql / g0) mod cy, z0 + ql / (g0 cy)).
struct StreamTile {
  int y0, z0, cy, cz, count;
  __device__ StreamTile(int g0, int g1, int g2) {
    const int nb = gridDim.x;
    int nz = 1;
    while ((nz + 1) * (nz + 1) <= nb) ++nz;
    const int ny = nb / nz;
    const int ty = (g1 + ny - 1) / ny, tz = (g2 + nz - 1) / nz;
    const int b = blockIdx.x, by = b % ny, bz = b / ny;
    y0 = by * ty;
    z0 = bz * tz;
    cy = (b < ny * nz) ? max(0, min(g1, y0 + ty) - y0) : 0;
    cz = (b < ny * nz) ? max(0, min(g2, z0 + tz) - z0) : 0;
    count = g0 * cy * cz;
  }
};

// Schedule of a pass (the shared-memory sweep's: class order by key rank
// within each sweep, parameters per class): one CTA per replica, one thread
// per (sweep, class).
__global__ void k_stream_sched(const __grid_constant__ CeTables T,
                               const __grid_constant__ StreamParams SP) {
  const int rep = blockIdx.x;
  const Replica &R = SP.reps[rep];
  const long long pass = SP.stats[rep].pass;
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const uint32_t plo = (uint32_t)pass, phi = (uint32_t)(pass >> 32) & 0xFFFFu;
  const int nc = SP.n_classes;
  const int dims[3] = {R.L[0] / 2, R.L[1] / 2, R.L[2] / 2};
  for (int e = threadIdx.x; e < SP.n_sub; e += blockDim.x) {
    const int sw = e / nc, c = e - sw * nc;
    const U4 r = philox4x32_10(U4{0xFFFFFFFFu - (uint32_t)e, 0u, plo, phi | (TAG_SCHED << 16)}, k0, k1);
    int rank = 0;
    for (int c2 = 0; c2 < nc; ++c2) {
      const uint32_t k2 = philox4x32_10(
          U4{0xFFFFFFFFu - (uint32_t)(sw * nc + c2), 0u, plo, phi | (TAG_SCHED << 16)}, k0, k1).x;
      rank += (k2 < r.x) || (k2 == r.x && c2 < c);
    }
    const uint32_t par = sched_param(r, R.ensemble, sw, SP.n_pair_sw, dims, T.n_nb[0]);
    SP.sched[(long long)rep * SP.n_sub + sw * nc + rank] = make_int2(c, (int)par);
  }
}

// One colour sub-step of every replica; the class's candidates are split
// into contiguous chunks, one per CTA. Canonical sub-steps compact the
// candidate pairs whose occupants differ (the proposals) per warp, then
// spread them over the CTA, as the shared-memory sweep does.
template <int PITCH>
__global__ void __launch_bounds__(256) k_stream_sub(const __grid_constant__ CeTables T,
                                                    const __grid_constant__ StreamParams SP) {
  extern __shared__ int s_list[];  // kept candidates of this CTA
  __shared__ int s_kept[8];
  __shared__ long long s_red[8][16];
  const int rep = blockIdx.y;
  const Replica &R = SP.reps[rep];
  const long long pass = SP.stats[rep].pass;
  const int ensemble = R.ensemble;
  const int2 sc = SP.sched[(long long)rep * SP.n_sub + SP.sub];
  const int c = sc.x;
  const uint32_t par = (uint32_t)sc.y;
  Geo G;
  G.L0 = R.L[0];
  G.L1 = R.L[1];
  G.L2 = R.L[2];
  G.R = 2;
  G.W = G.H = PITCH;
  G.V = PITCH * PITCH * (G.L2 + 4);
  int8_t *occ = SP.halo + (long long)rep * SP.halo_stride;
  const int cc0 = c & 1, cc1 = (c >> 1) & 1, cc2 = (c >> 2) & 1;  // class = parities (p = 2, even L)
  const int d0 = G.L0 / 2, d1 = G.L1 / 2, d2 = G.L2 / 2;
  const uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32);
  const uint32_t plo = (uint32_t)pass, phi = (uint32_t)(pass >> 32) & 0xFFFFu;
  const uint32_t ctr_sub = (uint32_t)SP.sub;
  const float beta_f = R.beta_f;
  const int sw = SP.sub / SP.n_classes;
  const SiteEval<2, PITCH> ev{&T, nullptr, nullptr, nullptr};
  EnergyAcc<2> eacc;
  int n_prop = 0, n_acc = 0, d1sum = 0;
  RegCounts<4> dsub;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto wrap_lt2 = [](int v, int L) { return v >= L ? v - L : v; };  // v < 2L
  if (ensemble == 0) {
    // ---------------- flips: every class site is a proposal
    const StreamTile tile(d0, d1, d2);
    const FastDiv f0(d0), fy(max(1, tile.cy));
    for (int q = threadIdx.x; q < tile.count; q += blockDim.x) {
      const int t = f0.div(q), tz = fy.div(t);
      const int x = 2 * (q - t * d0) + cc0, y = 2 * (tile.y0 + t - tz * tile.cy) + cc1,
                z = 2 * (tile.z0 + tz) + cc2;
      const int ad = G.addr(0, x, y, z);
      const int o_i = occ[ad];
      const int l = x + G.L0 * (y + G.L1 * z);
      const U4 r = philox4x32_10(U4{(uint32_t)l, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
      const int o_f = 1 - o_i;
      Acc<2> acc;
      acc.zero();
      ev.add(0, o_i, o_f, occ, ad, acc);
      FF d;
      const float de = sweep_de<2>(T, acc, nullptr, nullptr, R.dmu_hi[o_i * 2 + o_f],
                                   R.dmu_lo[o_i * 2 + o_f], d);
      ++n_prop;
      if (accept_de(de, beta_f, u24(r.x))) {
        ++n_acc;
        put_site(occ, G, 0, x, y, z, (int8_t)o_f);
        eacc.add(acc, d, 0.0);
        d1sum += o_f - o_i;
        dsub.add(sc_sublattice(x, y, z), o_f - o_i);
      }
    }
  } else {
    // ---------------- canonical: pairs inside the class or neighbour swaps
    const bool local = sw >= SP.n_pair_sw;
    int n = 0, g0 = 1, g1 = 1, pa = 0, pm = 1, prot = 0, pna = 1;
    int parity = 0, r0 = 0, r1 = 0, r2 = 0, du0 = 0, du1 = 0, du2 = 0;
    if (!local) {
      if (par != 0xFFFFFFFFu) {
        pa = par & 3;
        pm = (par >> 2) & 255;
        prot = (int)(par >> 10);
        pna = pa == 0 ? d0 : (pa == 1 ? d1 : d2);
        const int half = (pna / (2 * pm)) * pm;
        g0 = pa == 0 ? half : d0;
        g1 = pa == 1 ? half : d1;
        n = g0 * g1 * (pa == 2 ? half : d2);
      }
    } else if (T.n_nb[0] > 0) {
      parity = par & 7;
      const int dlt = (par >> 3) & 15;
      r0 = (int)((par >> 7) & 127);
      r1 = (int)((par >> 14) & 127);
      r2 = (int)((par >> 21) & 127);
      du0 = T.nb_du[0][dlt][0];
      du1 = T.nb_du[0][dlt][1];
      du2 = T.nb_du[0][dlt][2];
      g0 = d0 / 2;
      g1 = d1 / 2;
      n = g0 * g1 * (d2 / 2);
    }
    const int g2 = g1 > 0 && g0 > 0 ? n / (g0 * g1) : 0;
    const StreamTile tile(g0, g1, g2);
    const FastDiv fe0(g0), fey(max(1, tile.cy)), fpm(pm);
    auto sites_of = [&](int q, int &xa, int &ya, int &za, int &xb, int &yb, int &zb) {
      const int t = fe0.div(q), tz = fey.div(t);
      const int i0 = q - t * g0, i1 = tile.y0 + t - tz * tile.cy, i2 = tile.z0 + tz;
      if (!local) {
        const int jj = pa == 0 ? i0 : (pa == 1 ? i1 : i2);
        const int jq = fpm.div(jj);
        const int u = 2 * pm * jq + (jj - jq * pm);
        const int ja = wrap_lt2(u + prot, pna), jb = wrap_lt2(u + pm + prot, pna);
        xa = 2 * (pa == 0 ? ja : i0) + cc0;
        xb = 2 * (pa == 0 ? jb : i0) + cc0;
        ya = 2 * (pa == 1 ? ja : i1) + cc1;
        yb = 2 * (pa == 1 ? jb : i1) + cc1;
        za = 2 * (pa == 2 ? ja : i2) + cc2;
        zb = 2 * (pa == 2 ? jb : i2) + cc2;
      } else {
        xa = 2 * wrap_lt2(r0 + (parity & 1) + 2 * i0, d0) + cc0;
        ya = 2 * wrap_lt2(r1 + ((parity >> 1) & 1) + 2 * i1, d1) + cc1;
        za = 2 * wrap_lt2(r2 + ((parity >> 2) & 1) + 2 * i2, d2) + cc2;
        xb = wrapc(xa + du0, G.L0);
        yb = wrapc(ya + du1, G.L1);
        zb = wrapc(za + du2, G.L2);
      }
    };
    // phase A: this CTA's tile, split between its warps, compacted in order
    const int per = tile.count;
    const int nw = blockDim.x >> 5;
    const int wper = (per + nw - 1) / nw;
    const int wq0 = warp * wper, wq1 = min(per, wq0 + wper);
    int kept = 0;
    for (int qb = wq0; qb < wq1; qb += 32) {
      const int q = qb + lane;
      bool act = false;
      if (q < wq1) {
        int xa, ya, za, xb, yb, zb;
        sites_of(q, xa, ya, za, xb, yb, zb);
        act = occ[G.addr(0, xa, ya, za)] != occ[G.addr(0, xb, yb, zb)];
      }
      const unsigned m = __ballot_sync(0xffffffffu, act);
      if (act) s_list[warp * wper + kept + __popc(m & ((1u << lane) - 1u))] = q;
      kept += __popc(m);
    }
    if (lane == 0) s_kept[warp] = kept;
    __syncthreads();
    // phase B: kept pair i of the CTA goes to thread i mod block size
    int total = 0;
    for (int w = 0; w < nw; ++w) total += s_kept[w];
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      int wsel = 0, bsel = 0, run = 0;
      for (int w = 0; w < nw; ++w) {
        const int k = s_kept[w];
        if (i >= run) {
          wsel = w;
          bsel = run;
        }
        run += k;
      }
      const int q = s_list[wsel * wper + (i - bsel)];
      int xa, ya, za, xb, yb, zb;
      sites_of(q, xa, ya, za, xb, yb, zb);
      const int ada = G.addr(0, xa, ya, za), adb = G.addr(0, xb, yb, zb);
      const int oa = occ[ada], ob = occ[adb];
      const int la = xa + G.L0 * (ya + G.L1 * za);
      const U4 r = philox4x32_10(U4{(uint32_t)la, ctr_sub, plo, phi | (TAG_SITE << 16)}, k0, k1);
      Acc<2> acc;
      acc.zero();
      ev.add(0, oa, ob, occ, ada, acc);
      if (local) put_site(occ, G, 0, xa, ya, za, (int8_t)ob);  // first change applied
      ev.add(0, ob, oa, occ, adb, acc);
      FF d;
      const float de = sweep_de<2>(T, acc, nullptr, nullptr, 0.f, 0.f, d);
      ++n_prop;
      if (accept_de(de, beta_f, u24(r.x))) {
        ++n_acc;
        if (!local) put_site(occ, G, 0, xa, ya, za, (int8_t)ob);
        put_site(occ, G, 0, xb, yb, zb, (int8_t)oa);
        eacc.add(acc, d, 0.0);
        dsub.add(sc_sublattice(xa, ya, za), ob - oa);
        dsub.add(sc_sublattice(xb, yb, zb), oa - ob);
      } else if (local) {
        put_site(occ, G, 0, xa, ya, za, (int8_t)oa);
      }
    }
  }
  // block reduce -> per-replica accumulators
  long long vals[16];
  for (int k = 0; k < 16; ++k) vals[k] = 0;
  vals[0] = n_prop;
  vals[1] = n_acc;
  vals[2] = d1sum;
#pragma unroll
  for (int k = 0; k < 4; ++k) vals[4 + k] = dsub.v[k];
  for (int g = 0; g < MAX_ORBITS; ++g) vals[8 + g] = eacc.dc[g];
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
                                cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1,
                                const volatile int *stop_host, long long *launched) {
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
  if (st.sched_cap < n_sub) {
    cudaFree(st.sched);
    st.sched = nullptr;
    if ((e = cudaMalloc(&st.sched, sizeof(int2) * n_sub * n_rep)) != cudaSuccess) return e;
    st.sched_cap = n_sub;
    if (st.exec) cudaGraphExecDestroy(st.exec);
    st.exec = nullptr;
  }
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
    SP.sched = st.sched;
    SP.n_sub = n_sub;
    SP.n_classes = n_classes;
    SP.n_pair_sw = n_pair_sw;
    SP.n_local_sw = n_local_sw;
    for (int k = 0; k < 16; ++k) SP.RT[k] = RT[k];
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    const int blocks = 304;  // 2 x 152 SMs of CTAs per sub-step, over all replicas
    // candidates per CTA: at most (L/2)^3 per class, split into bx chunks
    // of at most 8192 (their list stays below 48 KB of shared memory), plus
    // rounding of the per-warp chunks
    const long long half = L2 / 2, n_max = half * half * half;
    int bx = blocks / n_rep > 0 ? blocks / n_rep : 1;
    if (bx < (n_max + 8191) / 8192) bx = (int)((n_max + 8191) / 8192);
    // list capacity: the largest tile (full x rows of the candidate grid over
    // a y, z tile; the grid is at most (L/2)^3), split over 8 warps
    int nz = 1;
    while ((nz + 1) * (nz + 1) <= bx) ++nz;
    const int ny = bx / nz;
    const long long tile_max = half * ((half + ny - 1) / ny) * ((half + nz - 1) / nz);
    const int smem = (int)(4 * (8 * ((tile_max + 7) / 8) + 8));
    k_stream_sched<<<n_rep, 64, 0, s>>>(T, SP);
    for (int sub = 0; sub < n_sub; ++sub) {
      SP.sub = sub;
      k_stream_sub<PITCH><<<dim3(bx, n_rep), 256, smem, s>>>(T, SP);
    }
    k_stream_end<<<(n_rep + 63) / 64, 64, 0, s>>>(T, SP, n_rep);
    if ((e = cudaStreamEndCapture(s, &graph)) != cudaSuccess) return e;
    e = cudaGraphInstantiate(&st.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    st.key = key;
  }
  if ((e = cudaEventRecord(ev0, s)) != cudaSuccess) return e;
  // one graph per pass; a stop request of the host ends the queueing (the
  // launch queue fills up on long runs, so the check sees it within the
  // passes already queued)
  long long p = 0;
  for (; p < n_passes; ++p) {
    if (stop_host && *stop_host) break;
    if ((e = cudaGraphLaunch(st.exec, s)) != cudaSuccess) return e;
  }
  if (launched) *launched = p;
  if ((e = cudaEventRecord(ev1, s)) != cudaSuccess) return e;
  k_halo_store<PITCH><<<g2, 256, 0, s>>>(reps, occ_all, st.halo, stride);
  return cudaGetLastError();
}

cudaError_t stream_run(const CeTables &T, StreamState &st, const Replica *reps, ReplicaStats *stats,
                       int8_t *occ_all, int n_rep, int L2, int pitch, int n_classes, int n_pair_sw,
                       int n_local_sw, const double *RT, long long n_passes, long long n_equil,
                       long long start_pass, double *samples, long long capacity, int width,
                       int count_sub, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1,
                       const volatile int *stop_host, long long *launched) {
  switch (pitch) {
    case 100:
      return stream_run_t<100>(T, st, reps, stats, occ_all, n_rep, L2, n_classes, n_pair_sw,
                               n_local_sw, RT, n_passes, n_equil, start_pass, samples, capacity,
                               width, count_sub, s, ev0, ev1, stop_host, launched);
    case 28:
      return stream_run_t<28>(T, st, reps, stats, occ_all, n_rep, L2, n_classes, n_pair_sw,
                              n_local_sw, RT, n_passes, n_equil, start_pass, samples, capacity,
                              width, count_sub, s, ev0, ev1, stop_host, launched);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace cem
