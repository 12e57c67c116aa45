// C ABI of the GB300 Metropolis hot path: object lifetimes, validation,
// transfers and launches. See include/cem.h for the contract.
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cem.h"
#include "cem_common.cuh"
#include "cem_internal.h"
#include "cem_learned.cuh"

using namespace cem;

namespace {

thread_local std::string g_error;

struct Err : std::runtime_error {
  int code;
  Err(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define CUDA_OK(x)                                                                    \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess)                                                            \
      throw Err(CEM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));      \
  } while (0)

// NVTX range over a host call (shows the library's runs on a profiler's
// timeline; costs nothing when no tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

template <class F>
int guard(F &&f) {
  try {
    f();
    return CEM_OK;
  } catch (Err &e) {
    g_error = e.what();
    return e.code;
  } catch (std::exception &e) {
    g_error = e.what();
    return CEM_ERR_INVALID;
  }
}

void require(bool ok, const std::string &msg, int code = CEM_ERR_INVALID) {
  if (!ok) throw Err(code, msg);
}

template <class T>
T *dev_copy(const std::vector<T> &v) {
  T *p = nullptr;
  if (v.empty()) return nullptr;
  CUDA_OK(cudaMalloc(&p, sizeof(T) * v.size()));
  CUDA_OK(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return p;
}

const double KB = 8.617333262e-5;  // eV/K
constexpr int MAX_SWEEPS_API = 8;

// block colouring of a ring of length L with blocks of size >= p
std::vector<int> axis_blocks(int L, int p) {
  int q = L / p;
  if (q == 0) return {};
  std::vector<int> sizes(q, p);
  int extra = L - q * p;
  for (int r = 0; r < extra; ++r) sizes[r % q] += 1;
  std::vector<int> col;
  for (int s : sizes)
    for (int t = 0; t < s; ++t) col.push_back(t);
  return col;
}

}  // namespace

struct cem_system {
  CeTables T{};
  int n_flower = 0, n_owned = 0;
  std::vector<double> w;
  std::vector<double> RT;
  // host copies used for colouring checks
  std::vector<int> fl_sub, fl_pb, fl_du;
  int nb_reach = 0;
  bool swaps_connect = false;  // local-swap displacements connect every site (canonical ergodicity)
  bool fcc_generated = false;  // flower matches the generated binary FCC evaluator
  bool big = false;            // more orbits than the register accumulators hold
  bool coop = false;           // big binary system for the warp-cooperative sweep
  bool split_ok = false;       // binary, split weights exist, orbits sorted by size
  std::vector<int> wq_host;    // split weights' integer parts per orbit
  std::vector<void *> owned;
  ~cem_system() {
    for (void *p : owned) cudaFree(p);
  }
};

struct cem_replicas {
  const cem_system *sys = nullptr;
  int n = 0, ensemble = 0;
  int device = 0;  // the device current when the batch was created
  // stop flag of the running sweep: page-locked host memory mapped into the
  // device's address space; the persistent kernels read it once per pass
  volatile int *h_stop = nullptr;
  int *d_stop = nullptr;
  std::vector<Replica> reps;
  std::vector<ReplicaStats> stats_host;
  Replica *d_reps = nullptr;
  ReplicaStats *d_stats = nullptr;
  int8_t *d_occ = nullptr;
  int64_t total_sites = 0;
  unsigned long long *d_counts = nullptr;  // scratch [n_funcs]
  long long *d_result = nullptr;
  double *d_samples = nullptr;
  long long sample_capacity = 0;
  int sample_width = 1;
  long long n_samples_recorded = 0;
  int max_classes = 1, sweep_smem = 0, pitch = 0;
  bool wide_records = false;  // cooperative sweep: keep 32-bit cluster records
  int n_pair_sweeps = 2, n_local_sweeps = 1;
  int threads = SWEEP_THREADS;
  // replica -> CTA schedule: 0 = CTA i runs replica i, 1 = largest replicas first
  int cta_order = 0;
  // CTAs per replica of the learned group sweep (0 automatic) and the last used
  int group_cluster = 0, last_group_cluster = 0;
  // CTAs per replica of the plain sweep (0 automatic) and the last used
  int sweep_cluster = 0, last_sweep_cluster = 1;
  int *d_cta_rep = nullptr;
  bool reps_dirty = true, stats_valid = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  // some replica is a non-diagonal supercell; the parallel sweep then runs
  // only for semi-grand batches whose twisted replicas all have a colouring,
  // on the run-time tables, one CTA per replica, shared memory
  bool twisted = false, twisted_parallel = true;
  // HBM-streamed batches (supercells too large for shared memory)
  bool streamed = false;
  int stream_pitch = 0;
  StreamState sstate;
  // end-to-end step graph (copy in, passes, copy out), captured per key
  cudaGraphExec_t step_exec = nullptr;
  const void *step_in = nullptr;
  void *step_out = nullptr;
  long long step_passes = -1;
  int step_threads = 0, step_order = -1, step_pitch = -1, step_pair = -1, step_local = -1,
      step_cluster = -1;
  long long stream_pass = 0;
  // learned-proposal state
  long long *d_lw = nullptr;             // per-site integer weights
  unsigned long long *d_trees = nullptr; // two sum trees per replica
  double *d_lsamples = nullptr;          // [rep][cap][3]
  long long lsample_capacity = 0, lsamples_recorded = 0;
  // n-fold way: per-replica rate trees
  double *d_nftree = nullptr;
  long long *d_nftree_off = nullptr;
  ~cem_replicas() {
    cudaFree(sstate.halo);
    cudaFree(sstate.acc);
    cudaFree(sstate.run);
    cudaFree(sstate.sched);
    if (sstate.exec) cudaGraphExecDestroy(sstate.exec);
    if (step_exec) cudaGraphExecDestroy(step_exec);
    cudaFree(d_lw);
    cudaFree(d_trees);
    cudaFree(d_lsamples);
    cudaFree(d_nftree);
    cudaFree(d_cta_rep);
    cudaFree(d_nftree_off);
    cudaFree(d_reps);
    cudaFree(d_stats);
    cudaFree(d_occ);
    cudaFree(d_counts);
    cudaFree(d_result);
    cudaFree(d_samples);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    if (h_stop) cudaFreeHost(const_cast<int *>(h_stop));
  }
  void upload_reps() {
    if (!reps_dirty) return;
    CUDA_OK(cudaMemcpyAsync(d_reps, reps.data(), sizeof(Replica) * n, cudaMemcpyHostToDevice,
                            stream));
    reps_dirty = false;
  }
};

namespace {

// Index in Z^3 of the lattice spanned by integer 3-vectors (0 below rank 3):
// integer row echelon form by Euclid's algorithm, |product of the pivots|.
long long lattice_index(std::vector<std::array<long long, 3>> rows) {
  long long det = 1;
  for (int col = 0; col < 3; ++col) {
    std::vector<std::array<long long, 3>> rest;
    bool have = false;
    std::array<long long, 3> piv{};
    for (auto r : rows) {
      if (r[0] == 0 && r[1] == 0 && r[2] == 0) continue;
      if (r[col] == 0) {
        rest.push_back(r);
      } else if (!have) {
        piv = r;
        have = true;
      } else {
        auto a = piv, b = r;
        while (b[col] != 0) {
          const long long q = a[col] / b[col];  // any quotient reduces |remainder| below |b[col]|
          for (int k = 0; k < 3; ++k) a[k] -= q * b[k];
          std::swap(a, b);
        }
        piv = a;
        rest.push_back(b);
      }
    }
    if (!have) return 0;
    det *= piv[col];
    rows.swap(rest);
  }
  return det < 0 ? -det : det;
}

// Whether swaps of site (b, x) with (nb_b, x + nb_du) connect every site of
// every sublattice on the infinite lattice: the graph over the sublattices is
// connected and the translations of its cycles generate Z^3. Swaps inside a
// colour class only permute the class, so this is what makes the canonical
// chain ergodic.
bool swaps_connect(const CeTables &T) {
  const int ns = T.n_sublat;
  std::vector<std::array<long long, 3>> pot(ns);
  std::vector<int> seen(ns, 0), stack{0};
  seen[0] = 1;
  pot[0] = {0, 0, 0};
  while (!stack.empty()) {
    const int b = stack.back();
    stack.pop_back();
    for (int b2 = 0; b2 < ns; ++b2)
      for (int k = 0; k < T.n_nb[b2]; ++k) {
        const int pb = T.nb_b[b2][k];
        const int *du = T.nb_du[b2][k];
        int from = -1, to = -1, sgn = 1;
        if (b2 == b && !seen[pb]) from = b, to = pb, sgn = 1;
        else if (pb == b && !seen[b2]) from = b, to = b2, sgn = -1;
        if (from < 0) continue;
        for (int a = 0; a < 3; ++a) pot[to][a] = pot[from][a] + sgn * du[a];
        seen[to] = 1;
        stack.push_back(to);
      }
  }
  for (int b = 0; b < ns; ++b)
    if (!seen[b]) return false;
  std::vector<std::array<long long, 3>> cycles;
  for (int b = 0; b < ns; ++b)
    for (int k = 0; k < T.n_nb[b]; ++k) {
      const int pb = T.nb_b[b][k];
      std::array<long long, 3> v;
      for (int a = 0; a < 3; ++a) v[a] = pot[b][a] + T.nb_du[b][k][a] - pot[pb][a];
      cycles.push_back(v);
    }
  return lattice_index(cycles) == 1;
}

// HBM-streamed mode: binary FCC of the generated topology, equal even cubic
// supercells whose pitch L + 4 has a compiled kernel
int stream_pitch_for(const cem_system &s, const std::vector<Replica> &reps) {
  if (!s.fcc_generated) return 0;
  const int L = reps[0].L[0];
  for (const Replica &R : reps)
    if (R.L[0] != L || R.L[1] != L || R.L[2] != L || (L & 1) || R.p != 2) return 0;
  return (L + 4 == 100 || L + 4 == 28) ? L + 4 : 0;
}

// CTAs per replica of the plain sweep: a thread-block cluster sharing each
// sub-step for the generated binary evaluator at 512 threads per replica.
// Automatic: the largest of 4, 2 that keeps every replica's cluster on its
// own SMs and leaves each CTA at least 20 000 sites of the replica, else 1
// (measured on 32 replicas at 90 K: 48^3 runs 1.44x faster on 4 CTAs, 24^3
// 1.3x slower, the cluster barriers then costing more than the work saved)
int sweep_cluster_for(int requested, int pitch, int threads, const std::vector<Replica> &reps) {
  if (pitch <= 0 || threads != SWEEP_THREADS) return 1;
  if (requested > 0) return requested;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  int min_sites = reps.empty() ? 0 : reps[0].n_sites;
  for (const Replica &R : reps) min_sites = std::min(min_sites, R.n_sites);
  const int n_rep = (int)reps.size();
  for (int c : {4, 2})
    if (n_rep * c <= sms && min_sites >= 20000 * c) return c;
  return 1;
}

// smallest block size whose colour classes hold no two interacting sites;
// canonical local pair moves also need 2p - reach(neighbour) > reach(flower).
// tw: the twists of a supercell in Hermite normal form (null: diagonal); the
// check follows every flower partner through the supercell's own periodicity,
// so a colouring it accepts is valid on the twisted box too.
int choose_colouring(const cem_system &s, const int L[3], int ensemble, const int *tw = nullptr) {
  const CeTables &T = s.T;
  const int n_uc = L[0] * L[1] * L[2];
  const Cells C{L[0], L[1], L[2], tw ? tw[0] : 0, tw ? tw[1] : 0, tw ? tw[2] : 0};
  for (int p = 2; p <= 8; ++p) {
    std::vector<int> col[3];
    bool ok = true;
    int ncol[3];
    for (int a = 0; a < 3; ++a) {
      col[a] = axis_blocks(L[a], p);
      if (col[a].empty()) ok = false;
      else ncol[a] = *std::max_element(col[a].begin(), col[a].end()) + 1;
      if (ok && ncol[a] > MAX_COLOURS) ok = false;
    }
    if (!ok) break;
    if (ensemble == CEM_CANONICAL && 2 * p - s.nb_reach <= T.reach) continue;
    auto cls = [&](int b, int x, int y, int z) {
      return b * ncol[0] * ncol[1] * ncol[2] + col[0][x] + ncol[0] * (col[1][y] + ncol[1] * col[2][z]);
    };
    for (int b = 0; b < T.n_sublat && ok; ++b)
      for (int z = 0; z < L[2] && ok; ++z)
        for (int y = 0; y < L[1] && ok; ++y)
          for (int x = 0; x < L[0] && ok; ++x) {
            const int c0 = cls(b, x, y, z);
            const int l0 = b * n_uc + x + L[0] * (y + L[1] * z);
            for (int c = T.fl_begin[b][0]; c < T.fl_begin[b][T.n_orbits] && ok; ++c)
              for (int q = 0; q < 3; ++q) {
                const int pb = s.fl_pb[c * 3 + q];
                if (pb < 0) continue;
                const int *du = &s.fl_du[c * 9 + q * 3];
                const int u1 = C.index(x + du[0], y + du[1], z + du[2]);
                const int px = u1 % L[0], py = (u1 / L[0]) % L[1], pz = u1 / (L[0] * L[1]);
                const int l1 = pb * n_uc + u1;
                if (l1 == l0)
                  throw Err(CEM_ERR_INVALID,
                            "supercell too small: a cluster contains one site twice");
                if (cls(pb, px, py, pz) == c0) ok = false;
              }
          }
    if (ok) return p;
  }
  throw Err(CEM_ERR_UNSUPPORTED, "no valid site colouring for this supercell");
}

// sub-steps of one pass (sweeps x colour classes): the size of the sweep
// kernel's per-pass schedule
int sub_steps(const cem_replicas *r) {
  const int sweeps = r->ensemble == CEM_CANONICAL ? r->n_pair_sweeps + r->n_local_sweeps : 1;
  return sweeps * r->max_classes;
}

// the cooperative sweep's 16-bit cluster records: every partner offset in
// every replica's halo'd layout and every integer weight fits in int16
bool fits_pack16(const cem_replicas *r) {
  const cem_system &s = *r->sys;
  const CeTables &T = s.T;
  if (!s.split_ok) return false;
  for (int a : s.wq_host)
    if (a < -32768 || a > 32767) return false;
  for (const Replica &R : r->reps) {
    const long long W = R.L[0] + 2 * T.reach, H = R.L[1] + 2 * T.reach;
    const long long V = W * H * (R.L[2] + 2 * T.reach);
    for (int b = 0; b < T.n_sublat; ++b)
      for (int c = T.fl_begin[b][0]; c < T.fl_begin[b][T.n_orbits]; ++c)
        for (int q = 0; q < 3; ++q) {
          const int pb = s.fl_pb[c * 3 + q];
          if (pb < 0) continue;
          const int *du = &s.fl_du[c * 9 + q * 3];
          const long long off = (pb - b) * V + du[0] + W * (du[1] + H * du[2]);
          if (off < -32768 || off > 32767) return false;
        }
  }
  return true;
}

// dynamic shared memory of the sweep kernel for a batch at a given pitch
// (the layout of the run-time tables depends on the evaluator)
int batch_smem(const cem_replicas *r, int pitch) {
  int smem = 0;
  for (const Replica &R : r->reps)
    smem = std::max(smem, sweep_smem_bytes(r->sys->T, R.L[0], R.L[1], R.L[2], sub_steps(r), pitch));
  return smem;
}

void check_rep(const cem_replicas *r, int i) {
  require(r != nullptr, "null replicas handle");
  require(i >= 0 && i < r->n, "replica index out of range");
}

void set_dmu(const cem_system &s, Replica &R) {
  const int no = s.T.n_occ;
  for (int a = 0; a < 16; ++a) R.dmu[a] = 0.0, R.dmu_hi[a] = 0.f, R.dmu_lo[a] = 0.f;
  if (R.ensemble != CEM_SEMIGRAND_CANONICAL) return;
  for (int oi = 0; oi < no; ++oi)
    for (int of = 0; of < no; ++of) {
      // mu . R^T dN with dN = e_of - e_oi (SemiGrandCanonicalCalculator.cc:201-212)
      double t = 0.0;
      for (int k = 0; k < no - 1; ++k) {
        double x = s.RT[k * no + of] - s.RT[k * no + oi];
        t += R.mu[k] * x;
      }
      R.dmu[oi * no + of] = t;
      float hi = (float)t;
      R.dmu_hi[oi * no + of] = hi;
      R.dmu_lo[oi * no + of] = (float)(t - (double)hi);
    }
}

// Lower-triangular Hermite normal form H = T U (U unimodular) of a supercell
// matrix T whose columns are the supercell lattice vectors in prim cell
// coordinates (row-major T[3 r + c]): H[r][r] > 0, 0 <= H[r][c] < H[r][r] for
// c < r, H[r][c] = 0 for c > r. Column operations only (Euclid's algorithm
// along each row, then reduction below the diagonal), so H generates the same
// superlattice.
std::array<long long, 9> hermite_lower(const int64_t *T) {
  long long h[3][3];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      require(T[3 * a + c] > -(1 << 20) && T[3 * a + c] < (1 << 20),
              "supercell matrix entry out of range", CEM_ERR_UNSUPPORTED);
      h[a][c] = T[3 * a + c];
    }
  auto col_sub = [&](int dst, int src, long long q) {
    for (int a = 0; a < 3; ++a) h[a][dst] -= q * h[a][src];
  };
  for (int a = 0; a < 3; ++a) {
    for (int c = a + 1; c < 3; ++c)
      while (h[a][c] != 0) {
        col_sub(a, c, h[a][a] / h[a][c]);
        for (int k = 0; k < 3; ++k) std::swap(h[k][a], h[k][c]);
      }
    require(h[a][a] != 0, "singular supercell matrix");
    if (h[a][a] < 0)
      for (int k = 0; k < 3; ++k) h[k][a] = -h[k][a];
  }
  auto fl = [](long long x, long long m) { return x >= 0 ? x / m : -((m - 1 - x) / m); };
  col_sub(0, 1, fl(h[1][0], h[1][1]));
  col_sub(0, 2, fl(h[2][0], h[2][2]));
  col_sub(1, 2, fl(h[2][1], h[2][2]));
  std::array<long long, 9> H;
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) H[3 * a + c] = h[a][c];
  return H;
}

// The learned proposals and the streamed batches keep each replica as an
// axis-aligned periodic box (cubic lattices of generated tables, halo tiles
// in HBM); non-diagonal supercells do not run there.
void require_box(const cem_replicas *r) {
  require(!r->twisted,
          "non-diagonal supercells support energies, energy changes, the sequential replay, "
          "the n-fold way, composition enforcement, state transfer and semi-grand parallel "
          "sweeps; these parallel runs need diagonal supercells",
          CEM_ERR_UNSUPPORTED);
}

// The plain sweep on a batch with non-diagonal supercells: semi-grand
// canonical flips only (the canonical pair geometry assumes an axis-aligned
// box), with a valid colouring of every twisted replica and the replicas in
// shared memory.
void require_sweepable(const cem_replicas *r) {
  require(!r->twisted || (r->ensemble == CEM_SEMIGRAND_CANONICAL && r->twisted_parallel),
          "non-diagonal supercells support energies, energy changes, the sequential replay, "
          "the n-fold way, composition enforcement, state transfer and semi-grand parallel "
          "sweeps (when an exact colouring exists); canonical parallel runs need diagonal "
          "supercells",
          CEM_ERR_UNSUPPORTED);
}

// L[3 i ..] diagonal of replica i's Hermite normal form, tw[3 i ..] its
// entries below the diagonal (null: diagonal supercells).
void create_replicas(const cem_system *sys, int n, const int *L, const int *tw, int ensemble,
                     cem_replicas **out) {
  {
    require(sys && L && out, "null argument");
    *out = nullptr;
    require(n >= 1, "need at least one replica");
    require(ensemble == CEM_CANONICAL || ensemble == CEM_SEMIGRAND_CANONICAL, "bad ensemble");
    require(ensemble != CEM_CANONICAL || sys->swaps_connect,
            "the local-swap displacements do not connect every site (their graph over the "
            "sublattices must be connected and its cycle translations generate the lattice): "
            "the canonical chain would not be ergodic");
    auto r = std::make_unique<cem_replicas>();
    r->sys = sys;
    r->n = n;
    r->ensemble = ensemble;
    CUDA_OK(cudaGetDevice(&r->device));
    r->reps.resize(n);
    std::map<std::vector<int>, int> pcache;
    int64_t off = 0;
    int max_cls = 1;
    for (int i = 0; i < n; ++i) {
      Replica &R = r->reps[i];
      std::memset(&R, 0, sizeof(R));
      const bool twist = tw && (tw[3 * i] || tw[3 * i + 1] || tw[3 * i + 2]);
      for (int a = 0; a < 3; ++a) {
        R.L[a] = L[3 * i + a];
        R.tw[a] = twist ? tw[3 * i + a] : 0;
        if (twist) continue;
        require(R.L[a] >= 1 && R.L[a] <= MAX_L, "supercell dimension out of range",
                CEM_ERR_UNSUPPORTED);
        require(R.L[a] >= 2 * sys->T.reach + 1,
                "supercell too small for the cluster expansion's reach");
      }
      if (twist) {
        const int64_t n_uc = (int64_t)R.L[0] * R.L[1] * R.L[2];
        require(R.L[0] >= 1 && R.L[1] >= 1 && R.L[2] >= 1 &&
                    n_uc * sys->T.n_sublat <= (int64_t)1 << 28,
                "supercell dimension out of range", CEM_ERR_UNSUPPORTED);
        require(R.tw[0] >= 0 && R.tw[0] < R.L[1] && R.tw[1] >= 0 && R.tw[1] < R.L[2] &&
                    R.tw[2] >= 0 && R.tw[2] < R.L[2],
                "supercell not in Hermite normal form");
        // no cluster may hold two periodic images of one site: every cluster
        // is some site's flower cluster, whose sites are the centre (b, 0) and
        // the partners (pb, du); two of them on one sublattice are images when
        // their cell offsets differ by a supercell lattice vector
        const Cells C = R.cells();
        for (int b = 0; b < sys->T.n_sublat; ++b)
          for (int c = sys->T.fl_begin[b][0]; c < sys->T.fl_begin[b][sys->T.n_orbits]; ++c) {
            int sb[4] = {b, -1, -1, -1}, su[4][3] = {{0, 0, 0}};
            for (int q = 0; q < 3; ++q) {
              sb[q + 1] = sys->fl_pb[c * 3 + q];
              for (int a = 0; a < 3; ++a) su[q + 1][a] = sys->fl_du[c * 9 + q * 3 + a];
            }
            for (int q1 = 0; q1 < 4; ++q1)
              for (int q2 = q1 + 1; q2 < 4; ++q2)
                require(sb[q1] < 0 || sb[q1] != sb[q2] ||
                            C.index(su[q1][0] - su[q2][0], su[q1][1] - su[q2][1],
                                    su[q1][2] - su[q2][2]) != 0,
                        "supercell too small: a cluster contains one site twice");
          }
        r->twisted = true;
      }
      R.n_sites = R.L[0] * R.L[1] * R.L[2] * sys->T.n_sublat;
      R.ensemble = ensemble;
      R.occ_offset = off;
      off += R.n_sites;
      int cls = sys->T.n_sublat;
      if (!twist) {
        std::vector<int> key{R.L[0], R.L[1], R.L[2]};
        auto it = pcache.find(key);
        int p = (it != pcache.end()) ? it->second
                                     : (pcache[key] = choose_colouring(*sys, R.L, ensemble));
        R.p = p;
        for (int a = 0; a < 3; ++a) {
          auto col = axis_blocks(R.L[a], p);
          R.n_col[a] = *std::max_element(col.begin(), col.end()) + 1;
          cls *= R.n_col[a];
        }
      } else {
        // twisted: the semi-grand parallel sweep runs when an exact colouring
        // exists (checked through the twisted periodicity)
        for (int a = 0; a < 3; ++a) R.n_col[a] = 1;
        bool coloured = false;
        if (ensemble == CEM_SEMIGRAND_CANONICAL && !sys->big) {
          std::vector<int> key{R.L[0], R.L[1], R.L[2], R.tw[0], R.tw[1], R.tw[2]};
          auto it = pcache.find(key);
          if (it != pcache.end()) {
            R.p = it->second;
          } else {
            try {
              R.p = choose_colouring(*sys, R.L, ensemble, R.tw);
            } catch (const Err &) {
              R.p = 0;  // no colouring: the batch does not sweep
            }
            pcache[key] = R.p;
          }
          coloured = R.p > 0;
        }
        if (coloured) {
          for (int a = 0; a < 3; ++a) {
            auto col = axis_blocks(R.L[a], R.p);
            R.n_col[a] = *std::max_element(col.begin(), col.end()) + 1;
            cls *= R.n_col[a];
          }
        } else {
          r->twisted_parallel = false;
        }
      }
      max_cls = std::max(max_cls, cls);
      R.temperature = 1000.0;
      R.beta = 1.0 / (KB * R.temperature);
      R.beta_f = (float)R.beta;
      R.seed = 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
      set_dmu(*sys, R);
    }
    r->total_sites = off;
    r->max_classes = max_cls;
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int need = 0;
    for (int i = 0; i < n; ++i)
      need = std::max({need, r->reps[i].L[0] + 2 * sys->T.reach, r->reps[i].L[1] + 2 * sys->T.reach});
    int pitch = 0;
    if (sys->fcc_generated) {
      // exact fit L + 2 reach when every replica has it, else the smallest that holds all
      bool same = true;
      for (int i = 0; i < n; ++i)
        same = same && r->reps[i].L[0] + 2 * sys->T.reach == need &&
               r->reps[i].L[1] + 2 * sys->T.reach == need;
      for (int cand : SWEEP_PITCHES) {
        if (cand < need) continue;
        if (same && cand != need && cand != 64) continue;
        pitch = cand;
        break;
      }
    }
    if (pitch && batch_smem(r.get(), pitch) > maxsm) pitch = 0;  // generated layout does not fit
    if (sys->big) pitch = sys->coop ? -2 : -1;  // one warp per site / one orbit at a time
    if (r->twisted) pitch = 0;
    r->pitch = pitch;
    r->sweep_smem = (r->twisted && !r->twisted_parallel) ? 0 : batch_smem(r.get(), pitch);
    if (r->twisted && r->sweep_smem > maxsm) r->twisted_parallel = false;
    if (!r->twisted && r->sweep_smem > maxsm && stream_pitch_for(*sys, r->reps)) {
      r->streamed = true;
      r->stream_pitch = stream_pitch_for(*sys, r->reps);
    }
    r->stats_host.assign(n, ReplicaStats{});
    CUDA_OK(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    CUDA_OK(cudaEventCreate(&r->ev0));
    CUDA_OK(cudaEventCreate(&r->ev1));
    CUDA_OK(cudaMalloc(&r->d_reps, sizeof(Replica) * n));
    CUDA_OK(cudaMalloc(&r->d_stats, sizeof(ReplicaStats) * n));
    CUDA_OK(cudaMemset(r->d_stats, 0, sizeof(ReplicaStats) * n));
    CUDA_OK(cudaMalloc(&r->d_occ, (size_t)off + 16));
    CUDA_OK(cudaMemset(r->d_occ, 0, (size_t)off + 16));
    CUDA_OK(cudaMalloc(&r->d_counts, sizeof(unsigned long long) * (MAX_FUNCS + 8)));
    CUDA_OK(cudaMalloc(&r->d_result, sizeof(long long) * 4));
    r->sample_width = sys->T.n_occ + 1;  // potential, (n_occ-1) compositions, order parameter
    {
      int *h = nullptr;
      CUDA_OK(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped));
      *h = 0;
      r->h_stop = h;
      CUDA_OK(cudaHostGetDevicePointer(reinterpret_cast<void **>(&r->d_stop), h, 0));
    }
    *out = r.release();
  }
}

}  // namespace

extern "C" {

const char *cem_last_error(void) { return g_error.c_str(); }

int cem_device_info(char *name, int name_len, int *sm_count, int *cc_major, int *cc_minor) {
  return guard([&] {
    int dev = 0;
    CUDA_OK(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CUDA_OK(cudaGetDeviceProperties(&p, dev));
    if (name && name_len > 0) {
      std::strncpy(name, p.name, name_len - 1);
      name[name_len - 1] = 0;
    }
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
  });
}

int cem_system_create(const cem_system_desc *d, cem_system **out) {
  return guard([&] {
    require(d && out, "null argument");
    *out = nullptr;
    require(d->n_sublat >= 1 && d->n_sublat <= MAX_SUBLAT, "n_sublat must be in 1..4",
            CEM_ERR_UNSUPPORTED);
    require(d->n_occ >= 2 && d->n_occ <= 3, "n_occ must be 2 or 3", CEM_ERR_UNSUPPORTED);
    require(d->n_funcs >= 1 && d->n_funcs <= MAX_FUNCS, "n_funcs out of range",
            CEM_ERR_UNSUPPORTED);
    require(d->n_orbits >= 1 && d->n_orbits <= MAX_ORBITS_ALL, "n_orbits out of range",
            CEM_ERR_UNSUPPORTED);
    auto s = std::make_unique<cem_system>();
    CeTables &T = s->T;
    T.n_sublat = d->n_sublat;
    T.n_occ = d->n_occ;
    T.n_sf = d->n_occ - 1;
    T.n_funcs = d->n_funcs;
    T.n_orbits = d->n_orbits;
    int fexp = 1;
    for (int g = 0; g < d->n_orbits; ++g) {
      T.orb_size[g] = d->orbit_size[g];
      T.orb_func_base[g] = d->orbit_func_begin[g];
      T.orb_n_funcs[g] = d->orbit_n_funcs[g];
      require(T.orb_size[g] >= 1 && T.orb_size[g] <= 4, "orbit size must be 1..4",
              CEM_ERR_UNSUPPORTED);
      require(T.orb_func_base[g] == fexp, "orbit functions must be contiguous, in order");
      require(T.orb_n_funcs[g] >= 1 && T.orb_n_funcs[g] <= 8,
              "at most 8 functions per orbit", CEM_ERR_UNSUPPORTED);
      require(d->n_occ > 2 || T.orb_n_funcs[g] == 1, "binary orbits have one function");
      fexp += T.orb_n_funcs[g];
    }
    require(fexp == d->n_funcs, "functions do not match orbits");
    const int stride = T.n_sf * T.n_sf * T.n_sf * T.n_sf;
    const int ncl = d->n_flower + d->n_owned;
    std::vector<int> pb(ncl * 3), du(ncl * 9), lutoff(ncl);
    std::vector<uint8_t> lut((size_t)ncl * stride, 0);
    auto load = [&](int base, int n, const int *sub, const int *orb, const int *psub,
                    const int *pdu, const int16_t *plut, int begin[MAX_SUBLAT][MAX_ORBITS_ALL + 1]) {
      int prev_b = 0, prev_g = 0;
      for (int b = 0; b < MAX_SUBLAT; ++b)
        for (int g = 0; g <= MAX_ORBITS_ALL; ++g) begin[b][g] = -1;
      for (int c = 0; c < n; ++c) {
        const int b = sub[c], g = orb[c];
        require(b >= 0 && b < d->n_sublat && g >= 0 && g < d->n_orbits, "bad cluster entry");
        require(b > prev_b || (b == prev_b && g >= prev_g) || c == 0,
                "clusters must be grouped by sublattice then orbit");
        prev_b = b;
        prev_g = g;
        for (int q = 0; q < 3; ++q) {
          const int p = psub[c * 3 + q];
          require(p >= -1 && p < d->n_sublat, "bad partner sublattice");
          require((q < T.orb_size[g] - 1) == (p >= 0), "partner count must match orbit size");
          pb[(base + c) * 3 + q] = p;
          for (int a = 0; a < 3; ++a) du[(base + c) * 9 + q * 3 + a] = pdu[c * 9 + q * 3 + a];
        }
        lutoff[base + c] = (base + c) * stride;
        int ncode = 1;
        for (int q = 0; q < T.orb_size[g]; ++q) ncode *= T.n_sf;
        for (int code = 0; code < ncode; ++code) {
          const int f = plut[(size_t)c * stride + code];
          require(f >= T.orb_func_base[g] && f < T.orb_func_base[g] + T.orb_n_funcs[g],
                  "decoration table refers to a function outside the cluster's orbit");
          lut[(size_t)(base + c) * stride + code] = (uint8_t)(f - T.orb_func_base[g]);
        }
      }
      // CSR bounds per (b, g)
      int c = 0;
      for (int b = 0; b < d->n_sublat; ++b)
        for (int g = 0; g < d->n_orbits; ++g) {
          begin[b][g] = c;
          while (c < n && sub[c] == b && orb[c] == g) ++c;
          begin[b][g + 1] = c;
        }
      require(c == n, "clusters are not grouped by sublattice then orbit");
      for (int b = d->n_sublat; b < MAX_SUBLAT; ++b)
        for (int g = 0; g <= MAX_ORBITS_ALL; ++g) begin[b][g] = n;
    };
    load(0, d->n_flower, d->flower_sublat, d->flower_orbit, d->flower_partner_sublat,
         d->flower_partner_du, d->flower_lut, T.fl_begin);
    // the owned begin indices are relative to the owned block
    load(d->n_flower, d->n_owned, d->owned_sublat, d->owned_orbit, d->owned_partner_sublat,
         d->owned_partner_du, d->owned_lut, T.ow_begin);
    T.n_fl = d->n_flower;
    T.n_ow = d->n_owned;
    int reach = 0;
    for (int c = 0; c < d->n_flower; ++c)
      for (int q = 0; q < 9; ++q) reach = std::max(reach, std::abs(du[c * 9 + q]));
    T.reach = reach;
    s->fl_pb.assign(pb.begin(), pb.begin() + d->n_flower * 3);
    s->fl_du.assign(du.begin(), du.begin() + d->n_flower * 9);
    s->fcc_generated = matches_generated_fcc(T, s->fl_pb.data(), s->fl_du.data());
    int nbr = 0;
    for (int b = 0; b < d->n_sublat; ++b) {
      T.n_nb[b] = d->n_neighbour ? d->n_neighbour[b] : 0;
      require(T.n_nb[b] >= 0 && T.n_nb[b] <= MAX_NB, "too many neighbour displacements");
      for (int k = 0; k < T.n_nb[b]; ++k) {
        T.nb_b[b][k] = d->neighbour_sublat[b * 16 + k];
        for (int a = 0; a < 3; ++a) {
          T.nb_du[b][k][a] = d->neighbour_du[(b * 16 + k) * 3 + a];
          nbr = std::max(nbr, std::abs(T.nb_du[b][k][a]));
        }
      }
    }
    s->nb_reach = nbr;
    s->swaps_connect = swaps_connect(T);
    s->w.assign(d->weights, d->weights + d->n_funcs);
    std::vector<float> whi(d->n_funcs), wlo(d->n_funcs);
    for (int f = 0; f < d->n_funcs; ++f) {
      require(std::isfinite(s->w[f]), "non-finite weight");
      whi[f] = (float)s->w[f];
      wlo[f] = (float)(s->w[f] - (double)whi[f]);
    }
    s->RT.assign(d->param_RT, d->param_RT + (d->n_occ - 1) * d->n_occ);
    // binary sweep weights: integer multiples of a power-of-two quantum plus
    // an f32 remainder, so the sweep's energy change is an exact int32 sum
    // plus one f32 FMA chain
    for (int g = 0; g < MAX_ORBITS; ++g) {
      T.wq[g] = 0;
      T.wr[g] = 0.f;
    }
    T.wq_scale = 1.f;
    s->big = T.n_orbits > MAX_ORBITS;
    std::vector<int> wq_all(T.n_orbits, 0);
    std::vector<float> wr_all(T.n_orbits, 0.f);
    if (d->n_occ == 2) {
      double wmax = 0.0;
      std::vector<long long> dcmax(T.n_orbits, 0);
      for (int g = 0; g < T.n_orbits; ++g) {
        wmax = std::max(wmax, std::fabs(s->w[T.orb_func_base[g]]));
        for (int b = 0; b < T.n_sublat; ++b)
          dcmax[g] = std::max<long long>(dcmax[g], 2 * (T.fl_begin[b][g + 1] - T.fl_begin[b][g]));
      }
      bool ok = wmax == 0.0;
      if (wmax > 0.0) {
        for (int bits = 13; bits >= 0; --bits) {
          const double q = std::ldexp(1.0, std::ilogb(wmax) - bits);
          long long bound = 0;
          std::vector<long long> A(T.n_orbits, 0);
          for (int g = 0; g < T.n_orbits; ++g) {
            A[g] = std::llround(s->w[T.orb_func_base[g]] / q);
            bound += std::llabs(A[g]) * dcmax[g];
          }
          if (bound < (1ll << 24)) {
            ok = true;
            T.wq_scale = (float)q;
            for (int g = 0; g < T.n_orbits; ++g) {
              wq_all[g] = (int)A[g];
              wr_all[g] = (float)(s->w[T.orb_func_base[g]] - (double)A[g] * q);
            }
            break;
          }
        }
      }
      // small systems: the register sweep needs the split; large ones fall
      // back to the orbit walk without it
      require(ok || s->big, "cluster expansion too large for the binary sweep weights",
              CEM_ERR_UNSUPPORTED);
      bool sorted = true;
      for (int g = 1; g < T.n_orbits; ++g) sorted = sorted && T.orb_size[g] >= T.orb_size[g - 1];
      s->split_ok = ok && sorted;
      s->wq_host = wq_all;
      s->coop = s->big && s->split_ok;
      if (!s->big)
        for (int g = 0; g < T.n_orbits; ++g) {
          T.wq[g] = wq_all[g];
          T.wr[g] = wr_all[g];
        }
    }
    int *dpb = dev_copy(pb), *ddu = dev_copy(du), *dlo = dev_copy(lutoff);
    uint8_t *dlut = dev_copy(lut);
    float *dwhi = dev_copy(whi), *dwlo = dev_copy(wlo);
    double *dw = dev_copy(s->w);
    // distinct flower partners per sublattice (the sites whose events see a
    // change of the centre site)
    std::vector<int> fp((size_t)d->n_sublat * MAX_FP * 4, 0);
    for (int b = 0; b < d->n_sublat; ++b) {
      int n = 0;
      for (int c = T.fl_begin[b][0]; c < T.fl_begin[b][T.n_orbits]; ++c)
        for (int q = 0; q < 3; ++q) {
          const int p = s->fl_pb[c * 3 + q];
          if (p < 0) continue;
          const int *u = &s->fl_du[c * 9 + q * 3];
          bool seen = false;
          for (int k = 0; k < n && !seen; ++k) {
            const int *e = &fp[((size_t)b * MAX_FP + k) * 4];
            seen = e[0] == p && e[1] == u[0] && e[2] == u[1] && e[3] == u[2];
          }
          if (seen) continue;
          require(n < MAX_FP, "too many distinct flower partners", CEM_ERR_UNSUPPORTED);
          int *e = &fp[((size_t)b * MAX_FP + n) * 4];
          e[0] = p;
          e[1] = u[0];
          e[2] = u[1];
          e[3] = u[2];
          ++n;
        }
      T.n_fp[b] = n;
    }
    int *dfp = dev_copy(fp);
    T.fp = dfp;
    int *dwq = dev_copy(wq_all);
    float *dwr = dev_copy(wr_all);
    T.wq_all = dwq;
    T.wr_all = dwr;
    s->owned = {dpb, ddu, dlo, dlut, dwhi, dwlo, dw, dfp, dwq, dwr};
    T.cl_pb = dpb;
    T.cl_du = ddu;
    T.cl_lut = dlo;
    T.lut = dlut;
    T.w_hi = dwhi;
    T.w_lo = dwlo;
    T.w = dw;
    s->n_flower = d->n_flower;
    s->n_owned = d->n_owned;
    *out = s.release();
  });
}

int cem_system_destroy(cem_system *sys) {
  return guard([&] { delete sys; });
}

int cem_replicas_create(const cem_system *sys, int n, const int *L, int ensemble,
                        cem_replicas **out) {
  return guard([&] { create_replicas(sys, n, L, nullptr, ensemble, out); });
}

int cem_supercell_hnf(const int64_t *T, int64_t *H) {
  return guard([&] {
    require(T && H, "null argument");
    const auto h = hermite_lower(T);
    for (int a = 0; a < 9; ++a) H[a] = h[a];
  });
}

int cem_replicas_create_supercells(const cem_system *sys, int n, const int64_t *T, int ensemble,
                                   cem_replicas **out) {
  return guard([&] {
    require(T != nullptr && n >= 1, "null argument");
    std::vector<int> L(3 * (size_t)n), tw(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      const auto H = hermite_lower(T + 9 * (size_t)i);
      for (int a = 0; a < 3; ++a)
        require(H[4 * a] < (1 << 20), "supercell dimension out of range", CEM_ERR_UNSUPPORTED);
      L[3 * i] = (int)H[0];
      L[3 * i + 1] = (int)H[4];
      L[3 * i + 2] = (int)H[8];
      tw[3 * i] = (int)H[3];
      tw[3 * i + 1] = (int)H[6];
      tw[3 * i + 2] = (int)H[7];
    }
    create_replicas(sys, n, L.data(), tw.data(), ensemble, out);
  });
}

int cem_replicas_destroy(cem_replicas *r) {
  return guard([&] { delete r; });
}

int cem_n_sites(const cem_replicas *r, int i, int64_t *n) {
  return guard([&] {
    check_rep(r, i);
    *n = r->reps[i].n_sites;
  });
}

int cem_set_conditions(cem_replicas *r, int i, double temperature, const double *mu) {
  return guard([&] {
    check_rep(r, i);
    require(std::isfinite(temperature) && temperature >= 0.0, "temperature must be >= 0");
    Replica &R = r->reps[i];
    R.temperature = temperature;
    // Conditions.hh:17-45: beta = inf when T is zero within 1e-10
    R.beta = (std::fabs(temperature) < 1e-10) ? INFINITY : 1.0 / (KB * temperature);
    R.beta_f = (float)R.beta;
    const int nc = r->sys->T.n_occ - 1;
    for (int k = 0; k < 3; ++k) R.mu[k] = 0.0;
    if (mu) {
      for (int k = 0; k < nc; ++k) {
        require(std::isfinite(mu[k]), "param_chem_pot must be finite");
        R.mu[k] = mu[k];
      }
    } else {
      require(r->ensemble == CEM_CANONICAL, "semi-grand canonical replicas need param_chem_pot");
    }
    set_dmu(*r->sys, R);
    r->reps_dirty = true;
  });
}

int cem_set_seed(cem_replicas *r, int i, uint64_t seed) {
  return guard([&] {
    check_rep(r, i);
    r->reps[i].seed = seed;
    r->reps_dirty = true;
  });
}

int cem_set_occupation(cem_replicas *r, int i, const int8_t *occ) {
  return guard([&] {
    check_rep(r, i);
    require(occ != nullptr, "null occupation");
    const Replica &R = r->reps[i];
    for (int l = 0; l < R.n_sites; ++l)
      require(occ[l] >= 0 && occ[l] < r->sys->T.n_occ, "occupant index out of range");
    CUDA_OK(cudaMemcpyAsync(r->d_occ + R.occ_offset, occ, R.n_sites, cudaMemcpyHostToDevice,
                            r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    r->stats_valid = false;
  });
}

int cem_get_occupation(cem_replicas *r, int i, int8_t *occ) {
  return guard([&] {
    check_rep(r, i);
    require(occ != nullptr, "null occupation");
    const Replica &R = r->reps[i];
    CUDA_OK(cudaMemcpyAsync(occ, r->d_occ + R.occ_offset, R.n_sites, cudaMemcpyDeviceToHost,
                            r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
  });
}

int cem_set_occupation_all(cem_replicas *r, const int8_t *packed) {
  return guard([&] {
    require(r && packed, "null argument");
    CUDA_OK(cudaMemcpyAsync(r->d_occ, packed, (size_t)r->total_sites, cudaMemcpyHostToDevice,
                            r->stream));
    r->stats_valid = false;
  });
}

int cem_get_occupation_all(cem_replicas *r, int8_t *packed) {
  return guard([&] {
    require(r && packed, "null argument");
    CUDA_OK(cudaMemcpyAsync(packed, r->d_occ, (size_t)r->total_sites, cudaMemcpyDeviceToHost,
                            r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
  });
}

int cem_host_alloc(int64_t bytes, void **ptr) {
  return guard([&] {
    require(ptr && bytes > 0, "bad argument");
    CUDA_OK(cudaMallocHost(ptr, (size_t)bytes));
  });
}

int cem_host_free(void *ptr) {
  return guard([&] { CUDA_OK(cudaFreeHost(ptr)); });
}

int cem_energy(cem_replicas *r, int i, double *energy, int64_t *counts) {
  return guard([&] {
    check_rep(r, i);
    const Replica &R = r->reps[i];
    const CeTables &T = r->sys->T;
    CUDA_OK(launch_energy(T, r->d_occ + R.occ_offset, R.cells(), r->d_counts, r->stream));
    std::vector<unsigned long long> c(T.n_funcs);
    CUDA_OK(cudaMemcpyAsync(c.data(), r->d_counts, sizeof(unsigned long long) * T.n_funcs,
                            cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    const int n_uc = R.L[0] * R.L[1] * R.L[2];
    double e = r->sys->w[0] * n_uc;
    for (int f = 1; f < T.n_funcs; ++f) e += r->sys->w[f] * (double)c[f];
    if (energy) *energy = e;
    if (counts) {
      counts[0] = n_uc;
      for (int f = 1; f < T.n_funcs; ++f) counts[f] = (int64_t)c[f];
    }
  });
}

int cem_delta_energy(cem_replicas *r, int i, int n_events, int k, const int64_t *sites,
                     const int32_t *new_occ, int potential, double *dE, int64_t *dcount) {
  return guard([&] {
    check_rep(r, i);
    require(n_events >= 0 && k >= 1 && k <= 4, "sites_per_event must be 1..4");
    require(sites && new_occ && dE, "null argument");
    if (n_events == 0) return;
    const Replica &R = r->reps[i];
    const CeTables &T = r->sys->T;
    for (int64_t e = 0; e < (int64_t)n_events * k; ++e) {
      require(sites[e] >= 0 && sites[e] < R.n_sites, "site index out of range");
      require(new_occ[e] >= 0 && new_occ[e] < T.n_occ, "occupant index out of range");
    }
    require(potential == 0 || r->ensemble == CEM_SEMIGRAND_CANONICAL,
            "the semi-grand potential needs semi-grand canonical replicas");
    long long *ds = nullptr;
    int *dn = nullptr;
    double *dde = nullptr, *ddmu = nullptr;
    long long *ddc = nullptr;
    auto cleanup = [&] {
      cudaFree(ds);
      cudaFree(dn);
      cudaFree(dde);
      cudaFree(ddmu);
      cudaFree(ddc);
    };
    try {
      const size_t ne = (size_t)n_events * k;
      CUDA_OK(cudaMalloc(&ds, ne * 8));
      CUDA_OK(cudaMalloc(&dn, ne * 4));
      CUDA_OK(cudaMalloc(&dde, (size_t)n_events * 8));
      CUDA_OK(cudaMemcpyAsync(ds, sites, ne * 8, cudaMemcpyHostToDevice, r->stream));
      CUDA_OK(cudaMemcpyAsync(dn, new_occ, ne * 4, cudaMemcpyHostToDevice, r->stream));
      if (potential) {
        CUDA_OK(cudaMalloc(&ddmu, 16 * 8));
        CUDA_OK(cudaMemcpyAsync(ddmu, R.dmu, 16 * 8, cudaMemcpyHostToDevice, r->stream));
      }
      if (dcount) CUDA_OK(cudaMalloc(&ddc, (size_t)n_events * T.n_funcs * 8));
      CUDA_OK(launch_delta(T, r->d_occ + R.occ_offset, R.cells(), n_events, k, ds, dn, ddmu, dde,
                           ddc, r->stream));
      CUDA_OK(cudaMemcpyAsync(dE, dde, (size_t)n_events * 8, cudaMemcpyDeviceToHost, r->stream));
      if (dcount)
        CUDA_OK(cudaMemcpyAsync(dcount, ddc, (size_t)n_events * T.n_funcs * 8,
                                cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int cem_replay(cem_replicas *r, int i, uint64_t mt_seed, int64_t n_steps, uint8_t *accept_seq,
               double *dE_seq, int64_t *site_seq, int64_t *n_accept, uint64_t *n_draws) {
  return guard([&] {
    check_rep(r, i);
    require(n_steps >= 0, "n_steps must be >= 0");
    const Replica &R = r->reps[i];
    const CeTables &T = r->sys->T;
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    require(replay_smem_bytes(R.n_sites, T.n_occ) <= maxsm,
            "supercell too large for the sequential replay kernel", CEM_ERR_UNSUPPORTED);
    ReplayParams P{};
    for (int a = 0; a < 3; ++a) {
      P.L[a] = R.L[a];
      P.tw[a] = R.tw[a];
    }
    P.n_sites = R.n_sites;
    P.ensemble = R.ensemble;
    P.beta = R.beta;
    for (int a = 0; a < 16; ++a) P.dmu[a] = R.dmu[a];
    P.mt_seed = mt_seed;
    P.n_steps = n_steps;
    P.occ = r->d_occ + R.occ_offset;
    P.result = r->d_result;
    unsigned char *dacc = nullptr;
    double *dde = nullptr;
    long long *dsite = nullptr;
    auto cleanup = [&] {
      cudaFree(dacc);
      cudaFree(dde);
      cudaFree(dsite);
    };
    try {
      if (accept_seq && n_steps) CUDA_OK(cudaMalloc(&dacc, (size_t)n_steps));
      if (dE_seq && n_steps) CUDA_OK(cudaMalloc(&dde, (size_t)n_steps * 8));
      if (site_seq && n_steps) CUDA_OK(cudaMalloc(&dsite, (size_t)n_steps * 16));
      P.accept_seq = dacc;
      P.de_seq = dde;
      P.site_seq = dsite;
      CUDA_OK(launch_replay(T, P, r->stream));
      long long res[3];
      CUDA_OK(cudaMemcpyAsync(res, r->d_result, 24, cudaMemcpyDeviceToHost, r->stream));
      if (dacc) CUDA_OK(cudaMemcpyAsync(accept_seq, dacc, (size_t)n_steps, cudaMemcpyDeviceToHost, r->stream));
      if (dde) CUDA_OK(cudaMemcpyAsync(dE_seq, dde, (size_t)n_steps * 8, cudaMemcpyDeviceToHost, r->stream));
      if (dsite) CUDA_OK(cudaMemcpyAsync(site_seq, dsite, (size_t)n_steps * 16, cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
      if (n_accept) *n_accept = res[0];
      if (n_draws) *n_draws = (uint64_t)res[1];
      if (res[2]) throw Err(CEM_ERR_DEVICE, "no event can be proposed from this occupation");
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    r->stats_valid = false;
  });
}

// Exact energies and species counts of every replica -> running stats
// (one batched kernel, no host round trip).
static void init_stats(cem_replicas *r) {
  r->upload_reps();
  int max_sites = 0;
  for (const Replica &R : r->reps) max_sites = std::max(max_sites, R.n_sites);
  CUDA_OK(launch_init_stats(r->sys->T, r->d_reps, r->d_stats, r->d_occ, r->n, max_sites,
                            r->stream));
  r->stats_valid = true;
}

int cem_reset_stats(cem_replicas *r) {
  return guard([&] {
    require(r != nullptr, "null handle");
    init_stats(r);
  });
}

// Replica -> CTA schedule of the shared-memory sweep. Mode 1 launches the
// largest replicas first (stable in replica order), so that a batch of uneven
// supercells does not end on a few large replicas; the results do not depend
// on the schedule.
static void set_cta_order(cem_replicas *r, int mode) {
  require(mode == 0 || mode == 1, "cta_order must be 0 (replica order) or 1 (largest first)");
  cudaFree(r->d_cta_rep);
  r->d_cta_rep = nullptr;
  r->cta_order = mode;
  if (mode == 0) return;
  std::vector<int> order(r->n);
  for (int i = 0; i < r->n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return r->reps[a].n_sites > r->reps[b].n_sites; });
  CUDA_OK(cudaMalloc(&r->d_cta_rep, sizeof(int) * r->n));
  CUDA_OK(cudaMemcpy(r->d_cta_rep, order.data(), sizeof(int) * r->n, cudaMemcpyHostToDevice));
}

// Zero the sampled moments of every replica (keeps energy, species counts and
// the pass / event counters).
static void reset_moments(cem_replicas *r) {
  std::vector<ReplicaStats> st(r->n);
  CUDA_OK(cudaMemcpyAsync(st.data(), r->d_stats, sizeof(ReplicaStats) * r->n,
                          cudaMemcpyDeviceToHost, r->stream));
  CUDA_OK(cudaStreamSynchronize(r->stream));
  for (auto &x : st) {
    x.n_samples = 0;
    x.sum_e = x.sum_e2 = x.sum_f = 0;
    for (int k = 0; k < 3; ++k) x.sum_x[k] = x.sum_ex[k] = 0;
    for (int k = 0; k < 9; ++k) x.sum_xx[k] = 0;
    x.status = 0;
  }
  CUDA_OK(cudaMemcpyAsync(r->d_stats, st.data(), sizeof(ReplicaStats) * r->n,
                          cudaMemcpyHostToDevice, r->stream));
}

int cem_nfold_run(cem_replicas *r, int64_t n_events, int64_t n_equil, int64_t record_capacity,
                  int64_t *rec_site, int32_t *rec_occ, double *rec_dt) {
  return guard([&] {
    require(r != nullptr, "null handle");
    require(r->ensemble == CEM_SEMIGRAND_CANONICAL,
            "the n-fold way runs semi-grand canonical replicas");
    require(n_events >= 0 && n_equil >= 0 && record_capacity >= 0, "counts must be >= 0");
    require(record_capacity == 0 || (rec_site && rec_occ && rec_dt), "null record buffers");
    const CeTables &T = r->sys->T;
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // generated evaluator when every replica has the 24^3 or 10^3 pitch
    int pitch = 0;
    if (r->sys->fcc_generated) {
      const int p0 = r->reps[0].L[0] + 4;
      bool same = p0 == 28 || p0 == 14;
      for (const Replica &R : r->reps)
        same = same && R.L[0] + 4 == p0 && R.L[1] + 4 == p0;
      if (same) pitch = p0;
    }
    // rate trees in shared memory when every replica's fits beside its
    // occupation, else in global memory
    int smem = 0, smem_tree = 0;
    for (const Replica &R : r->reps) {
      smem = std::max(smem, nfold_smem_bytes(T, R.L[0], R.L[1], R.L[2], pitch, 0));
      smem_tree = std::max(smem_tree, nfold_smem_bytes(T, R.L[0], R.L[1], R.L[2], pitch, 1));
    }
    require(smem <= maxsm, "supercell does not fit in shared memory for the n-fold kernel",
            CEM_ERR_UNSUPPORTED);
    const int tree_smem = smem_tree <= maxsm ? 1 : 0;
    if (tree_smem) smem = smem_tree;
    if (!r->d_nftree) {
      std::vector<long long> off(r->n);
      long long total = 0;
      for (int i = 0; i < r->n; ++i) {
        off[i] = total;
        total += rate_tree_size((long long)r->reps[i].n_sites * (T.n_occ - 1));
      }
      CUDA_OK(cudaMalloc(&r->d_nftree, sizeof(double) * (size_t)total));
      CUDA_OK(cudaMalloc(&r->d_nftree_off, sizeof(long long) * r->n));
      CUDA_OK(cudaMemcpy(r->d_nftree_off, off.data(), sizeof(long long) * r->n,
                         cudaMemcpyHostToDevice));
    }
    r->upload_reps();
    if (!r->stats_valid) init_stats(r);
    reset_moments(r);
    NfoldParams P{};
    P.reps = r->d_reps;
    P.stats = r->d_stats;
    P.occ = r->d_occ;
    P.tree = r->d_nftree;
    P.tree_off = r->d_nftree_off;
    P.tree_smem = tree_smem;
    P.n_events = n_events;
    P.n_equil = n_equil;
    P.rec_cap = record_capacity;
    for (size_t k = 0; k < r->sys->RT.size() && k < 16; ++k) P.RT[k] = r->sys->RT[k];
    long long *dsite = nullptr;
    int *docc = nullptr;
    double *ddt = nullptr;
    auto cleanup = [&] {
      cudaFree(dsite);
      cudaFree(docc);
      cudaFree(ddt);
    };
    try {
      const size_t nrec = (size_t)record_capacity * r->n;
      if (nrec) {
        CUDA_OK(cudaMalloc(&dsite, sizeof(long long) * nrec));
        CUDA_OK(cudaMalloc(&docc, sizeof(int) * nrec));
        CUDA_OK(cudaMalloc(&ddt, sizeof(double) * nrec));
        CUDA_OK(cudaMemsetAsync(dsite, 0xFF, sizeof(long long) * nrec, r->stream));
      }
      P.rec_site = dsite;
      P.rec_occ = docc;
      P.rec_dt = ddt;
      CUDA_OK(cudaEventRecord(r->ev0, r->stream));
      CUDA_OK(launch_nfold(T, P, r->n, smem, pitch, r->stream));
      CUDA_OK(cudaEventRecord(r->ev1, r->stream));
      if (nrec) {
        CUDA_OK(cudaMemcpyAsync(rec_site, dsite, sizeof(long long) * nrec, cudaMemcpyDeviceToHost,
                                r->stream));
        CUDA_OK(cudaMemcpyAsync(rec_occ, docc, sizeof(int) * nrec, cudaMemcpyDeviceToHost,
                                r->stream));
        CUDA_OK(cudaMemcpyAsync(rec_dt, ddt, sizeof(double) * nrec, cudaMemcpyDeviceToHost,
                                r->stream));
      }
      std::vector<ReplicaStats> st(r->n);
      CUDA_OK(cudaMemcpyAsync(st.data(), r->d_stats, sizeof(ReplicaStats) * r->n,
                              cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
      for (const auto &x : st)
        if (x.status) throw Err(CEM_ERR_DEVICE, "no event has a non-zero rate (zero temperature in a local minimum)");
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int cem_enforce_composition(cem_replicas *r, const double *target_mol, uint64_t mt_seed,
                            int64_t *n_flips) {
  return guard([&] {
    require(r != nullptr, "null replica batch");
    require(target_mol != nullptr, "null target composition");
    const int nocc = r->sys->T.n_occ;
    for (int i = 0; i < r->n * nocc; ++i)
      require(std::isfinite(target_mol[i]), "target composition must be finite");
    int *scratch = nullptr;
    double *d_target = nullptr;
    long long *d_out = nullptr;
    auto cleanup = [&] {
      cudaFree(scratch);
      cudaFree(d_target);
      cudaFree(d_out);
    };
    std::vector<long long> res(3 * (size_t)r->n);
    try {
      CUDA_OK(cudaMalloc(&scratch, (size_t)r->total_sites * (nocc + 1) * sizeof(int)));
      CUDA_OK(cudaMalloc(&d_target, sizeof(double) * r->n * nocc));
      CUDA_OK(cudaMalloc(&d_out, sizeof(long long) * 3 * r->n));
      r->upload_reps();
      CUDA_OK(cudaMemcpyAsync(d_target, target_mol, sizeof(double) * r->n * nocc,
                              cudaMemcpyHostToDevice, r->stream));
      long long max_sites = 0;
      for (const Replica &R : r->reps) max_sites = std::max<long long>(max_sites, R.n_sites);
      CUDA_OK(launch_enforce(nocc, r->d_reps, r->n, r->d_occ, d_target, mt_seed,
                             r->sys->T.n_sublat, scratch, d_out, 4 * max_sites + 16, r->stream));
      CUDA_OK(cudaMemcpyAsync(res.data(), d_out, sizeof(long long) * 3 * r->n,
                              cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    r->stats_valid = false;
    for (int i = 0; i < r->n; ++i) {
      if (res[3 * i + 2] == 3) throw Err(CEM_ERR_INVALID, "occupation holds an occupant index outside [0, n_occ)");
      if (res[3 * i + 2] != 0) throw Err(CEM_ERR_DEVICE, "composition enforcement did not terminate");
      if (n_flips) n_flips[i] = res[3 * i];
    }
  });
}

int cem_step_async(cem_replicas *r, const int8_t *host_in, int8_t *host_out, int64_t n_passes) {
  return guard([&] {
    require(r && host_in && host_out, "null argument");
    require_sweepable(r);
    require(n_passes >= 1, "n_passes must be >= 1");
    require(!r->streamed, "HBM-streamed batches run through cem_run", CEM_ERR_UNSUPPORTED);
    for (const void *p : {(const void *)host_in, (const void *)host_out}) {
      cudaPointerAttributes a{};
      CUDA_OK(cudaPointerGetAttributes(&a, p));
      require(a.type == cudaMemoryTypeHost,
              "cem_step_async needs page-locked host buffers (cem_host_alloc)");
    }
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    require(r->sweep_smem <= maxsm, "supercell does not fit in shared memory", CEM_ERR_UNSUPPORTED);
    r->upload_reps();
    const bool same = r->step_exec && r->step_in == host_in && r->step_out == host_out &&
                      r->step_passes == n_passes && r->step_threads == r->threads &&
                      r->step_order == r->cta_order && r->step_pitch == r->pitch &&
                      r->step_pair == r->n_pair_sweeps && r->step_local == r->n_local_sweeps &&
                      r->step_cluster == r->sweep_cluster;
    if (!same) {
      if (r->step_exec) cudaGraphExecDestroy(r->step_exec);
      r->step_exec = nullptr;
      const CeTables &T = r->sys->T;
      SweepParams P{};
      P.reps = r->d_reps;
      P.stats = r->d_stats;
      P.occ = r->d_occ;
      P.n_passes = n_passes;
      P.n_equil = 0;
      P.max_classes = r->max_classes;
      P.max_sub = sub_steps(r);
      P.pack16 = (r->pitch == -2 && !r->wide_records && fits_pack16(r)) ? 1 : 0;
      P.n_pair_sweeps = r->n_pair_sweeps;
      P.n_local_sweeps = r->n_local_sweeps;
      P.cta_rep = r->d_cta_rep;
      P.cluster = sweep_cluster_for(r->sweep_cluster, r->pitch, r->threads, r->reps);
      r->last_sweep_cluster = P.cluster;
      P.init = (T.n_occ == 2 && r->pitch >= 0) ? 1 : 0;
      for (size_t k = 0; k < r->sys->RT.size() && k < 16; ++k) P.RT[k] = r->sys->RT[k];
      int max_sites = 0;
      for (const Replica &R : r->reps) max_sites = std::max(max_sites, R.n_sites);
      cudaGraph_t graph;
      CUDA_OK(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaMemcpyAsync(r->d_occ, host_in, (size_t)r->total_sites,
                                      cudaMemcpyHostToDevice, r->stream);
      if (e == cudaSuccess && !P.init)
        e = launch_init_stats(T, r->d_reps, r->d_stats, r->d_occ, r->n, max_sites, r->stream);
      if (e == cudaSuccess)
        e = launch_sweep(T, P, r->n, r->sweep_smem, r->pitch, r->threads, r->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_out, r->d_occ, (size_t)r->total_sites, cudaMemcpyDeviceToHost,
                            r->stream);
      const cudaError_t e2 = cudaStreamEndCapture(r->stream, &graph);
      CUDA_OK(e);
      CUDA_OK(e2);
      e = cudaGraphInstantiate(&r->step_exec, graph, 0);
      cudaGraphDestroy(graph);
      CUDA_OK(e);
      r->step_in = host_in;
      r->step_out = host_out;
      r->step_passes = n_passes;
      r->step_threads = r->threads;
      r->step_order = r->cta_order;
      r->step_pitch = r->pitch;
      r->step_pair = r->n_pair_sweeps;
      r->step_local = r->n_local_sweeps;
      r->step_cluster = r->sweep_cluster;
    }
    CUDA_OK(cudaEventRecord(r->ev0, r->stream));
    CUDA_OK(cudaGraphLaunch(r->step_exec, r->stream));
    CUDA_OK(cudaEventRecord(r->ev1, r->stream));
    r->stats_valid = true;
  });
}

int cem_run(cem_replicas *r, int64_t n_passes, int64_t n_equil, int record_samples) {
  return guard([&] {
    require(r != nullptr, "null handle");
    require_sweepable(r);
    require(n_passes >= 0 && n_equil >= 0, "pass counts must be >= 0");
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    require(r->streamed || r->sweep_smem <= maxsm,
            "supercell does not fit in shared memory (" + std::to_string(r->sweep_smem) +
                " bytes needed) and has no HBM-streamed kernel",
            CEM_ERR_UNSUPPORTED);
    r->upload_reps();
    *r->h_stop = 0;  // a stop request applies to the run in flight
    NvtxRange nvtx("cem_run");
    if (r->streamed) {
      const int L = r->reps[0].L[0];
      const long long hb = stream_halo_bytes(L, r->stream_pitch);
      if (!r->sstate.halo) {
        CUDA_OK(cudaMalloc(&r->sstate.halo, (size_t)hb * r->n));
        CUDA_OK(cudaMalloc(&r->sstate.acc, sizeof(long long) * 16 * r->n));
        CUDA_OK(cudaMalloc(&r->sstate.run, sizeof(StreamRun)));
      }
      const bool fresh = !r->stats_valid;
      if (fresh) init_stats(r);
      r->stats_valid = true;
      double *samples = nullptr;
      long long cap = 0;
      if (record_samples) {
        cap = std::max<long long>(1, n_passes - n_equil);
        if (cap > r->sample_capacity) {
          cudaFree(r->d_samples);
          r->d_samples = nullptr;
          CUDA_OK(cudaMalloc(&r->d_samples, sizeof(double) * cap * r->sample_width * r->n));
          r->sample_capacity = cap;
        }
        samples = r->d_samples;
        cap = r->sample_capacity;
        r->n_samples_recorded = std::max<long long>(0, n_passes - n_equil);
      }
      {
        // pass counter at the start of this run (restored states keep theirs);
        // samples are indexed by the sample count: restart the moments
        std::vector<ReplicaStats> st(r->n);
        CUDA_OK(cudaMemcpyAsync(st.data(), r->d_stats, sizeof(ReplicaStats) * r->n,
                                cudaMemcpyDeviceToHost, r->stream));
        CUDA_OK(cudaStreamSynchronize(r->stream));
        r->stream_pass = st[0].pass;
        for (const auto &x : st)
          require(x.pass == r->stream_pass, "streamed replicas must share one pass counter");
        if (fresh || record_samples) {
          for (auto &x : st) {
            x.n_samples = 0;
            x.sum_e = x.sum_e2 = x.sum_f = 0;
            for (int k = 0; k < 3; ++k) x.sum_x[k] = x.sum_ex[k] = 0;
            for (int k = 0; k < 9; ++k) x.sum_xx[k] = 0;
          }
          CUDA_OK(cudaMemcpyAsync(r->d_stats, st.data(), sizeof(ReplicaStats) * r->n,
                                  cudaMemcpyHostToDevice, r->stream));
        }
      }
      double RT[16] = {0};
      for (size_t k = 0; k < r->sys->RT.size() && k < 16; ++k) RT[k] = r->sys->RT[k];
      long long launched = 0;
      CUDA_OK(stream_run(r->sys->T, r->sstate, r->d_reps, r->d_stats, r->d_occ, r->n, L,
                         r->stream_pitch, r->max_classes,
                         r->ensemble == CEM_CANONICAL ? r->n_pair_sweeps : 0,
                         r->ensemble == CEM_CANONICAL ? r->n_local_sweeps : 1, RT, n_passes, n_equil,
                         r->stream_pass, samples, cap, r->sample_width, fresh ? 1 : 0, r->stream,
                         r->ev0, r->ev1, r->h_stop, &launched));
      r->stream_pass += launched;
      return;
    }
    // binary systems compute the exact initial stats inside the sweep kernel
    // (the orbit-at-a-time kernel has no fused initial energy)
    const bool fused_init = !r->stats_valid && r->sys->T.n_occ == 2 && r->pitch >= 0;
    if (!r->stats_valid && !fused_init) init_stats(r);
    SweepParams P{};
    P.init = fused_init ? 1 : 0;
    r->stats_valid = true;
    P.reps = r->d_reps;
    P.stats = r->d_stats;
    P.occ = r->d_occ;
    P.n_passes = n_passes;
    P.n_equil = n_equil;
    P.max_classes = r->max_classes;
    P.max_sub = sub_steps(r);
    P.pack16 = (r->pitch == -2 && !r->wide_records && fits_pack16(r)) ? 1 : 0;
    P.n_pair_sweeps = r->n_pair_sweeps;
    P.n_local_sweeps = r->n_local_sweeps;
    P.cta_rep = r->d_cta_rep;
    P.stop = r->d_stop;
    P.cluster = sweep_cluster_for(r->sweep_cluster, r->pitch, r->threads, r->reps);
    r->last_sweep_cluster = P.cluster;
    const CeTables &T = r->sys->T;
    for (size_t k = 0; k < r->sys->RT.size() && k < 16; ++k) P.RT[k] = r->sys->RT[k];
    if (record_samples) {
      const long long cap = std::max<long long>(1, n_passes - n_equil);
      if (cap > r->sample_capacity) {
        cudaFree(r->d_samples);
        r->d_samples = nullptr;
        CUDA_OK(cudaMalloc(&r->d_samples, sizeof(double) * cap * r->sample_width * r->n));
        r->sample_capacity = cap;
      }
      P.samples = r->d_samples;
      P.sample_capacity = r->sample_capacity;
      P.sample_width = r->sample_width;
      // samples are indexed by the replica's sample count: restart it
      std::vector<ReplicaStats> s(r->n);
      CUDA_OK(cudaMemcpyAsync(s.data(), r->d_stats, sizeof(ReplicaStats) * r->n,
                              cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
      for (auto &x : s) {
        x.n_samples = 0;
        x.sum_e = x.sum_e2 = x.sum_f = 0;
        for (int k = 0; k < 3; ++k) x.sum_x[k] = x.sum_ex[k] = 0;
        for (int k = 0; k < 9; ++k) x.sum_xx[k] = 0;
      }
      CUDA_OK(cudaMemcpyAsync(r->d_stats, s.data(), sizeof(ReplicaStats) * r->n,
                              cudaMemcpyHostToDevice, r->stream));
      r->n_samples_recorded = std::max<long long>(0, n_passes - n_equil);
    }
    CUDA_OK(cudaEventRecord(r->ev0, r->stream));
    CUDA_OK(launch_sweep(T, P, r->n, r->sweep_smem, r->pitch, r->threads, r->stream));
    CUDA_OK(cudaEventRecord(r->ev1, r->stream));
  });
}

int cem_get_stats(cem_replicas *r, int i, cem_stats *out) {
  return guard([&] {
    check_rep(r, i);
    require(out != nullptr, "null output");
    ReplicaStats S;
    CUDA_OK(cudaMemcpyAsync(&S, r->d_stats + i, sizeof(S), cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    if (S.status == 5)
      throw Err(CEM_ERR_DEVICE,
                "a shared-memory staging copy did not complete; the replica was left unchanged");
    if (S.status == 8)
      throw Err(CEM_ERR_DEVICE,
                "a tensor-core MMA of the learned group sweep did not complete within the wait "
                "limit; the run's results are invalid");
    if (S.status == 6)
      throw Err(CEM_ERR_DEVICE,
                "a shared-memory staging copy did not complete and was still in flight when the "
                "kernel gave up waiting; the replica was left unchanged");
    std::memset(out, 0, sizeof(*out));
    const int nc = r->sys->T.n_occ - 1;
    out->n_samples = S.n_samples;
    const double n = S.n_samples;
    if (n > 0) {
      out->mean_potential = S.sum_e / n;
      out->var_potential = S.sum_e2 / n - out->mean_potential * out->mean_potential;
      out->mean_formation = S.sum_f / n;
      for (int k = 0; k < nc; ++k) out->mean_comp[k] = S.sum_x[k] / n;
      for (int k = 0; k < nc; ++k) {
        out->cov_e_comp[k] = S.sum_ex[k] / n - out->mean_potential * out->mean_comp[k];
        for (int k2 = 0; k2 < nc; ++k2)
          out->cov_comp[k * 3 + k2] = S.sum_xx[k * 3 + k2] / n - out->mean_comp[k] * out->mean_comp[k2];
      }
    }
    out->energy = S.energy;
    out->n_proposed = S.n_proposed;
    out->n_accepted = S.n_accepted;
    out->passes = S.pass;
  });
}

int cem_get_samples(cem_replicas *r, int i, double *potential, double *comp, int64_t capacity,
                    int64_t *n_samples) {
  return guard([&] {
    check_rep(r, i);
    require(r->d_samples != nullptr, "no samples were recorded");
    const int64_t n = std::min<int64_t>(r->n_samples_recorded, r->sample_capacity);
    const int64_t m = std::min<int64_t>(n, capacity);
    std::vector<double> buf((size_t)m * r->sample_width);
    if (m > 0)
      CUDA_OK(cudaMemcpyAsync(buf.data(),
                              r->d_samples + (size_t)i * r->sample_capacity * r->sample_width,
                              sizeof(double) * buf.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    const int nc = r->sys->T.n_occ - 1;
    for (int64_t s = 0; s < m; ++s) {
      if (potential) potential[s] = buf[s * r->sample_width];
      if (comp)
        for (int k = 0; k < nc; ++k) comp[s * nc + k] = buf[s * r->sample_width + 1 + k];
    }
    if (n_samples) *n_samples = m;
  });
}

int cem_smem_bandwidth(double *gbs) {
  return guard([&] {
    require(gbs != nullptr, "null output");
    CUDA_OK(smem_bandwidth(gbs, 0));
  });
}

int cem_autotune(cem_replicas *r, int64_t trial_passes, double *best_ms) {
  return guard([&] {
    require(r != nullptr, "null handle");
    require_sweepable(r);
    require(trial_passes > 0, "trial_passes must be > 0");
    if (best_ms) *best_ms = 0.0;
    if (r->streamed) return;  // one fixed graph per pass
    int8_t *occ_save = nullptr;
    ReplicaStats *st_save = nullptr;
    auto cleanup = [&] {
      cudaFree(occ_save);
      cudaFree(st_save);
    };
    try {
      CUDA_OK(cudaMalloc(&occ_save, (size_t)r->total_sites + 16));
      CUDA_OK(cudaMalloc(&st_save, sizeof(ReplicaStats) * r->n));
      CUDA_OK(cudaMemcpyAsync(occ_save, r->d_occ, (size_t)r->total_sites, cudaMemcpyDeviceToDevice,
                              r->stream));
      CUDA_OK(cudaMemcpyAsync(st_save, r->d_stats, sizeof(ReplicaStats) * r->n,
                              cudaMemcpyDeviceToDevice, r->stream));
      const bool valid0 = r->stats_valid;
      auto restore = [&] {
        CUDA_OK(cudaMemcpyAsync(r->d_occ, occ_save, (size_t)r->total_sites,
                                cudaMemcpyDeviceToDevice, r->stream));
        CUDA_OK(cudaMemcpyAsync(r->d_stats, st_save, sizeof(ReplicaStats) * r->n,
                                cudaMemcpyDeviceToDevice, r->stream));
        r->stats_valid = valid0;
      };
      double best = 1e300;
      int bt = r->threads, bo = r->cta_order;
      for (int th : {SWEEP_THREADS, 256})
        for (int order : {0, 1}) {
          if (th != SWEEP_THREADS && r->sys->big) continue;
          restore();
          r->threads = th;
          set_cta_order(r, order);
          if (cem_run(r, trial_passes, 0, 0) != CEM_OK) throw Err(CEM_ERR_CUDA, cem_last_error());
          CUDA_OK(cudaEventSynchronize(r->ev1));
          float ms = 0.f;
          CUDA_OK(cudaEventElapsedTime(&ms, r->ev0, r->ev1));
          if (ms < best) {
            best = ms;
            bt = th;
            bo = order;
          }
        }
      restore();
      r->threads = bt;
      set_cta_order(r, bo);
      CUDA_OK(cudaStreamSynchronize(r->stream));
      if (best_ms) *best_ms = best;
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int cem_set_option(cem_replicas *r, const char *key, int64_t value) {
  return guard([&] {
    require(r && key, "null argument");
    const std::string k(key);
    if (k == "pair_sweeps") {
      require(value >= 0 && value + r->n_local_sweeps <= MAX_SWEEPS_API, "too many sweeps");
      r->n_pair_sweeps = (int)value;
    } else if (k == "local_sweeps") {
      require(value >= 1 && value + r->n_pair_sweeps <= MAX_SWEEPS_API,
              "local_sweeps must be >= 1 (swaps between colour classes keep the chain ergodic)");
      r->n_local_sweeps = (int)value;
    } else if (k == "streamed") {
      require(value == 1, "streamed can only be switched on");
      const int sp = stream_pitch_for(*r->sys, r->reps);
      require(sp != 0, "this batch has no HBM-streamed kernel", CEM_ERR_UNSUPPORTED);
      r->streamed = true;
      r->stream_pitch = sp;
    } else if (k == "threads") {
      require(value == 512 || value == 256, "threads must be 512 or 256 (two replicas per SM)");
      require(value == 512 || !r->sys->big,
              "cluster expansions with more than 8 orbits run 512 threads per replica",
              CEM_ERR_UNSUPPORTED);
      r->threads = (int)value;
    } else if (k == "cta_order") {
      set_cta_order(r, (int)value);
    } else if (k == "sweep_cluster") {
      // CTAs per replica of the plain sweep (0: automatic); the chain does
      // not depend on it
      require(value == 0 || value == 1 || value == 2 || value == 4 || value == 8,
              "sweep_cluster must be 0 (automatic), 1, 2, 4 or 8");
      r->sweep_cluster = (int)value;
    } else if (k == "group_cluster") {
      // CTAs per replica of the learned group sweep (0: as many of 4, 2, 1
      // as keep every replica's cluster on its own SMs)
      require(value == 0 || value == 1 || value == 2 || value == 4,
              "group_cluster must be 0 (automatic), 1, 2 or 4");
      r->group_cluster = (int)value;
    } else if (k == "orbit_walk") {
      // the kernels of large cluster expansions, also for small ones:
      // 1 = one thread per site walking the tables one orbit at a time,
      // 2 = one warp per site change (binary, orbits sorted by size)
      require(value == 1 || value == 2, "orbit_walk must be 1 or 2");
      require(value == 1 || r->sys->split_ok,
              "orbit_walk 2 needs a binary system with split weights", CEM_ERR_UNSUPPORTED);
      r->pitch = value == 1 ? -1 : -2;
      r->threads = SWEEP_THREADS;
    } else if (k == "wide_records") {
      // the cooperative sweep's 32-bit cluster records even where 16-bit
      // ones fit (same sums, same chain)
      r->wide_records = value != 0;
      if (r->step_exec) cudaGraphExecDestroy(r->step_exec);  // captured with the old layout
      r->step_exec = nullptr;
    } else if (k == "generic_evaluator") {
      if (value) {
        r->pitch = r->sys->big ? (r->sys->coop ? -2 : -1) : 0;
      } else {
        throw Err(CEM_ERR_INVALID, "generic_evaluator can only be switched on");
      }
    } else {
      throw Err(CEM_ERR_INVALID, "unknown option '" + k + "'");
    }
    // the evaluator and the sweep counts set the kernel's shared-memory layout
    r->sweep_smem = batch_smem(r, r->pitch);
  });
}

int cem_get_option(cem_replicas *r, const char *key, int64_t *value) {
  return guard([&] {
    require(r && key && value, "null argument");
    const std::string k(key);
    if (k == "pair_sweeps") *value = r->n_pair_sweeps;
    else if (k == "local_sweeps") *value = r->n_local_sweeps;
    else if (k == "pitch") *value = r->pitch;
    else if (k == "smem_bytes") *value = r->sweep_smem;
    else if (k == "colour_classes") *value = r->max_classes;
    else if (k == "streamed") *value = r->streamed ? 1 : 0;
    else if (k == "threads") *value = r->threads;
    else if (k == "cta_order") *value = r->cta_order;
    else if (k == "group_cluster") *value = r->last_group_cluster;
    else if (k == "sweep_cluster") *value = r->last_sweep_cluster;
    else throw Err(CEM_ERR_INVALID, "unknown option '" + k + "'");
  });
}

int cem_state_bytes(const cem_replicas *r, int64_t *bytes) {
  return guard([&] {
    require(r && bytes, "null argument");
    *bytes = (int64_t)sizeof(ReplicaStats);
  });
}

int cem_get_state(cem_replicas *r, int i, int8_t *occ, void *state) {
  return guard([&] {
    check_rep(r, i);
    require(occ && state, "null argument");
    const Replica &R = r->reps[i];
    if (!r->stats_valid) {
      r->upload_reps();
      init_stats(r);
    }
    CUDA_OK(cudaMemcpyAsync(occ, r->d_occ + R.occ_offset, R.n_sites, cudaMemcpyDeviceToHost,
                            r->stream));
    CUDA_OK(cudaMemcpyAsync(state, r->d_stats + i, sizeof(ReplicaStats), cudaMemcpyDeviceToHost,
                            r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
  });
}

int cem_set_state(cem_replicas *r, int i, const int8_t *occ, const void *state) {
  return guard([&] {
    check_rep(r, i);
    require(occ && state, "null argument");
    const Replica &R = r->reps[i];
    for (int l = 0; l < R.n_sites; ++l)
      require(occ[l] >= 0 && occ[l] < r->sys->T.n_occ, "occupant index out of range");
    ReplicaStats S;
    std::memcpy(&S, state, sizeof(S));
    long long tot = 0;
    for (int a = 0; a < r->sys->T.n_occ; ++a) tot += S.n_species[a];
    require(tot == R.n_sites && std::isfinite(S.energy), "state does not belong to this replica");
    if (!r->stats_valid) {
      r->upload_reps();
      init_stats(r);
    }
    CUDA_OK(cudaMemcpyAsync(r->d_occ + R.occ_offset, occ, R.n_sites, cudaMemcpyHostToDevice,
                            r->stream));
    CUDA_OK(cudaMemcpyAsync(r->d_stats + i, &S, sizeof(S), cudaMemcpyHostToDevice, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    r->stats_valid = true;
  });
}

int cem_get_order_samples(cem_replicas *r, int i, double *order, int64_t capacity,
                          int64_t *n_samples) {
  return guard([&] {
    check_rep(r, i);
    require(r->d_samples != nullptr, "no samples were recorded");
    const int64_t n = std::min<int64_t>(r->n_samples_recorded, r->sample_capacity);
    const int64_t m = std::min<int64_t>(n, capacity);
    std::vector<double> buf((size_t)m * r->sample_width);
    if (m > 0)
      CUDA_OK(cudaMemcpyAsync(buf.data(),
                              r->d_samples + (size_t)i * r->sample_capacity * r->sample_width,
                              sizeof(double) * buf.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    for (int64_t s = 0; s < m; ++s) order[s] = buf[s * r->sample_width + r->sys->T.n_occ];
    if (n_samples) *n_samples = m;
  });
}

int cem_synchronize(cem_replicas *r) {
  int stopped = 0;
  const int rc = guard([&] {
    require(r != nullptr, "null handle");
    CUDA_OK(cudaStreamSynchronize(r->stream));
    stopped = *r->h_stop;
  });
  return rc == CEM_OK && stopped ? CEM_STOPPED : rc;
}

int cem_request_stop(cem_replicas *r) {
  if (!r) return CEM_ERR_INVALID;
  *r->h_stop = 1;
  std::atomic_thread_fence(std::memory_order_seq_cst);
  return CEM_OK;
}

int cem_last_kernel_ms(cem_replicas *r, double *ms) {
  return guard([&] {
    require(r && ms, "null argument");
    CUDA_OK(cudaEventSynchronize(r->ev1));
    float f = 0.f;
    CUDA_OK(cudaEventElapsedTime(&f, r->ev0, r->ev1));
    *ms = f;
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Delta energies without any device allocation.
//
// Some callers cannot allocate device memory: a host program whose device
// memory is owned by another framework's pool (which reserves the device and
// expects no raw cudaMalloc), or a Monte Carlo driver that evaluates events in
// a tight per-event loop and cannot afford the device-wide synchronisation that
// cudaMalloc/cudaFree imply. cem_delta_energy_noalloc serves them: it stages
// the events and results in one fixed array in device global memory that is
// part of the library image (every device that loads the library holds it
// until the process exits), instead of allocating per call.
//
// Limits: at most CEM_NOALLOC_MAX_EVENTS events of at most
// CEM_NOALLOC_MAX_SITES sites per call; larger calls are rejected. The array
// is CEM_NOALLOC_SCRATCH_BYTES bytes (cem.h; checked below against its
// layout), dominated by the delta-correlation section sized for MAX_FUNCS
// functions per event.
// All calls share the array and it keeps the last call's contents; calls that
// overlap on the GPU (different streams or batches at the same time) race.
namespace {

constexpr int NOALLOC_MAX_EVENTS = CEM_NOALLOC_MAX_EVENTS;
constexpr int NOALLOC_MAX_SITES = CEM_NOALLOC_MAX_SITES;
constexpr size_t NA_SITES = 0;                                                   // int64
constexpr size_t NA_NEW = NA_SITES + 8ull * NOALLOC_MAX_EVENTS * NOALLOC_MAX_SITES;  // int32
constexpr size_t NA_DE = NA_NEW + 4ull * NOALLOC_MAX_EVENTS * NOALLOC_MAX_SITES;    // double
constexpr size_t NA_DC = NA_DE + 8ull * NOALLOC_MAX_EVENTS;                         // int64
constexpr size_t NA_DMU = NA_DC + 8ull * NOALLOC_MAX_EVENTS * MAX_FUNCS;            // double[16]
constexpr size_t NA_BYTES = NA_DMU + 8 * 16;
static_assert(NA_NEW % 256 == 0 && NA_DE % 256 == 0 && NA_DC % 256 == 0 && NA_DMU % 256 == 0,
              "scratch sections are 256-byte aligned");
static_assert(NA_BYTES == CEM_NOALLOC_SCRATCH_BYTES,
              "the scratch size stated in cem.h is the size of the array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[NA_MAX_DEVICES] = {nullptr};

// Device address of the scratch array on the batch's device; resolved once
// per device (the host-side name is only a stand-in, not a device address).
// The batch's device must be the calling thread's current device: the
// address, the batch's stream and its occupations all belong to it.
unsigned char *noalloc_scratch(const cem_replicas *r) {
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  require(dev == r->device,
          "cem_delta_energy_noalloc: the current device (" + std::to_string(dev) +
              ") is not the device the batch was created on (" + std::to_string(r->device) +
              "); make that device current first");
  require(dev >= 0 && dev < NA_MAX_DEVICES, "device index out of range", CEM_ERR_UNSUPPORTED);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    CUDA_OK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
  }
  return g_noalloc_ptr[dev];
}

}  // namespace

extern "C" int cem_delta_energy_noalloc(cem_replicas *r, int i, int n_events, int k,
                                        const int64_t *sites, const int32_t *new_occ,
                                        int potential, double *dE, int64_t *dcount) {
  return guard([&] {
    check_rep(r, i);
    require(n_events >= 0 && k >= 1 && k <= 4, "sites_per_event must be 1..4");
    require(n_events <= NOALLOC_MAX_EVENTS,
            "cem_delta_energy_noalloc handles at most " + std::to_string(NOALLOC_MAX_EVENTS) +
                " events per call (got " + std::to_string(n_events) + ")",
            CEM_ERR_UNSUPPORTED);
    require(sites && new_occ && dE, "null argument");
    unsigned char *base = noalloc_scratch(r);  // first call on a device resolves the address
    if (n_events == 0) return;
    const Replica &R = r->reps[i];
    const CeTables &T = r->sys->T;
    for (int64_t e = 0; e < (int64_t)n_events * k; ++e) {
      require(sites[e] >= 0 && sites[e] < R.n_sites, "site index out of range");
      require(new_occ[e] >= 0 && new_occ[e] < T.n_occ, "occupant index out of range");
    }
    require(potential == 0 || r->ensemble == CEM_SEMIGRAND_CANONICAL,
            "the semi-grand potential needs semi-grand canonical replicas");
    long long *ds = reinterpret_cast<long long *>(base + NA_SITES);
    int *dn = reinterpret_cast<int *>(base + NA_NEW);
    double *dde = reinterpret_cast<double *>(base + NA_DE);
    long long *ddc = reinterpret_cast<long long *>(base + NA_DC);
    double *ddmu = reinterpret_cast<double *>(base + NA_DMU);
    const size_t ne = (size_t)n_events * k;
    CUDA_OK(cudaMemcpyAsync(ds, sites, ne * 8, cudaMemcpyHostToDevice, r->stream));
    CUDA_OK(cudaMemcpyAsync(dn, new_occ, ne * 4, cudaMemcpyHostToDevice, r->stream));
    if (potential)
      CUDA_OK(cudaMemcpyAsync(ddmu, R.dmu, 16 * 8, cudaMemcpyHostToDevice, r->stream));
    // every dE (and dcount) entry of the call is written by the kernel
    CUDA_OK(launch_delta(T, r->d_occ + R.occ_offset, R.cells(), n_events, k, ds, dn,
                         potential ? ddmu : nullptr, dde, dcount ? ddc : nullptr, r->stream));
    CUDA_OK(cudaMemcpyAsync(dE, dde, (size_t)n_events * 8, cudaMemcpyDeviceToHost, r->stream));
    if (dcount)
      CUDA_OK(cudaMemcpyAsync(dcount, ddc, (size_t)n_events * T.n_funcs * 8,
                              cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
  });
}

// ---------------------------------------------------------------------------
// Learned proposal: network objects and the sampler.
struct cem_mlp {
  float *d_master = nullptr, *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr;
  __nv_bfloat16 *d_params = nullptr;
  double *d_loss = nullptr;
  int step = 0;
  cudaStream_t stream = nullptr;
  ~cem_mlp() {
    cudaFree(d_master);
    cudaFree(d_grad);
    cudaFree(d_m);
    cudaFree(d_v);
    cudaFree(d_params);
    cudaFree(d_loss);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int cem_mlp_info(int *n_inputs, int *n_hidden, int *n_params) {
  return guard([&] {
    if (n_inputs) *n_inputs = MLP_IN;
    if (n_hidden) *n_hidden = MLP_H;
    if (n_params) *n_params = MLP_NPARAM;
  });
}

int cem_mlp_create(uint64_t seed, cem_mlp **out) {
  return guard([&] {
    require(out != nullptr, "null output");
    *out = nullptr;
    auto m = std::make_unique<cem_mlp>();
    CUDA_OK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    CUDA_OK(cudaMalloc(&m->d_master, MLP_NPARAM * 4));
    CUDA_OK(cudaMalloc(&m->d_grad, MLP_NPARAM * 4));
    CUDA_OK(cudaMalloc(&m->d_m, MLP_NPARAM * 4));
    CUDA_OK(cudaMalloc(&m->d_v, MLP_NPARAM * 4));
    CUDA_OK(cudaMalloc(&m->d_params, MLP_NPARAM * 2));
    CUDA_OK(cudaMalloc(&m->d_loss, 8));
    CUDA_OK(cudaMemset(m->d_grad, 0, MLP_NPARAM * 4));
    CUDA_OK(cudaMemset(m->d_m, 0, MLP_NPARAM * 4));
    CUDA_OK(cudaMemset(m->d_v, 0, MLP_NPARAM * 4));
    // He-style initialisation from a seeded stream (host side, once)
    std::vector<float> h(MLP_NPARAM, 0.f);
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + 1ull;
    auto gauss = [&]() {
      double s = 0.0;  // sum of 12 uniforms - 6: approximately N(0, 1)
      for (int k = 0; k < 12; ++k) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        s += (double)(x >> 11) * (1.0 / 9007199254740992.0);
      }
      return (float)(s - 6.0);
    };
    for (int i = 0; i < MLP_IN * MLP_H; ++i) h[MLP_W1 + i] = gauss() * std::sqrt(2.f / MLP_IN);
    for (int i = 0; i < MLP_H * MLP_H; ++i) h[MLP_W2 + i] = gauss() * std::sqrt(2.f / MLP_H);
    for (int i = 0; i < MLP_H; ++i) h[MLP_W3 + i] = gauss() * std::sqrt(1.f / MLP_H);
    CUDA_OK(cudaMemcpy(m->d_master, h.data(), MLP_NPARAM * 4, cudaMemcpyHostToDevice));
    CUDA_OK(mlp_pack(m->d_master, m->d_params, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
    *out = m.release();
  });
}

int cem_mlp_destroy(cem_mlp *m) {
  return guard([&] { delete m; });
}

int cem_mlp_get_params(cem_mlp *m, float *master) {
  return guard([&] {
    require(m && master, "null argument");
    CUDA_OK(cudaMemcpy(master, m->d_master, MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
  });
}

int cem_mlp_set_params(cem_mlp *m, const float *master) {
  return guard([&] {
    require(m && master, "null argument");
    for (int i = 0; i < MLP_NPARAM; ++i) require(std::isfinite(master[i]), "non-finite parameter");
    CUDA_OK(cudaMemcpy(m->d_master, master, MLP_NPARAM * 4, cudaMemcpyHostToDevice));
    CUDA_OK(mlp_pack(m->d_master, m->d_params, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  });
}

int cem_mlp_forward(cem_mlp *m, int64_t n, const int8_t *features, float *logits) {
  return guard([&] {
    require(m && features && logits && n >= 0, "bad argument");
    if (n == 0) return;
    int8_t *dx = nullptr;
    float *dz = nullptr;
    try {
      CUDA_OK(cudaMalloc(&dx, (size_t)n * MLP_IN));
      CUDA_OK(cudaMalloc(&dz, (size_t)n * 4));
      CUDA_OK(cudaMemcpyAsync(dx, features, (size_t)n * MLP_IN, cudaMemcpyHostToDevice, m->stream));
      CUDA_OK(mlp_forward(m->d_params, dx, n, dz, m->stream));
      CUDA_OK(cudaMemcpyAsync(logits, dz, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream));
      CUDA_OK(cudaStreamSynchronize(m->stream));
    } catch (...) {
      cudaFree(dx);
      cudaFree(dz);
      throw;
    }
    cudaFree(dx);
    cudaFree(dz);
  });
}

int cem_mlp_forward_tc(cem_mlp *m, int64_t n, const int8_t *features, float *logits) {
  return guard([&] {
    require(m && features && logits && n >= 0, "bad argument");
    if (n == 0) return;
    int8_t *dx = nullptr;
    float *dz = nullptr;
    int *dst = nullptr;
    auto cleanup = [&] {
      cudaFree(dx);
      cudaFree(dz);
      cudaFree(dst);
    };
    try {
      CUDA_OK(cudaMalloc(&dx, (size_t)n * MLP_IN));
      CUDA_OK(cudaMalloc(&dz, (size_t)n * 4));
      CUDA_OK(cudaMalloc(&dst, 4));
      CUDA_OK(cudaMemsetAsync(dst, 0, 4, m->stream));
      CUDA_OK(cudaMemcpyAsync(dx, features, (size_t)n * MLP_IN, cudaMemcpyHostToDevice, m->stream));
      CUDA_OK(mlp_forward_tc(m->d_params, dx, n, dz, dst, m->stream));
      int status = 0;
      CUDA_OK(cudaMemcpyAsync(logits, dz, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream));
      CUDA_OK(cudaMemcpyAsync(&status, dst, 4, cudaMemcpyDeviceToHost, m->stream));
      CUDA_OK(cudaStreamSynchronize(m->stream));
      if (status) throw Err(CEM_ERR_DEVICE, "a tensor-core MMA did not complete within the wait limit");
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int cem_mlp_gradient(cem_mlp *m, int64_t n, const int8_t *features, const float *targets,
                     float *grad, double *loss) {
  return guard([&] {
    require(m && features && targets && grad && n > 0, "bad argument");
    int8_t *dx = nullptr;
    float *dt = nullptr;
    try {
      CUDA_OK(cudaMalloc(&dx, (size_t)n * MLP_IN));
      CUDA_OK(cudaMalloc(&dt, (size_t)n * 4));
      CUDA_OK(cudaMemcpyAsync(dx, features, (size_t)n * MLP_IN, cudaMemcpyHostToDevice, m->stream));
      CUDA_OK(cudaMemcpyAsync(dt, targets, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
      CUDA_OK(cudaMemsetAsync(m->d_grad, 0, MLP_NPARAM * 4, m->stream));
      CUDA_OK(cudaMemsetAsync(m->d_loss, 0, 8, m->stream));
      CUDA_OK(mlp_grad(m->d_params, dx, dt, nullptr, 0, n, m->d_grad, m->d_loss, m->stream));
      CUDA_OK(cudaMemcpyAsync(grad, m->d_grad, MLP_NPARAM * 4, cudaMemcpyDeviceToHost, m->stream));
      double l = 0.0;
      CUDA_OK(cudaMemcpyAsync(&l, m->d_loss, 8, cudaMemcpyDeviceToHost, m->stream));
      CUDA_OK(cudaMemsetAsync(m->d_grad, 0, MLP_NPARAM * 4, m->stream));
      CUDA_OK(cudaStreamSynchronize(m->stream));
      if (loss) *loss = l / (double)n;
    } catch (...) {
      cudaFree(dx);
      cudaFree(dt);
      throw;
    }
    cudaFree(dx);
    cudaFree(dt);
  });
}

int cem_mlp_train(cem_mlp *m, int64_t n, const int8_t *features, const float *targets,
                  int epochs, int batch, float lr, uint64_t seed, double *loss_per_epoch) {
  return guard([&] {
    require(m && features && targets && n > 0 && epochs >= 1 && batch >= 1 && lr > 0.f,
            "bad argument");
    require(n < (1ll << 31), "too many training samples");
    int8_t *dx = nullptr;
    float *dt = nullptr;
    int *dord = nullptr;
    auto cleanup = [&] {
      cudaFree(dx);
      cudaFree(dt);
      cudaFree(dord);
    };
    try {
      CUDA_OK(cudaMalloc(&dx, (size_t)n * MLP_IN));
      CUDA_OK(cudaMalloc(&dt, (size_t)n * 4));
      CUDA_OK(cudaMalloc(&dord, (size_t)n * 4));
      CUDA_OK(cudaMemcpyAsync(dx, features, (size_t)n * MLP_IN, cudaMemcpyHostToDevice, m->stream));
      CUDA_OK(cudaMemcpyAsync(dt, targets, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
      std::vector<int> order((size_t)n);
      for (int64_t i = 0; i < n; ++i) order[i] = (int)i;
      std::mt19937_64 eng(seed);
      for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), eng);
        CUDA_OK(cudaMemcpyAsync(dord, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice,
                                m->stream));
        CUDA_OK(cudaMemsetAsync(m->d_loss, 0, 8, m->stream));
        for (int64_t b0 = 0; b0 < n; b0 += batch) {
          const int64_t nb = std::min<int64_t>(batch, n - b0);
          CUDA_OK(mlp_grad(m->d_params, dx, dt, dord, b0, nb, m->d_grad, m->d_loss, m->stream));
          CUDA_OK(mlp_adam(m->d_master, m->d_params, m->d_grad, m->d_m, m->d_v, lr, ++m->step,
                           m->stream));
        }
        double l = 0.0;
        CUDA_OK(cudaMemcpyAsync(&l, m->d_loss, 8, cudaMemcpyDeviceToHost, m->stream));
        CUDA_OK(cudaStreamSynchronize(m->stream));
        if (loss_per_epoch) loss_per_epoch[ep] = l / (double)n;
      }
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

static void require_learned(const cem_replicas *r) {
  require(r->sys->fcc_generated && r->ensemble == CEM_CANONICAL,
          "the learned proposal supports canonical binary FCC systems of the generated topology",
          CEM_ERR_UNSUPPORTED);
  for (const Replica &R : r->reps)
    require(R.L[0] == R.L[1] && R.L[1] == R.L[2] && R.L[0] == r->reps[0].L[0] &&
                (R.L[0] + 4 == 14 || R.L[0] + 4 == 28 || R.L[0] + 4 == 36 || R.L[0] + 4 == 52),
            "the learned proposal needs equal cubic supercells of 10, 24, 32 or 48 cells",
            CEM_ERR_UNSUPPORTED);
}

int cem_learned_features(cem_replicas *r, int i, int8_t *features, float *targets) {
  return guard([&] {
    check_rep(r, i);
    require_box(r);
    require(features && targets, "null argument");
    require(r->sys->fcc_generated && r->ensemble == CEM_CANONICAL,
            "the learned proposal supports canonical binary FCC systems of the generated topology",
            CEM_ERR_UNSUPPORTED);
    require(r->reps[i].L[0] == r->reps[i].L[1] && r->reps[i].L[1] == r->reps[i].L[2],
            "features need a cubic supercell", CEM_ERR_UNSUPPORTED);
    const Replica &R = r->reps[i];
    const int n = R.n_sites;
    int8_t *dx = nullptr;
    float *dt = nullptr;
    double *dw = nullptr;
    int *dof = nullptr;
    auto cleanup = [&] {
      cudaFree(dx);
      cudaFree(dt);
      cudaFree(dw);
      cudaFree(dof);
    };
    try {
      CUDA_OK(cudaMalloc(&dx, (size_t)n * MLP_IN));
      CUDA_OK(cudaMalloc(&dt, (size_t)n * 4));
      CUDA_OK(cudaMalloc(&dw, 8 * r->sys->w.size()));
      CUDA_OK(cudaMalloc(&dof, 4 * MAX_ORBITS));
      CUDA_OK(cudaMemcpyAsync(dw, r->sys->w.data(), 8 * r->sys->w.size(), cudaMemcpyHostToDevice,
                              r->stream));
      CUDA_OK(cudaMemcpyAsync(dof, r->sys->T.orb_func_base, 4 * MAX_ORBITS, cudaMemcpyHostToDevice,
                              r->stream));
      CUDA_OK(learned_features(r->d_occ + R.occ_offset, R.L[0], dw, dof, R.beta, dx, dt, r->stream));
      CUDA_OK(cudaMemcpyAsync(features, dx, (size_t)n * MLP_IN, cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaMemcpyAsync(targets, dt, (size_t)n * 4, cudaMemcpyDeviceToHost, r->stream));
      CUDA_OK(cudaStreamSynchronize(r->stream));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int cem_learned_run(cem_replicas *r, const cem_mlp *m, int64_t n_passes, int64_t n_equil,
                    int record_samples) {
  return guard([&] {
    require(r != nullptr, "null handle");
    require_box(r);
    require(n_passes >= 0 && n_equil >= 0, "pass counts must be >= 0");
    require_learned(r);
    const int L = r->reps[0].L[0], n = r->reps[0].n_sites;
    const int pitch = L + 4;
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    require(learned_smem_bytes(L, pitch) <= maxsm, "supercell does not fit in shared memory",
            CEM_ERR_UNSUPPORTED);
    r->upload_reps();
    const long long tsize = learned_tree_size(n);
    if (!r->d_lw) {
      CUDA_OK(cudaMalloc(&r->d_lw, sizeof(long long) * (size_t)n * r->n));
      CUDA_OK(cudaMalloc(&r->d_trees, sizeof(unsigned long long) * (size_t)tsize * 2 * r->n));
    }
    double *samples = nullptr;
    long long cap = 0;
    if (record_samples) {
      cap = std::max<long long>(1, n_passes - n_equil);
      if (cap > r->lsample_capacity) {
        cudaFree(r->d_lsamples);
        r->d_lsamples = nullptr;
        CUDA_OK(cudaMalloc(&r->d_lsamples, sizeof(double) * 3 * cap * r->n));
        r->lsample_capacity = cap;
      }
      samples = r->d_lsamples;
      cap = r->lsample_capacity;
      r->lsamples_recorded = std::max<long long>(0, n_passes - n_equil);
    }
    CUDA_OK(cudaEventRecord(r->ev0, r->stream));
    CUDA_OK(learned_run(r->sys->T, r->d_reps, r->d_stats, r->d_occ, m ? m->d_params : nullptr,
                        m ? 1 : 0, r->d_lw, n, r->d_trees, tsize, n, r->n, L, n_passes, n_equil,
                        samples, cap, pitch, r->stream));
    CUDA_OK(cudaEventRecord(r->ev1, r->stream));
    r->stats_valid = false;  // the sweep recomputes its own state next time
  });
}

int cem_learned_group_run(cem_replicas *r, const cem_mlp *m, int weights, int rounds,
                          int local_substeps, int64_t n_passes, int64_t n_equil,
                          int record_samples) {
  return guard([&] {
    require(r != nullptr, "null handle");
    require_box(r);
    require(n_passes >= 0 && n_equil >= 0, "pass counts must be >= 0");
    require(weights >= 0 && weights <= 2, "weights must be 0 (uniform), 1 (network) or 2 (exact)");
    require(weights != 1 || m != nullptr, "network weights need a network");
    require(rounds >= 1 && rounds <= CEM_LGROUP_MAX_ROUNDS, "rounds must be 1..32");
    require(local_substeps >= 1 && local_substeps <= CEM_LGROUP_MAX_LOCAL,
            "local_substeps must be 1..64 (they keep the chain ergodic)");
    require(r->sys->fcc_generated && r->ensemble == CEM_CANONICAL,
            "the learned group sweep supports canonical binary FCC systems of the generated "
            "topology",
            CEM_ERR_UNSUPPORTED);
    const int L = r->reps[0].L[0];
    for (const Replica &R : r->reps)
      require(R.L[0] == L && R.L[1] == L && R.L[2] == L && lgroup_supported(L),
              "the learned group sweep needs equal cubic supercells of 12, 24, 36 or 48 cells",
              CEM_ERR_UNSUPPORTED);
    int dev = 0, maxsm = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    require(lgroup_smem_bytes(L) <= maxsm, "supercell does not fit in shared memory",
            CEM_ERR_UNSUPPORTED);
    r->upload_reps();
    const int n = r->reps[0].n_sites;
    (void)n;
    double *samples = nullptr;
    long long cap = 0;
    if (record_samples) {
      cap = std::max<long long>(1, n_passes - n_equil);
      if (cap > r->lsample_capacity) {
        cudaFree(r->d_lsamples);
        r->d_lsamples = nullptr;
        CUDA_OK(cudaMalloc(&r->d_lsamples, sizeof(double) * 3 * cap * r->n));
        r->lsample_capacity = cap;
      }
      samples = r->d_lsamples;
      cap = r->lsample_capacity;
      r->lsamples_recorded = std::max<long long>(0, n_passes - n_equil);
    }
    int cl = r->group_cluster;
    if (cl == 0) {
      int sms = 0;
      CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      cl = (4 * r->n <= sms) ? 4 : ((2 * r->n <= sms) ? 2 : 1);
    }
    r->last_group_cluster = cl;
    *r->h_stop = 0;
    NvtxRange nvtx("cem_learned_group_run");
    CUDA_OK(cudaEventRecord(r->ev0, r->stream));
    CUDA_OK(lgroup_run(r->sys->T, r->d_reps, r->d_stats, r->d_occ,
                       weights == 1 ? m->d_params : nullptr, weights, rounds, local_substeps, r->n,
                       L, n_passes, n_equil, samples, cap, r->d_stop, cl, r->stream));
    CUDA_OK(cudaEventRecord(r->ev1, r->stream));
    r->stats_valid = false;  // the sweep recomputes its own state next time
  });
}

int cem_learned_samples(cem_replicas *r, int i, double *energy, double *order, int64_t capacity,
                        int64_t *n_samples) {
  return guard([&] {
    check_rep(r, i);
    require(r->d_lsamples != nullptr, "no learned-proposal samples were recorded");
    const int64_t nrec = std::min<int64_t>(r->lsamples_recorded, r->lsample_capacity);
    const int64_t mm = std::min<int64_t>(nrec, capacity);
    std::vector<double> buf((size_t)mm * 3);
    if (mm > 0)
      CUDA_OK(cudaMemcpyAsync(buf.data(), r->d_lsamples + (size_t)i * r->lsample_capacity * 3,
                              sizeof(double) * buf.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_OK(cudaStreamSynchronize(r->stream));
    for (int64_t s = 0; s < mm; ++s) {
      if (energy) energy[s] = buf[s * 3];
      if (order) order[s] = buf[s * 3 + 2];
    }
    if (n_samples) *n_samples = mm;
  });
}

}  // extern "C"
