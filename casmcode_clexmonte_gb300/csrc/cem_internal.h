// Internal launch interface between the C ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cuda_bf16.h>

#include "cem_common.cuh"

namespace cem {

constexpr int SWEEP_THREADS = 512;
// pitches of the generated evaluator: L + 4 for L = 10, 24, 32, 48 (a warp's
// class rows fall on distinct shared-memory banks), and 64 for the rest
constexpr int SWEEP_PITCHES[5] = {14, 28, 36, 52, 64};

struct ReplayParams {
  int L[3];
  int tw[3];                   // Hermite normal form below the diagonal (0: diagonal)
  int n_sites;
  int ensemble;
  double beta;
  double dmu[16];
  unsigned long long mt_seed;
  long long n_steps;
  int8_t *occ;                 // device, updated in place
  unsigned char *accept_seq;   // device, optional
  double *de_seq;              // device, optional
  long long *site_seq;         // device, optional (2 per step)
  long long *result;           // device [3]: n_accept, draws, stopped
};

struct SweepParams {
  const Replica *reps;
  ReplicaStats *stats;
  int8_t *occ;                 // packed occupations of all replicas
  double *samples;             // [n_rep][capacity][width] or null
  long long sample_capacity;
  int sample_width;
  long long n_passes, n_equil;
  int max_classes;
  int max_sub;  // sub-steps per pass (sweeps x colour classes): sizes the schedule
  int n_pair_sweeps, n_local_sweeps;  // canonical pass composition
  int init;                    // binary systems: compute the exact initial stats in-kernel
  int pack16;                  // cooperative sweep: 16-bit partner offsets and weights
  const int *cta_rep;          // replica of each CTA (null: CTA i runs replica i)
  const volatile int *stop;    // host-mapped stop flag (null: none)
  int cluster;                 // CTAs per replica (thread-block cluster; <= 1: one CTA)
  double RT[16];               // (n_occ-1) x n_occ
};

cudaError_t launch_energy(const CeTables &T, const int8_t *occ, const Cells &C,
                          unsigned long long *counts, cudaStream_t st);
cudaError_t launch_delta(const CeTables &T, const int8_t *occ, const Cells &C, int n_events, int k_sites, const long long *sites, const int *new_occ,
                         const double *dmu, double *dE, long long *dcount, cudaStream_t st);
int replay_smem_bytes(int n_sites, int n_occ);
cudaError_t launch_replay(const CeTables &T, const ReplayParams &P, cudaStream_t st);
// Greedy composition enforcement, one warp per replica; scratch holds
// (n_occ + 1) ints per site; out[3 r + {0,1,2}] = flips, draws, status.
cudaError_t launch_enforce(int n_occ, const Replica *reps, int n_reps, int8_t *occ,
                           const double *target, unsigned long long seed, int n_sublat,
                           int *scratch, long long *out, long long max_flips, cudaStream_t st);
cudaError_t launch_init_stats(const CeTables &T, const Replica *reps, ReplicaStats *stats,
                              const int8_t *occ, int n_replicas, int max_sites, cudaStream_t st);
cudaError_t smem_bandwidth(double *gbs, cudaStream_t st);
int sweep_smem_bytes(const CeTables &T, int L0, int L1, int L2, int n_sub, int pitch);
// pitch 0: run-time tables; otherwise the generated binary FCC evaluator with
// that x/y pitch (one of SWEEP_PITCHES)
cudaError_t launch_sweep(const CeTables &T, const SweepParams &P, int n_replicas, int smem,
                         int pitch, int threads, cudaStream_t st);
// true if the system is the binary FCC topology of the generated evaluator
bool matches_generated_fcc(const CeTables &T, const int *pb, const int *du);

// HBM-streamed sweep (cem_stream.cu)
struct StreamRun {       // device-resident run parameters, written per run
  long long n_equil;
  long long start_pass;  // pass counter at the start of the run
  double *samples;
  long long sample_capacity;
  int sample_width;
  int pad;
};
struct StreamState {
  int8_t *halo = nullptr;        // [n_rep][halo bytes]
  long long *acc = nullptr;      // [n_rep][16]
  StreamRun *run = nullptr;      // device
  int2 *sched = nullptr;         // [n_rep][n_sub] schedule of the current pass
  int sched_cap = 0;             // entries allocated per replica
  cudaGraphExec_t exec = nullptr;
  int key = -1;
};
long long stream_halo_bytes(int L2, int pitch);
cudaError_t stream_run(const CeTables &T, StreamState &st, const Replica *reps, ReplicaStats *stats,
                       int8_t *occ_all, int n_rep, int L2, int pitch, int n_classes, int n_pair_sw,
                       int n_local_sw, const double *RT, long long n_passes, long long n_equil,
                       long long start_pass, double *samples, long long capacity, int width,
                       int count_sub, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1,
                       const volatile int *stop_host, long long *launched);

// learned proposal (cem_learned.cu)
struct TreeGeo;
cudaError_t mlp_forward(const __nv_bfloat16 *params, const int8_t *X, long long n, float *z,
                        cudaStream_t st);
cudaError_t mlp_grad(const __nv_bfloat16 *params, const int8_t *X, const float *t,
                     const int *order, long long b0, long long n, float *grad, double *loss,
                     cudaStream_t st);
cudaError_t mlp_adam(float *master, __nv_bfloat16 *params, float *grad, float *m, float *v,
                     float lr, int step, cudaStream_t st);
cudaError_t mlp_pack(const float *master, __nv_bfloat16 *params, cudaStream_t st);
cudaError_t learned_features(const int8_t *occ, int L, const double *w, const int *orb_func,
                             double beta, int8_t *X, float *t, cudaStream_t st);
int learned_tree_size(int n_sites);
int learned_smem_bytes(int L, int pitch);
cudaError_t learned_run(const CeTables &T, const Replica *reps, ReplicaStats *stats,
                        int8_t *occ, const __nv_bfloat16 *params, int use_mlp, long long *weights,
                        long long w_stride, unsigned long long *trees, long long tree_stride,
                        int n_sites, int n_replicas, int L, long long n_passes, long long n_equil,
                        double *samples, long long capacity, int pitch, cudaStream_t st);

// learned group sweep (cem_lgroup.cu)
cudaError_t mlp_forward_tc(const __nv_bfloat16 *params, const int8_t *X, long long n, float *z,
                           int *status, cudaStream_t st);
bool lgroup_supported(int L);
int lgroup_smem_bytes(int L);
cudaError_t lgroup_run(const CeTables &T, const Replica *reps, ReplicaStats *stats, int8_t *occ,
                       const __nv_bfloat16 *params, int mode, int rounds, int n_local,
                       int n_replicas, int L, long long n_passes, long long n_equil,
                       double *samples, long long capacity, const volatile int *stop,
                       int cluster, cudaStream_t st);

// n-fold way (cem_nfold.cu)
// 32-ary sum tree over n leaves: level 0 = leaves, level k + 1 has
// ceil(n_k / 32) nodes, the last level one node; levels stored back to back.
struct RateTree {
  int n_lev;
  long long off[8], n[8];
};
__host__ __device__ inline void rate_tree_geo(long long n_leaves, RateTree &g) {
  g.n_lev = 1;
  g.off[0] = 0;
  g.n[0] = n_leaves;
  while (g.n[g.n_lev - 1] > 1 && g.n_lev < 8) {
    const int k = g.n_lev;
    g.off[k] = g.off[k - 1] + g.n[k - 1];
    g.n[k] = (g.n[k - 1] + 31) / 32;
    g.n_lev = k + 1;
  }
}
__host__ __device__ inline long long rate_tree_size(long long n_leaves) {
  RateTree g;
  rate_tree_geo(n_leaves, g);
  return g.off[g.n_lev - 1] + 1;
}
struct NfoldParams {
  const Replica *reps;
  ReplicaStats *stats;
  int8_t *occ;
  double *tree;               // per replica trees, back to back (tree_smem == 0)
  const long long *tree_off;  // [n_rep] offset of each replica's tree
  int tree_smem;              // 1: each CTA keeps its replica's tree in shared memory
  long long n_events, n_equil;
  long long rec_cap;          // recorded events per replica (0: none)
  long long *rec_site;
  int *rec_occ;
  double *rec_dt;
  double RT[16];
};
int nfold_smem_bytes(const CeTables &T, int L0, int L1, int L2, int pitch, int tree_smem);
cudaError_t launch_nfold(const CeTables &T, const NfoldParams &P, int n_replicas, int smem,
                         int pitch, cudaStream_t st);

}  // namespace cem
