// Run-time dispatch on the number of occupants per site.
#include "cem_kernels.cuh"

namespace cem {

// The launchers are instantiated in the kernel translation units (cem_k2.cu,
// cem_k3.cu, cem_kfcc.cu, cem_kfcc_b.cu); extern declarations keep this file
// from compiling a second copy of every kernel.
#define CEM_EXTERN(N)                                                                          \
  extern template cudaError_t launch_energy_t<N>(const CeTables &, const int8_t *,             \
                                                 const Cells &, unsigned long long *,          \
                                                 cudaStream_t);                                \
  extern template cudaError_t launch_delta_t<N>(const CeTables &, const int8_t *,              \
                                                const Cells &, int, int, const long long *,    \
                                                const int *, const double *, double *,         \
                                                long long *, cudaStream_t);                    \
  extern template cudaError_t launch_replay_t<N>(const CeTables &, const ReplayParams &,       \
                                                 cudaStream_t);                                \
  extern template cudaError_t launch_init_stats_t<N>(const CeTables &, const Replica *,        \
                                                     ReplicaStats *, const int8_t *, int, int, \
                                                     cudaStream_t);                            \
  extern template cudaError_t launch_sweep_t<N, 0, SWEEP_THREADS>(                             \
      const CeTables &, const SweepParams &, int, int, cudaStream_t);
CEM_EXTERN(2)
CEM_EXTERN(3)
#define CEM_EXTERN_PITCH(P)                                                        \
  extern template cudaError_t launch_sweep_t<2, P, SWEEP_THREADS>(const CeTables &, \
                                                                 const SweepParams &, int, int, \
                                                                 cudaStream_t);
CEM_EXTERN_PITCH(14)
CEM_EXTERN_PITCH(28)
CEM_EXTERN_PITCH(36)
CEM_EXTERN_PITCH(52)
CEM_EXTERN_PITCH(64)
// 256-thread variants (two replicas per SM), cem_k256a.cu / cem_k256b.cu
#define CEM_EXTERN_256(N, P)                                                                 \
  extern template cudaError_t launch_sweep_t<N, P, 256>(const CeTables &, const SweepParams &, \
                                                        int, int, cudaStream_t);
CEM_EXTERN_256(2, 14)
CEM_EXTERN_256(2, 28)
CEM_EXTERN_256(2, 36)
CEM_EXTERN_256(2, 52)
CEM_EXTERN_256(2, 64)
CEM_EXTERN_256(2, 0)
CEM_EXTERN_256(3, 0)
// one orbit at a time (cem_kbig.cu)
extern template cudaError_t launch_sweep_t<2, -1, SWEEP_THREADS>(const CeTables &,
                                                                 const SweepParams &, int, int,
                                                                 cudaStream_t);
extern template cudaError_t launch_sweep_t<3, -1, SWEEP_THREADS>(const CeTables &,
                                                                 const SweepParams &, int, int,
                                                                 cudaStream_t);
extern template cudaError_t launch_sweep_t<2, -2, SWEEP_THREADS>(const CeTables &,
                                                                 const SweepParams &, int, int,
                                                                 cudaStream_t);

cudaError_t launch_energy(const CeTables &T, const int8_t *occ, const Cells &C,
                          unsigned long long *counts, cudaStream_t st) {
  if (T.n_occ == 2) return launch_energy_t<2>(T, occ, C, counts, st);
  if (T.n_occ == 3) return launch_energy_t<3>(T, occ, C, counts, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_delta(const CeTables &T, const int8_t *occ, const Cells &C, int n_events,
                         int k_sites, const long long *sites, const int *new_occ,
                         const double *dmu, double *dE, long long *dcount, cudaStream_t st) {
  if (T.n_occ == 2)
    return launch_delta_t<2>(T, occ, C, n_events, k_sites, sites, new_occ, dmu, dE, dcount, st);
  if (T.n_occ == 3)
    return launch_delta_t<3>(T, occ, C, n_events, k_sites, sites, new_occ, dmu, dE, dcount, st);
  return cudaErrorInvalidValue;
}

int replay_smem_bytes(int n_sites, int n_occ) { return replay_smem_bytes_impl(n_sites, n_occ); }

cudaError_t launch_replay(const CeTables &T, const ReplayParams &P, cudaStream_t st) {
  if (T.n_occ == 2) return launch_replay_t<2>(T, P, st);
  if (T.n_occ == 3) return launch_replay_t<3>(T, P, st);
  return cudaErrorInvalidValue;
}

int sweep_smem_bytes(const CeTables &T, int L0, int L1, int L2, int n_sub, int pitch) {
  return sweep_smem_bytes_impl(T, L0, L1, L2, n_sub, pitch);
}

template <int TH>
static cudaError_t launch_sweep_th(const CeTables &T, const SweepParams &P, int n_replicas,
                                   int smem, int pitch, cudaStream_t st) {
  if (pitch == 14) return launch_sweep_t<2, 14, TH>(T, P, n_replicas, smem, st);
  if (pitch == 28) return launch_sweep_t<2, 28, TH>(T, P, n_replicas, smem, st);
  if (pitch == 36) return launch_sweep_t<2, 36, TH>(T, P, n_replicas, smem, st);
  if (pitch == 52) return launch_sweep_t<2, 52, TH>(T, P, n_replicas, smem, st);
  if (pitch == 64) return launch_sweep_t<2, 64, TH>(T, P, n_replicas, smem, st);
  if (pitch != 0) return cudaErrorInvalidValue;
  if (T.n_occ == 2) return launch_sweep_t<2, 0, TH>(T, P, n_replicas, smem, st);
  if (T.n_occ == 3) return launch_sweep_t<3, 0, TH>(T, P, n_replicas, smem, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep(const CeTables &T, const SweepParams &P, int n_replicas, int smem,
                         int pitch, int threads, cudaStream_t st) {
  if (pitch == -2) {  // binary, one warp per site change, 512 threads
    if (threads != SWEEP_THREADS || T.n_occ != 2) return cudaErrorInvalidValue;
    return launch_sweep_t<2, -2, SWEEP_THREADS>(T, P, n_replicas, smem, st);
  }
  if (pitch == -1) {  // one orbit at a time, 512 threads
    if (threads != SWEEP_THREADS) return cudaErrorInvalidValue;
    if (T.n_occ == 2) return launch_sweep_t<2, -1, SWEEP_THREADS>(T, P, n_replicas, smem, st);
    if (T.n_occ == 3) return launch_sweep_t<3, -1, SWEEP_THREADS>(T, P, n_replicas, smem, st);
    return cudaErrorInvalidValue;
  }
  if (threads == SWEEP_THREADS) return launch_sweep_th<SWEEP_THREADS>(T, P, n_replicas, smem, pitch, st);
  if (threads == 256) return launch_sweep_th<256>(T, P, n_replicas, smem, pitch, st);
  return cudaErrorInvalidValue;
}

bool matches_generated_fcc(const CeTables &T, const int *pb, const int *du) {
  if (T.n_sublat != 1 || T.n_occ != 2 || T.n_orbits != gen_fcc::N_ORBITS) return false;
  if (T.reach != 2) return false;
  for (int g = 0; g < T.n_orbits; ++g) {
    if (T.orb_size[g] != gen_fcc::ORBIT_SIZE[g]) return false;
    if (T.fl_begin[0][g + 1] - T.fl_begin[0][g] != gen_fcc::ORBIT_CLUSTERS[g]) return false;
  }
  if (T.n_fl != gen_fcc::N_CL) return false;
  for (int c = 0; c < T.n_fl; ++c)
    for (int q = 0; q < 3; ++q) {
      const int k = gen_fcc::CL_P[c][q];
      if ((k < 0) != (pb[c * 3 + q] < 0)) return false;
      if (k < 0) continue;
      if (pb[c * 3 + q] != 0) return false;
      for (int a = 0; a < 3; ++a)
        if (du[c * 9 + q * 3 + a] != gen_fcc::NB[k][a]) return false;
    }
  return true;
}

cudaError_t launch_init_stats(const CeTables &T, const Replica *reps, ReplicaStats *stats,
                              const int8_t *occ, int n_replicas, int max_sites, cudaStream_t st) {
  if (T.n_occ == 2) return launch_init_stats_t<2>(T, reps, stats, occ, n_replicas, max_sites, st);
  if (T.n_occ == 3) return launch_init_stats_t<3>(T, reps, stats, occ, n_replicas, max_sites, st);
  return cudaErrorInvalidValue;
}

// Shared-memory read bandwidth probe: every thread streams 16-byte vector
// loads over a 64 KB shared buffer; one CTA per SM slot.
__global__ void k_smem_probe(int iters, unsigned long long *sink) {
  extern __shared__ __align__(16) uint4 buf[];
  const int n = 65536 / 16;
  for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = make_uint4(i, i + 1, i + 2, i + 3);
  __syncthreads();
  uint32_t acc = 0;
  int idx = threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll 8
    for (int k = 0; k < 8; ++k) {
      const uint4 v = buf[(idx + k * blockDim.x) & (n - 1)];
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    idx = (idx + 8 * blockDim.x) & (n - 1);
  }
  if (acc == 0x12345678u) sink[blockIdx.x] = acc;
}

// Shared-memory read bandwidth (GB/s) over all SMs, from CUDA events.
cudaError_t smem_bandwidth(double *gbs, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int smem = 65536, threads = 1024, iters = 4096, blocks = sms * 2;
  e = cudaFuncSetAttribute(k_smem_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  unsigned long long *sink = nullptr;
  e = cudaMalloc(&sink, sizeof(unsigned long long) * blocks);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_smem_probe<<<blocks, threads, smem, st>>>(64, sink);  // warm-up
  cudaEventRecord(a, st);
  k_smem_probe<<<blocks, threads, smem, st>>>(iters, sink);
  cudaEventRecord(b, st);
  e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  const double bytes = (double)blocks * threads * iters * 8.0 * 16.0;
  *gbs = bytes / (ms * 1e-3) / 1e9;
  return cudaGetLastError();
}

}  // namespace cem
