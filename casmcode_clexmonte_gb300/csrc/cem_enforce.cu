// Composition enforcement: greedy semi-grand canonical flips toward a target
// composition, restating clexmonte::enforce_composition
// (include/casm/clexmonte/state/enforce_composition.hh:56-126, 172-210)
// step for step, with the same draws from std::mt19937_64:
//
//   repeat:
//     for every flip type a -> b (a != b, a-major order) with sites of
//     species a: the composition after one flip, and its Euclidean distance
//     to the target (mol per unit cell); keep the types that improve the
//     distance by more than tol = 1e-3 / n_unitcells, the best ones within
//     tol of each other;
//     none left -> stop;
//     choose one of them with probability proportional to its number of
//     sites (one random_real), then one site of species a uniformly
//     (one random_int over the occupant list) and flip it.
//
// One warp per replica: the lanes build the per-species occupant lists in
// increasing site order (the order OccLocation is initialised in); lane 0
// then runs the sequential loop, with swap-with-last removal and append, as
// OccLocation::apply does. Double arithmetic is spelled with explicitly
// rounded intrinsics so that no multiply-add is contracted; distances are
// then bit-identical to the host's.
#include "cem_kernels.cuh"

namespace cem {

namespace {

template <int NOCC>
__device__ inline double distance(const double *m, const double *t) {
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < NOCC; ++c) {
    const double d = __dsub_rn(m[c], t[c]);
    s = __dadd_rn(s, __dmul_rn(d, d));
  }
  return __dsqrt_rn(s);
}

template <int NOCC>
__global__ void __launch_bounds__(32) k_enforce(const Replica *__restrict__ reps, int8_t *occ_all,
                                                const double *__restrict__ target_all,
                                                unsigned long long seed, int n_sublat,
                                                int *scratch, long long *out,
                                                long long max_flips) {
  __shared__ MtState mt;
  __shared__ int size[NOCC];
  const int r = blockIdx.x, lane = threadIdx.x;
  const int N = reps[r].n_sites;
  const long long off = reps[r].occ_offset;
  int8_t *occ = occ_all + off;
  int *lists = scratch + off * (NOCC + 1);
  int *pos = lists + (long long)NOCC * N;

  // ordered occupant lists: warp-wide ballots per species
  int cnt[NOCC];
#pragma unroll
  for (int s = 0; s < NOCC; ++s) cnt[s] = 0;
  for (int base = 0; base < N; base += 32) {
    const int l = base + lane;
    const int a = l < N ? (int)occ[l] : -1;
#pragma unroll
    for (int s = 0; s < NOCC; ++s) {
      const unsigned m = __ballot_sync(0xffffffffu, a == s);
      if (a == s) {
        const int p = cnt[s] + __popc(m & ((1u << lane) - 1u));
        lists[(long long)s * N + p] = l;
        pos[l] = p;
      }
      cnt[s] += __popc(m);
    }
  }
  __syncwarp();
  if (lane != 0) return;

  int total = 0;
#pragma unroll
  for (int s = 0; s < NOCC; ++s) {
    size[s] = cnt[s];
    total += cnt[s];
  }
  if (total != N) {  // an occupant index outside [0, NOCC)
    out[3 * r + 0] = 0;
    out[3 * r + 1] = 0;
    out[3 * r + 2] = 3;
    return;
  }
  mt.mt[0] = seed + (unsigned long long)r;
  for (int i = 1; i < MT_N; ++i)
    mt.mt[i] = 6364136223846793005ull * (mt.mt[i - 1] ^ (mt.mt[i - 1] >> 62)) + (unsigned long long)i;
  mt.idx = MT_N;
  mt.draws = 0;

  const double volume = (double)(N / n_sublat);
  const double dn = 1.0 / volume;
  const double tol = __dmul_rn(dn, 1e-3);
  double cur[NOCC], tgt[NOCC];
#pragma unroll
  for (int c = 0; c < NOCC; ++c) {
    cur[c] = __ddiv_rn((double)size[c], volume);
    tgt[c] = target_all[(long long)r * NOCC + c];
  }

  constexpr int NT = NOCC * (NOCC - 1);
  long long n_flips = 0;
  int status = 0;
  for (;;) {
    const double orig = distance<NOCC>(cur, tgt);
    double best = orig;
    int n_ch = 0;
    int ch_a[NT], ch_b[NT];
    double ch_m[NT][NOCC];
    for (int a = 0; a < NOCC; ++a) {
      for (int b = 0; b < NOCC; ++b) {
        if (a == b || size[a] == 0) continue;
        double tm[NOCC];
#pragma unroll
        for (int c = 0; c < NOCC; ++c) tm[c] = cur[c];
        tm[a] = __dsub_rn(tm[a], dn);
        tm[b] = __dadd_rn(tm[b], dn);
        const double d = distance<NOCC>(tm, tgt);
        bool push = false;
        if (d > __dsub_rn(orig, tol)) {
          continue;
        } else if (d < __dsub_rn(best, tol)) {
          n_ch = 0;
          push = true;
          best = d;
        } else if (d < __dadd_rn(best, tol)) {
          push = true;
        }
        if (push) {
          ch_a[n_ch] = a;
          ch_b[n_ch] = b;
#pragma unroll
          for (int c = 0; c < NOCC; ++c) ch_m[n_ch][c] = tm[c];
          ++n_ch;
        }
      }
    }
    if (n_ch == 0) break;
    if (n_flips >= max_flips) {
      status = 2;
      break;
    }
    double sum = 0.0;
    for (int k = 0; k < n_ch; ++k) sum = __dadd_rn(sum, (double)size[ch_a[k]]);
    const double u = __dadd_rn(__dmul_rn(std_random_real(mt), sum), 0.0);
    sum = 0.0;
    int pick = -1;
    for (int k = 0; k < n_ch; ++k) {
      sum = __dadd_rn(sum, (double)size[ch_a[k]]);
      if (u < sum) {
        pick = k;
        break;
      }
    }
    if (pick < 0) {
      status = 4;
      break;
    }
#pragma unroll
    for (int c = 0; c < NOCC; ++c) cur[c] = ch_m[pick][c];
    const int a = ch_a[pick], b = ch_b[pick];
    const long long ia = std_random_int(mt, (long long)size[a] - 1);
    const int l = lists[(long long)a * N + ia];
    const int last = lists[(long long)a * N + size[a] - 1];
    lists[(long long)a * N + pos[l]] = last;
    pos[last] = pos[l];
    size[a] -= 1;
    pos[l] = size[b];
    lists[(long long)b * N + size[b]] = l;
    size[b] += 1;
    occ[l] = (int8_t)b;
    ++n_flips;
  }
  out[3 * r + 0] = n_flips;
  out[3 * r + 1] = (long long)mt.draws;
  out[3 * r + 2] = status;
}

template <int NOCC>
cudaError_t launch_enforce_t(const Replica *reps, int n_reps, int8_t *occ, const double *target,
                             unsigned long long seed, int n_sublat, int *scratch, long long *out,
                             long long max_flips, cudaStream_t st) {
  k_enforce<NOCC><<<n_reps, 32, 0, st>>>(reps, occ, target, seed, n_sublat, scratch, out,
                                         max_flips);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_enforce(int n_occ, const Replica *reps, int n_reps, int8_t *occ,
                           const double *target, unsigned long long seed, int n_sublat,
                           int *scratch, long long *out, long long max_flips, cudaStream_t st) {
  if (n_occ == 2)
    return launch_enforce_t<2>(reps, n_reps, occ, target, seed, n_sublat, scratch, out, max_flips, st);
  if (n_occ == 3)
    return launch_enforce_t<3>(reps, n_reps, occ, target, seed, n_sublat, scratch, out, max_flips, st);
  return cudaErrorInvalidValue;
}

}  // namespace cem
