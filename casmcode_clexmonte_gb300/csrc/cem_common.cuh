// Shared types and device helpers for the GB300 Metropolis hot path.
//
// Arithmetic contract (the oracle restates the same operation order):
//  * delta correlations are integer cluster-count changes per function;
//  * the ECI dot is a float-float sum: W_f = hi_f + lo_f (two floats),
//    each term hi_f * dC_f is split exactly with an FMA, summed with TwoSum
//    (Knuth), errors and lo_f * dC_f accumulated in a second float;
//  * parallel-mode acceptance: u < exp(-beta * dE) with the project's own
//    Cody-Waite exp (below), u a 24-bit uniform from Philox4x32-10;
//  * replay-mode acceptance: the reference's FP64 rule (dE < 0 accepts,
//    else u < exp(-dE * beta) with u from std::uniform_real_distribution
//    over std::mt19937_64).
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define CEM_HD __host__ __device__ __forceinline__
#else
#define CEM_HD inline
#endif

namespace cem {

constexpr int MAX_SUBLAT = 4;
constexpr int MAX_ORBITS = 8;        // orbits held in register accumulators
constexpr int MAX_ORBITS_ALL = 128;  // non-empty orbits of a system (more than
                                     // MAX_ORBITS: one orbit at a time)
constexpr int MAX_FUNCS = 128;
constexpr int MAX_PARTNERS = 3;  // clusters of up to 4 sites
constexpr int MAX_NB = 16;       // nearest-neighbour displacements per sublattice
constexpr int MAX_COLOURS = 8;   // per axis
constexpr int MAX_L = 128;       // per axis
constexpr int MAX_FP = 256;      // distinct flower partners per sublattice

// Cluster-expansion tables in device memory (built once per system).
struct CeTables {
  int n_sublat, n_occ, n_sf, n_funcs, n_orbits;
  int orb_func_base[MAX_ORBITS_ALL];
  int orb_n_funcs[MAX_ORBITS_ALL];
  int orb_size[MAX_ORBITS_ALL];
  // flower clusters, grouped by centre sublattice then orbit:
  // clusters of (b, g) are [fl_begin[b][g], fl_begin[b][g+1])
  int fl_begin[MAX_SUBLAT][MAX_ORBITS_ALL + 1];
  int n_fl;
  // owned clusters (each periodic cluster counted once), same grouping
  int ow_begin[MAX_SUBLAT][MAX_ORBITS_ALL + 1];
  int n_ow;
  int reach;  // max |cell offset component| over flower partners
  // neighbour displacements per sublattice (canonical local swaps)
  int n_nb[MAX_SUBLAT];
  int nb_b[MAX_SUBLAT][MAX_NB];
  int nb_du[MAX_SUBLAT][MAX_NB][3];
  // device arrays
  const int *cl_pb;      // [n_cl * 3] partner sublattice
  const int *cl_du;      // [n_cl * 9] partner cell offsets
  const int *cl_lut;     // [n_cl] offset into lut (general path)
  const uint8_t *lut;    // local function index per decoration code
  const float *w_hi;     // [n_funcs]
  const float *w_lo;     // [n_funcs]
  const double *w;       // [n_funcs]; w[0] = ECI of the empty cluster
  // binary systems (one function per orbit): w[orbit function] = wq * wq_scale
  // + wr, wq integer, wq_scale a power of two chosen so that sum_g wq * dC
  // stays below 2^24 in magnitude; zero for padding orbits and other systems
  int wq[MAX_ORBITS];
  float wr[MAX_ORBITS];
  float wq_scale;
  // the same split for every orbit (binary systems of any size), device arrays
  const int *wq_all;    // [n_orbits]
  const float *wr_all;  // [n_orbits]
  // distinct partner sites of each sublattice's flower clusters (the sites
  // whose energy changes see a change of the centre): (sublattice, du[3])
  int n_fp[MAX_SUBLAT];
  const int *fp;  // [n_sublat][MAX_FP][4]
  // owned clusters use index n_fl + i in the cl_* arrays
};

// floor(x / n) for n > 0 (one division only for |x| beyond one period).
CEM_HD int floor_div(int x, int n) {
  if (x >= 0) return x < n ? 0 : x / n;
  return x >= -n ? -1 : -((n - 1 - x) / n);
}

// Unit cells of a supercell in lower-triangular Hermite normal form: the
// superlattice is generated by the columns (L0, t10, t20), (0, L1, t21) and
// (0, 0, L2) in prim cell coordinates (0 <= t10 < L1, 0 <= t20, t21 < L2).
// Cell (i, j, k) with 0 <= i < L0, 0 <= j < L1, 0 <= k < L2 has index
// i + L0 (j + L1 k); any integer cell reduces along i first (shifting j and k
// by the first column), then along j (shifting k), then along k. Diagonal
// supercells have t = 0 and reduce axis by axis.
struct Cells {
  int L0, L1, L2, t10, t20, t21;
  CEM_HD int index(int i, int j, int k) const {
    int q = floor_div(i, L0);
    i -= q * L0;
    j -= q * t10;
    k -= q * t20;
    q = floor_div(j, L1);
    j -= q * L1;
    k -= q * t21;
    k -= floor_div(k, L2) * L2;
    return i + L0 * (j + L1 * k);
  }
};

// Per-replica description (device memory array).
struct Replica {
  int L[3];
  int tw[3];  // Hermite normal form below the diagonal: t10, t20, t21 (0 if diagonal)
  int n_sites;
  int ensemble;           // 0 = semi-grand canonical flips, 1 = canonical swaps
  int64_t occ_offset;     // into the packed occupation buffer
  double beta;            // 1/(kB T), +inf at T == 0
  float beta_f;
  double temperature;
  double mu[3];           // param_chem_pot (semi-grand canonical)
  double dmu[16];         // [o_i * n_occ + o_f]: mu . R^T (e_f - e_i)
  float dmu_hi[16], dmu_lo[16];
  uint64_t seed;
  // colouring: per axis block size >= p, colour of each coordinate
  int n_col[3];
  int p;
  CEM_HD Cells cells() const { return Cells{L[0], L[1], L[2], tw[0], tw[1], tw[2]}; }
};

// Per-replica running results (device memory array).
struct ReplicaStats {
  double energy;          // running formation energy per supercell
  double n_samples;
  double sum_e, sum_e2;   // potential energy per unit cell moments
  double sum_x[3], sum_xx[9], sum_ex[3];
  double sum_f;           // formation energy per unit cell
  int64_t n_species[8];   // current species counts
  int64_t n_sub[4];       // binary FCC: occupant-1 counts on the 4 simple-cubic sublattices
  int64_t n_proposed, n_accepted;
  int64_t pass;
  int status;             // nonzero: device-side error code
  int pad;
};

// ------------------------------------------------------------------ Philox
// Philox4x32-10, Salmon et al., SC'11 ("Parallel random numbers: as easy as
// 1, 2, 3"), round function and Weyl key schedule from the paper.
struct U4 {
  uint32_t x, y, z, w;
};

CEM_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// 24-bit uniform in [0, 1)
CEM_HD float u24(uint32_t r) { return (float)(r >> 8) * 5.9604644775390625e-8f; }

// ------------------------------------------------------- exact float ops
#ifdef __CUDA_ARCH__
#define FADD(a, b) __fadd_rn((a), (b))
#define FSUB(a, b) __fsub_rn((a), (b))
#define FMUL(a, b) __fmul_rn((a), (b))
#define FFMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define FADD(a, b) ((float)((a) + (b)))
#define FSUB(a, b) ((float)((a) - (b)))
#define FMUL(a, b) ((float)((a) * (b)))
#define FFMA(a, b, c) std::fmaf((a), (b), (c))
#endif

// Float-float accumulator for sum_f W_f * dC_f.
struct FF {
  float s, e;
};

CEM_HD void ff_add_term(FF &acc, float hi, float lo, int dc) {
  float c = (float)dc;
  float p = FMUL(hi, c);
  float pe = FFMA(hi, c, -p);  // exact error of the product
  float t = FADD(acc.s, p);     // TwoSum(acc.s, p)
  float z = FSUB(t, acc.s);
  float err = FADD(FSUB(acc.s, FSUB(t, z)), FSUB(p, z));
  acc.s = t;
  acc.e = FADD(acc.e, FADD(err, pe));
  acc.e = FFMA(lo, c, acc.e);
}

CEM_HD void ff_add_ff(FF &acc, float hi, float lo) {
  float t = FADD(acc.s, hi);
  float z = FSUB(t, acc.s);
  float err = FADD(FSUB(acc.s, FSUB(t, z)), FSUB(hi, z));
  acc.s = t;
  acc.e = FADD(acc.e, FADD(err, lo));
}

// ------------------------------------------------------------------ exp
// exp(x) for x <= 0 by Cody-Waite range reduction (Cody & Waite, "Software
// Manual for the Elementary Functions", 1980): x = n ln2 + r, |r| <= ln2/2,
// ln2 split in a short high part and a low part, e^r by its degree-7 Taylor
// polynomial (truncation < 3e-9 relative), scaled by 2^n through the exponent
// bits. Results below 2^-126 flush to 0.
CEM_HD float cem_expf_neg(float x) {
  if (!(x > -87.0f)) return 0.0f;  // also maps NaN to 0
  const float log2e = 1.44269504088896341f;
  const float ln2_hi = 0.693145751953125f;      // 0x3F317200: few mantissa bits
  const float ln2_lo = 1.42860682030941723e-6f;  // ln2 - ln2_hi
  float n = FMUL(x, log2e);
#ifdef __CUDA_ARCH__
  n = rintf(n);
#else
  n = std::nearbyint(n);
#endif
  float r = FFMA(-n, ln2_hi, x);
  r = FFMA(-n, ln2_lo, r);
  float p = 1.0f / 5040.0f;
  p = FFMA(p, r, 1.0f / 720.0f);
  p = FFMA(p, r, 1.0f / 120.0f);
  p = FFMA(p, r, 1.0f / 24.0f);
  p = FFMA(p, r, 1.0f / 6.0f);
  p = FFMA(p, r, 0.5f);
  p = FFMA(p, r, 1.0f);
  p = FFMA(p, r, 1.0f);
  int e = (int)n + 127;
  if (e <= 0) return 0.0f;
  uint32_t bits = (uint32_t)e << 23;
  float scale;
#ifdef __CUDA_ARCH__
  scale = __uint_as_float(bits);
#else
  __builtin_memcpy(&scale, &bits, 4);
#endif
  return FMUL(p, scale);
}

// exp(x) for x <= 0 in FP64, for n-fold rates: Cody-Waite reduction
// x = n ln2 + r with the fdlibm split of ln2 (ln2_hi has 32 significant bits,
// so n ln2_hi is exact), e^r by its degree-13 Taylor polynomial with fused
// multiply-adds as 1 + (r + r^2 T(r)), T in Estrin's scheme (|r| <= ln2/2:
// truncation below 2^-56 relative; within 1 ulp of libm), scaled by 2^n. Every operation is explicitly rounded, so host
// and device give the same bits. x < -745 (or NaN) returns 0.
#ifdef __CUDA_ARCH__
#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))
#define DFMA(a, b, c) __fma_rn((a), (b), (c))
#else
#define DADD(a, b) ((double)((a) + (b)))
#define DSUB(a, b) ((double)((a) - (b)))
#define DMUL(a, b) ((double)((a) * (b)))
#define DDIV(a, b) ((double)((a) / (b)))
#define DFMA(a, b, c) std::fma((a), (b), (c))
#endif

CEM_HD double cem_exp_neg(double x) {
  if (!(x >= -745.0)) return 0.0;
  if (x > 0.0) x = 0.0;
  const double log2e = 0x1.71547652b82fep+0;
  const double ln2_hi = 0x1.62e42fee00000p-1;
  const double ln2_lo = 0x1.a39ef35793c76p-33;
#ifdef __CUDA_ARCH__
  const double n = rint(DMUL(x, log2e));
#else
  const double n = std::nearbyint(DMUL(x, log2e));
#endif
  double r = DFMA(-n, ln2_hi, x);
  r = DFMA(-n, ln2_lo, r);
  const double c[14] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                        0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                        0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                        0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                        0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};  // 1/k!
  // p = 1 + (r + r^2 T(r)), T = c2 + c3 r + ... + c13 r^11 in Estrin's
  // scheme: 6 dependent steps instead of 13, the large low-order terms added
  // last
  const double r2 = DMUL(r, r), r4 = DMUL(r2, r2);
  const double a0 = DFMA(c[3], r, c[2]), a1 = DFMA(c[5], r, c[4]), a2 = DFMA(c[7], r, c[6]),
               a3 = DFMA(c[9], r, c[8]), a4 = DFMA(c[11], r, c[10]), a5 = DFMA(c[13], r, c[12]);
  const double b0 = DFMA(a1, r2, a0), b1 = DFMA(a3, r2, a2), b2 = DFMA(a5, r2, a4);
  const double t = DFMA(DFMA(b2, r4, b1), r4, b0);
  const double p = DADD(DFMA(r2, t, r), c[0]);
#ifdef __CUDA_ARCH__
  return ldexp(p, (int)n);
#else
  return std::ldexp(p, (int)n);
#endif
}

// Uniform double in [0, 1) with 53 random bits from two Philox words.
CEM_HD double u53(uint32_t a, uint32_t b) {
  return DMUL(DADD(DMUL((double)(a >> 5), 67108864.0), (double)(b >> 6)),
              0x1.0p-53);
}

// ------------------------------------------------------------ MT19937-64
// Matsumoto & Nishimura 64-bit Mersenne Twister (parameters of
// std::mt19937_64), warp-parallel twist in shared memory.
constexpr int MT_N = 312, MT_M = 156;
constexpr uint64_t MT_A = 0xB5026F5AA96619E9ull;
constexpr uint64_t MT_UM = 0xFFFFFFFF80000000ull, MT_LM = 0x7FFFFFFFull;

CEM_HD uint64_t mt_temper(uint64_t x) {
  x ^= (x >> 29) & 0x5555555555555555ull;
  x ^= (x << 17) & 0x71D67FFFEDA60000ull;
  x ^= (x << 37) & 0xFFF7EEE000000000ull;
  x ^= (x >> 43);
  return x;
}

CEM_HD uint64_t mt_next_word(uint64_t cur, uint64_t nxt, uint64_t far) {
  uint64_t y = (cur & MT_UM) | (nxt & MT_LM);
  return far ^ (y >> 1) ^ ((y & 1ull) ? MT_A : 0ull);
}

}  // namespace cem
