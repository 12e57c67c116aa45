/*
 * cem.h - C ABI of the GB300 cluster-expansion Metropolis hot path.
 *
 * The library replaces, behind a plain C ABI (no exceptions, no C++ or torch
 * types), the per-event potential change and the Metropolis loop of
 * libcasm-clexmonte's canonical and semi-grand canonical calculators:
 *
 *   occ_delta_per_supercell  BaseMonteCalculator.hh:41-43 (BaseMontePotential),
 *                            CanonicalCalculator.cc:137-140,
 *                            SemiGrandCanonicalCalculator.cc:186-213
 *   per_supercell            BaseMonteCalculator.hh:33, CanonicalCalculator.cc:127-129
 *   run                      BaseMonteCalculator.hh:223-225,
 *                            CanonicalCalculator.cc:413-462,
 *                            SemiGrandCanonicalCalculator.cc:423-466
 *   occupation_metropolis_v2 include/casm/clexmonte/methods/occupation_metropolis.hh:72-123
 *
 * (paths relative to the CASMcode_clexmonte source tree). Every function
 * returns CEM_OK or an error code; cem_last_error() gives the message of the
 * last failure on the calling thread. Objects are not thread-safe: one host
 * thread drives one cem_replicas at a time, as the reference's calculators
 * are single-threaded (CanonicalCalculator.cc:413-462).
 */
#ifndef CEM_GB300_H
#define CEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CEM_OK 0
#define CEM_ERR_INVALID 1     /* bad argument or inconsistent input */
#define CEM_ERR_CUDA 2        /* CUDA runtime error (message says which) */
#define CEM_ERR_UNSUPPORTED 3 /* valid input outside the library's limits */
#define CEM_ERR_DEVICE 4      /* a kernel reported an error status */
#define CEM_STOPPED 5         /* cem_synchronize: the run was stopped early by
                                 cem_request_stop (not an error: the state is
                                 consistent at a pass boundary) */

#define CEM_SEMIGRAND_CANONICAL 0
#define CEM_CANONICAL 1

typedef struct cem_system cem_system;
typedef struct cem_replicas cem_replicas;

/* Cluster-expansion tables (built by the host-side system builder).
 * Occupation basis: site function k of occupant o is [o == k+1]; occupant 0
 * is the reference species. Function 0 is the empty cluster. Energies:
 * E = weights[0]*n_unitcells + sum_{f>=1} weights[f]*count_f, with count_f
 * the number of clusters whose decoration is in class f and
 * weights[f] = eci_f * coeff_f / mult_f. */
typedef struct cem_system_desc {
  int n_sublat;               /* sublattices with an occupation degree of
                                 freedom per unit cell, 1..4 (single-occupant
                                 sublattices are left out) */
  int n_occ;                  /* occupants per site, 2 or 3 */
  int n_funcs;                /* functions including the empty function, <= 128 */
  int n_orbits;               /* non-empty orbits, 1..128, in function order
                                 (more than 8: the sweep, the n-fold way, the
                                 delta and replay kernels walk the tables one
                                 orbit at a time; the HBM-streamed mode and the
                                 learned proposal need the generated binary FCC
                                 topology) */
  const int *orbit_size;      /* [n_orbits] sites per cluster, 1..4 */
  const int *orbit_func_begin;/* [n_orbits] first function index */
  const int *orbit_n_funcs;   /* [n_orbits] number of functions */
  const double *weights;      /* [n_funcs] */
  /* flower: every cluster containing site (b, cell 0), grouped by b, then
   * by orbit; partner j of cluster c is site (partner_sublat[3c+j],
   * cell partner_du[9c+3j .. 9c+3j+2]); -1 marks an unused slot. */
  int n_flower;
  const int *flower_sublat;
  const int *flower_orbit;
  const int *flower_partner_sublat;
  const int *flower_partner_du;
  /* [n_flower * lut_stride] global function index of the decoration
   * code sum_j (occ_j - 1) * (n_occ-1)^j (j = 0: centre, j >= 1: partners),
   * -1 if none; lut_stride = (n_occ-1)^4 */
  const int16_t *flower_lut;
  /* owned clusters: each periodic cluster listed once, at its anchor site */
  int n_owned;
  const int *owned_sublat;
  const int *owned_orbit;
  const int *owned_partner_sublat;
  const int *owned_partner_du;
  const int16_t *owned_lut;
  /* canonical local-swap displacements, per sublattice: site (b, x) swaps
     with (neighbour_sublat, x + neighbour_du). They must connect every site
     (graph over the sublattices connected, cycle translations generating
     Z^3), else canonical batches are refused: swaps inside a colour class
     only permute that class. The Python builder takes the partners of the
     shortest pair orbits until this holds. */
  const int *n_neighbour;       /* [n_sublat], each <= 16 */
  const int *neighbour_sublat;  /* [n_sublat*16] */
  const int *neighbour_du;      /* [n_sublat*16*3] */
  /* R^T = dparam_dmol ((n_occ-1) x n_occ, row-major): change of parametric
   * composition per change of species counts
   * (SemiGrandCanonicalCalculator.cc:144) */
  const double *param_RT;
} cem_system_desc;

/* Run statistics of one replica (moments over the sampled passes). */
typedef struct cem_stats {
  double n_samples;
  double mean_potential;   /* <potential energy per unit cell> */
  double var_potential;    /* population variance of the same */
  double mean_formation;   /* <formation energy per unit cell> */
  double mean_comp[3];     /* <param composition> */
  double cov_comp[9];      /* cov(param composition) */
  double cov_e_comp[3];    /* cov(potential, param composition) */
  double energy;           /* current formation energy per supercell (running) */
  int64_t n_proposed;      /* proposals with a real occupation change */
  int64_t n_accepted;
  int64_t passes;
} cem_stats;

/* Last error message of the calling thread. */
const char *cem_last_error(void);

/* Device of the calling thread: name, SM count, compute capability. */
int cem_device_info(char *name, int name_len, int *sm_count, int *cc_major, int *cc_minor);

/* System tables -> device. Replaces the System / Clexulator set-up
 * (System.cc:633-640 get_clex, StateData.cc:64-79). */
int cem_system_create(const cem_system_desc *desc, cem_system **out);
int cem_system_destroy(cem_system *sys);

/* A batch of replicas (independent Monte Carlo states) of diagonal
 * supercells L[3r..3r+2] of the system, one ensemble for the batch
 * (CEM_CANONICAL or CEM_SEMIGRAND_CANONICAL). Occupations live in HBM.
 * Replaces state construction + set_state_and_potential
 * (CanonicalCalculator.cc:377-399). Linear site index:
 * l = b*n_uc + i + L0*(j + L1*k): sublattice-major as in
 * canonical_metropolis_test.cpp:34-36, unit cells i fastest. */
int cem_replicas_create(const cem_system *sys, int n_replicas, const int *L, int ensemble,
                        cem_replicas **out);
/* The same for general supercells: T[9r..9r+8] is replica r's integer
 * transformation_matrix_to_super, row-major, columns = the supercell lattice
 * vectors in prim cell coordinates (Configuration.hh:29-50). Unit cells are
 * indexed on the matrix's lower-triangular Hermite normal form H (same
 * superlattice): cell (i, j, k), 0 <= i < H00, 0 <= j < H11, 0 <= k < H22,
 * has index i + H00*(j + H11*k); for a diagonal matrix with positive entries
 * this is the order of cem_replicas_create. Non-diagonal supercells support
 * energies, energy changes, the sequential replay, the n-fold way,
 * composition enforcement, state transfer and semi-grand canonical parallel
 * sweeps (when a colouring exists; run-time tables, shared memory);
 * canonical parallel runs, the learned proposals and streamed batches return
 * CEM_ERR_UNSUPPORTED for them.
 * A non-diagonal supercell in which some cluster holds two periodic images
 * of one site is refused. */
int cem_replicas_create_supercells(const cem_system *sys, int n_replicas, const int64_t *T,
                                   int ensemble, cem_replicas **out);
/* The lower-triangular Hermite normal form H (row-major) that
 * cem_replicas_create_supercells indexes the supercell T on (no device
 * needed). */
int cem_supercell_hnf(const int64_t *T, int64_t *H);
int cem_replicas_destroy(cem_replicas *r);
int cem_n_sites(const cem_replicas *r, int replica, int64_t *n_sites);

/* Conditions: temperature (K) and param_chem_pot ([n_occ-1], SGC only; may be
 * NULL for canonical). beta = 1/(kB T), infinite at T == 0
 * (Conditions.hh:17-45). */
int cem_set_conditions(cem_replicas *r, int replica, double temperature,
                       const double *param_chem_pot);
/* Seed of the replica's counter-based random stream (parallel mode). */
int cem_set_seed(cem_replicas *r, int replica, uint64_t seed);

/* Host <-> device occupations (int8 occupant indices, n_sites). */
int cem_set_occupation(cem_replicas *r, int replica, const int8_t *occ);
int cem_get_occupation(cem_replicas *r, int replica, int8_t *occ);

/* Packed host <-> device occupations of all replicas, concatenated in
 * replica order (sum of n_sites bytes). */
int cem_set_occupation_all(cem_replicas *r, const int8_t *packed);
int cem_get_occupation_all(cem_replicas *r, int8_t *packed);

/* Page-locked host buffers for the transfers above. */
int cem_host_alloc(int64_t bytes, void **ptr);
int cem_host_free(void *ptr);

/* Formation energy per supercell of the current occupation, with the integer
 * function counts (count[0] = n_unitcells). Replaces per_supercell()
 * (CanonicalCalculator.cc:127-129). */
int cem_energy(cem_replicas *r, int replica, double *energy, int64_t *counts);

/* Potential change of n_events events, each a series of sites_per_event
 * occupation changes applied in order (sequential semantics,
 * canonical/canonical.hh:42-45). potential = 0: formation energy only
 * (CanonicalPotential); 1: semi-grand potential
 * dE - param_chem_pot . R^T dN (SemiGrandCanonicalPotential). dcount, if not
 * NULL, receives the integer delta correlations [n_events * n_funcs].
 * Replaces occ_delta_per_supercell (BaseMonteCalculator.hh:41-43). */
int cem_delta_energy(cem_replicas *r, int replica, int n_events, int sites_per_event,
                     const int64_t *sites, const int32_t *new_occ, int potential,
                     double *dE, int64_t *dcount);

/* Same result as cem_delta_energy, without allocating device memory. This
 * entry point has no counterpart in the reference. It is for callers that
 * cannot allocate on the device: a host program whose device memory belongs
 * to another framework's pool, or a per-event Monte Carlo loop that cannot
 * afford the device-wide synchronisation cudaMalloc and cudaFree imply.
 * Events and results are staged in one fixed array in device memory that is
 * part of the library (CEM_NOALLOC_SCRATCH_BYTES = 4 423 808 bytes, about
 * 4.4 MB, held by every device that loads the library until the process
 * exits). At most CEM_NOALLOC_MAX_EVENTS events of at most
 * CEM_NOALLOC_MAX_SITES sites per call; larger calls return
 * CEM_ERR_UNSUPPORTED. The batch's device must be current (CEM_ERR_INVALID
 * otherwise). The first call on a device looks up the array's device address
 * for that device, so make that first call before any stream capture. All
 * calls share the array and it keeps the last call's contents; calls that
 * overlap on the GPU (from different streams or batches at the same time)
 * race. */
#define CEM_NOALLOC_MAX_EVENTS 4096
#define CEM_NOALLOC_MAX_SITES 4
#define CEM_NOALLOC_SCRATCH_BYTES 4423808
int cem_delta_energy_noalloc(cem_replicas *r, int replica, int n_events, int sites_per_event,
                             const int64_t *sites, const int32_t *new_occ, int potential,
                             double *dE, int64_t *dcount);

/* Sequential replay: n_steps steps of occupation_metropolis_v2
 * (occupation_metropolis.hh:92-120) on one replica, consuming the
 * std::mt19937_64 stream seeded with mt_seed exactly as the reference's
 * RandomNumberGenerator does (uniform_int_distribution<long> /
 * uniform_real_distribution<double>), with the event proposal, occupant
 * location update and acceptance restated from libcasm-monte. Optional
 * outputs per step: accept flag, dE, proposed sites (2 per step, -1 unused).
 * Updates the replica's occupation on the device. */
int cem_replay(cem_replicas *r, int replica, uint64_t mt_seed, int64_t n_steps,
               uint8_t *accept_seq, double *dE_seq, int64_t *site_seq, int64_t *n_accept,
               uint64_t *n_draws);

/* n-fold way (rejection-free semi-grand canonical Monte Carlo, Bortz-Kalos-
 * Lebowitz): each replica draws n_equil + n_events events, an event being a
 * single-site occupant change drawn with probability proportional to its
 * Metropolis rate (1 if dE <= 0, else exp(-beta dE), dE the semi-grand
 * canonical potential change), and applies it. After the n_equil first
 * events, the state before each event enters the statistics with weight
 * n_possible / (sum of rates), its expected residence time in Metropolis
 * trials (n_possible = sites x n_occ x (n_occ - 1)); cem_get_stats then
 * returns time-weighted moments (n_samples = total weight). Optional records
 * per replica (record_capacity per replica, replica-major): changed site,
 * new occupant and weight of each of the first events. Replaces
 * clexmonte::nfold::Nfold::run (include/casm/clexmonte/nfold/nfold_impl.hh:20-108)
 * and CompleteEventCalculator::calculate_rate
 * (src/casm/clexmonte/nfold/nfold_events.cc:24-60). Semi-grand canonical
 * batches only; CEM_ERR_DEVICE when a replica has no event of non-zero rate. */
int cem_nfold_run(cem_replicas *r, int64_t n_events, int64_t n_equil, int64_t record_capacity,
                  int64_t *rec_site, int32_t *rec_occ, double *rec_dt);

/* Composition enforcement: greedy semi-grand canonical flips that move each
 * replica toward target_mol (n_occ values per replica, replica-major:
 * species count per unit cell, e.g. {1 - x, x} for a one-site binary cell)
 * until no flip type brings it closer; replica i draws from
 * std::mt19937_64(mt_seed + i) exactly as the reference's
 * RandomNumberGenerator does. Replaces clexmonte::enforce_composition
 * (include/casm/clexmonte/state/enforce_composition.hh:172-210; python
 * binding python/src/clexmonte_functions.cpp:71-140). n_flips (optional,
 * n_replicas values) receives the flips applied per replica. Invalidates the
 * running statistics of every replica. */
int cem_enforce_composition(cem_replicas *r, const double *target_mol, uint64_t mt_seed,
                            int64_t *n_flips);

/* Parallel Metropolis: n_passes passes over every replica; each pass updates
 * colour classes of mutually non-interacting sites at once (flips for SGC,
 * pair swaps for canonical). Passes after n_equil contribute to the
 * statistics; record_samples != 0 keeps per-pass samples for
 * autocorrelation analysis. Replaces run() (CanonicalCalculator.cc:413-462,
 * SemiGrandCanonicalCalculator.cc:423-466). */
int cem_run(cem_replicas *r, int64_t n_passes, int64_t n_equil, int record_samples);

/* Autotuner of the shared-memory sweep's launch schedule: times trial_passes
 * passes with each of {512 threads per replica, 256 threads (two replicas per
 * SM)} x {replica order, largest replicas first}, from the same saved state,
 * then restores the state and keeps the fastest (options "threads" and
 * "cta_order"). The chain does not depend on the schedule (for binary systems
 * bit for bit; ternary running energies may differ in the last bits, their
 * FP64 sums being reduced in another order). No-op for HBM-streamed batches.
 * Replaces no reference function (the reference has no GPU launch
 * schedule). */
int cem_autotune(cem_replicas *r, int64_t trial_passes, double *best_ms);

/* One end-to-end step of a batch as a CUDA graph: copy the packed
 * occupations of all replicas in from host_in, run n_passes passes (the
 * exact initial statistics recomputed on the device), copy the occupations
 * out to host_out. The graph is captured at the first call for these buffers
 * and pass count and replayed afterwards. Host buffers must be page-locked
 * (cem_host_alloc); asynchronous on the batch's stream (cem_synchronize
 * waits). Shared-memory batches only. Replaces no single reference function:
 * it is the batch form of set state -> run -> read state
 * (CanonicalCalculator.cc:413-462). */
int cem_step_async(cem_replicas *r, const int8_t *host_in, int8_t *host_out, int64_t n_passes);

/* Run options of a batch (canonical pass composition and evaluator):
 *   "pair_sweeps"  (default 2): sweeps of swaps between sites of one colour
 *                  class per pass;
 *   "local_sweeps" (default 1, >= 1): sweeps of swaps with a nearest
 *                  neighbour per pass (these move atoms between classes);
 *   "generic_evaluator" (1): use the run-time cluster tables even where the
 *                  generated binary FCC evaluator applies;
 *   "orbit_walk" (1): walk the run-time tables one orbit at a time, the
 *                  kernel that cluster expansions with more than 8 orbits
 *                  (real CASM basis sets) always use; running energy as an
 *                  FP64 sum of accepted changes; 512 threads per replica;
 *   "wide_records" (0 or 1): 1 keeps the cooperative binary sweep's 32-bit
 *                  cluster records where 16-bit ones (partner offsets and
 *                  integer weights packed two per word) would fit; the
 *                  chain is the same, the 16-bit records are faster;
 *   "streamed" (1): keep the occupations in HBM and run one kernel per colour
 *                  sub-step over many CTAs per replica (a captured CUDA graph
 *                  per pass); chosen automatically when a supercell does not
 *                  fit in shared memory (binary FCC, equal even supercells);
 *   "threads" (512 or 256): threads per replica of the shared-memory sweep
 *                  (256: two replicas per SM);
 *   "cta_order" (0 or 1): replica -> CTA schedule (1: largest first);
 *   "group_cluster" (0, 1, 2, 4): CTAs per replica of cem_learned_group_run,
 *                  a thread-block cluster whose CTAs share the replica's
 *                  sub-steps through distributed shared memory (0, the
 *                  default: 4, 2 or 1, the largest that keeps every cluster
 *                  on its own SMs; the chain does not depend on it).
 * cem_get_option also reads "pitch" (> 0 generated evaluator, 0 run-time
 * tables, -1 one orbit at a time), "smem_bytes", "colour_classes" and
 * "streamed". */
int cem_set_option(cem_replicas *r, const char *key, int64_t value);
int cem_get_option(cem_replicas *r, const char *key, int64_t *value);

/* ---- Learned proposal (canonical swaps, binary FCC of the generated topology).
 * A network scores each site's environment (its 42 neighbours in the first
 * three shells, 0/1 occupants) -> 64 -> 64 -> 1 logit z, with bf16 parameters
 * and fp32 accumulation, trained toward -beta dE_AB / 2 (dE_AB: energy change
 * of putting B on the site in that environment). A site holding A has weight
 * w = max(1, round(4096 exp(z))), a site holding B the same of -z, z clamped
 * to [-10, 10]. cem_learned_run: a swap draws one A site and one B site with
 * probability proportional to w from per-species int64 sum trees over the
 * whole replica; acceptance min(1, exp(-beta dE) q_rev / q_fwd) with the exact
 * proposal probabilities, so the canonical distribution is sampled whatever
 * the network predicts. cem_learned_group_run: the same proposal inside
 * groups of non-interacting sites, many swaps in flight per replica.
 * Parameter vector (fp32 masters): W1[42][64] (input-major), b1[64],
 * W2[64][64] (input-major), b2[64], w3[64], b3. No counterpart in the
 * reference (its canonical proposal is uniform, CanonicalCalculator.cc:78-83). */
typedef struct cem_mlp cem_mlp;
int cem_mlp_info(int *n_inputs, int *n_hidden, int *n_params);
int cem_mlp_create(uint64_t seed, cem_mlp **out);
int cem_mlp_destroy(cem_mlp *m);
int cem_mlp_get_params(cem_mlp *m, float *master);
int cem_mlp_set_params(cem_mlp *m, const float *master);
/* logits of n environments (n x 42 int8 occupants) */
int cem_mlp_forward(cem_mlp *m, int64_t n, const int8_t *features, float *logits);
/* the same logits on the 5th-generation tensor cores, the inference path of
 * cem_learned_group_run: tcgen05.mma with bf16 operands in shared memory and
 * fp32 accumulators in tensor memory, 128 environments per warpgroup,
 * layer-1 activations rounded to bf16 as layer 2's operand; CEM_ERR_DEVICE if
 * an MMA wait ran out */
int cem_mlp_forward_tc(cem_mlp *m, int64_t n, const int8_t *features, float *logits);
/* gradient of the mean-squared error 1/(2n) sum (z - t)^2 at the current
 * (bf16) parameters, and the loss */
int cem_mlp_gradient(cem_mlp *m, int64_t n, const int8_t *features, const float *targets,
                     float *grad, double *loss);
/* Adam (Kingma & Ba 2015) on the same loss, minibatches in a seeded order */
int cem_mlp_train(cem_mlp *m, int64_t n, const int8_t *features, const float *targets,
                  int epochs, int batch, float lr, uint64_t seed, double *loss_per_epoch);
/* Environments of every site of a replica (n_sites x 42) and the training
 * target t = clamp(-beta dE_AB / 2, -10, 10) (half the log Metropolis weight
 * of putting B on the site), from the device occupation. */
int cem_learned_features(cem_replicas *r, int replica, int8_t *features, float *targets);
/* n_passes x n_sites proposals per replica with the learned proposal
 * (m == NULL: every weight 1, i.e. the uniform global swap proposal).
 * Samples per pass: energy per unit cell and the L1_2 order parameter
 * sqrt(sum_k (x_k - x)^2) over the four simple-cubic sublattices. */
int cem_learned_run(cem_replicas *r, const cem_mlp *m, int64_t n_passes, int64_t n_equil,
                    int record_samples);
/* Learned group sweep: n_passes passes per replica of a parallel canonical
 * sampler in which the proposal weights choose the swaps. A pass visits the 27
 * colour classes of period 3 (sites whose cell coordinates agree modulo 3: no
 * two share a cluster) in a random order; each class is split into groups of
 * 32 sites by a random permutation drawn per sub-step, and each group runs
 * `rounds` Metropolis-Hastings swaps: one A site drawn with probability
 * w_A / W_A and one B site with w_B / W_B among the group's members, accepted
 * with min(1, exp(-beta dE) q_rev / q_fwd) from the exact integer weights and
 * totals (the members do not interact, so dE is the sum of the two sites'
 * exact flip energies and only the two swapped sites change weight). Then
 * `local_substeps` sub-steps of nearest-neighbour swaps (plain Metropolis)
 * move atoms between classes, which keeps the chain ergodic.
 * weights: 0 every weight 1 (uniform swaps inside groups); 1 the network m
 * (w_A = round(2^12 exp(z)), w_B = round(2^12 exp(-z)) of the site's
 * environment logit z, evaluated once per site and sub-step on the tensor
 * cores, tcgen05); 2 the exact locally balanced weights, z = -beta dE_AB / 2, the
 * quantity the network is trained to predict. rounds 1..CEM_LGROUP_MAX_ROUNDS,
 * local_substeps 1..CEM_LGROUP_MAX_LOCAL. Equal cubic supercells of 12, 24,
 * 36 or 48 cells. Samples per pass as cem_learned_run (cem_learned_samples);
 * statistics as cem_run (cem_get_stats). No counterpart in the reference (its
 * canonical proposal is uniform, CanonicalCalculator.cc:78-83). */
#define CEM_LGROUP_MAX_ROUNDS 32
#define CEM_LGROUP_MAX_LOCAL 64
int cem_learned_group_run(cem_replicas *r, const cem_mlp *m, int weights, int rounds,
                          int local_substeps, int64_t n_passes, int64_t n_equil,
                          int record_samples);
int cem_learned_samples(cem_replicas *r, int replica, double *energy, double *order,
                        int64_t capacity, int64_t *n_samples);

/* Statistics and samples of one replica (after cem_run). */
int cem_get_stats(cem_replicas *r, int replica, cem_stats *out);
int cem_get_samples(cem_replicas *r, int replica, double *potential, double *comp,
                    int64_t capacity, int64_t *n_samples);
int cem_reset_stats(cem_replicas *r);
/* Per-pass L1_2 order parameter sqrt(sum_k (x_k - x)^2) over the four
 * simple-cubic sublattices (binary FCC with the generated evaluator; 0
 * otherwise), from the last cem_run with record_samples. */
int cem_get_order_samples(cem_replicas *r, int replica, double *order, int64_t capacity,
                          int64_t *n_samples);

/* Measured shared-memory read bandwidth of the device, GB/s (all SMs,
 * 16-byte vector loads); the roofline denominator of the shared-memory
 * resident sweep. */
int cem_smem_bandwidth(double *gbs);

/* Checkpoint / restart of one replica: occupation plus an opaque state
 * block (running energy, species and sublattice counts, moments, pass
 * counter; cem_state_bytes bytes). The random streams are counter based
 * (seed, pass, sub-step, site), so restoring the occupation and the state
 * into a batch with the same seed continues the chain bit for bit. The
 * reference restarts whole runs from completed_runs.json and saved final
 * states (canonical_fullrun_test.cpp:337-344); this restarts inside a run. */
int cem_state_bytes(const cem_replicas *r, int64_t *bytes);
int cem_get_state(cem_replicas *r, int replica, int8_t *occ, void *state);
int cem_set_state(cem_replicas *r, int replica, const int8_t *occ, const void *state);

/* Wait for all work of this batch. Returns CEM_STOPPED when a stop was
 * requested (cem_request_stop) during the last run. */
int cem_synchronize(cem_replicas *r);

/* Ask the run in flight (cem_run, cem_learned_group_run) to stop early. The
 * only entry point that may be called from another host thread while a run is
 * in flight: it writes a flag in page-locked host memory mapped into the
 * device. The persistent shared-memory kernels read it once per pass and
 * leave at the next pass boundary, writing back occupations and statistics
 * as a completed run does (cem_get_stats reports the passes actually run);
 * an HBM-streamed run stops queueing its per-pass graphs, so it ends after
 * the passes already queued. Each run clears the flag when it starts. The
 * reference stops long runs from the host through its run manager's
 * completion checks (BaseMonteCalculator.hh:223-225, RunManager); this is
 * the batch form of that control for one long launch. */
int cem_request_stop(cem_replicas *r);

/* Device time of the last cem_run's main kernel, in milliseconds (CUDA
 * events on the batch's stream). */
int cem_last_kernel_ms(cem_replicas *r, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* CEM_GB300_H */
