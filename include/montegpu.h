/*
 * montegpu.h -- C-ABI of the GB300 lattice Metropolis library (libmontegpu.so).
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every function returns an
 * int status (MG_OK = 0); on failure mg_last_error() returns a message in the style of
 * the reference's std::runtime_error texts ("Error in ...").  No function throws across
 * the ABI.  Caller-owned buffers are copied; the library owns its handles.  A handle
 * must not be used from two host threads at once (the reference's own event
 * proposal helpers are non-reentrant too: function-local statics in
 * include/casm/monte/events/OccEventProposal.hh:127,279).
 *
 * Which reference interface each group replaces (paths within libcasm-monte):
 *   - RandomNumberEngine / RandomNumberGenerator:
 *       include/casm/monte/RandomNumberGenerator.hh:15-42, definitions.hh:17,
 *       python/src/monte.cpp:469-545 (seed, seed_seq, dump, load, random_int, random_real)
 *   - Ising serial replay: the main loop of
 *       include/casm/monte/methods/basic_occupation_metropolis.hh:354-425 as driven by
 *       include/casm/monte/ising_cpp/basic_semigrand_canonical.hh:416-470 (run), with the
 *       model of include/casm/monte/ising_cpp/model.hh:164-436
 *   - CE batch: the semi-grand canonical potential slot
 *       (basic_semigrand_canonical.hh:104-199, occ_delta_per_supercell) filled by a
 *       cluster-expansion formation energy, and the per-step loop of
 *       include/casm/monte/methods/occupation_metropolis.hh:114-150, run as coloured sweeps
 *   - statistics: src/casm/monte/checks/EquilibrationCheck.cc:50-162,
 *       src/casm/monte/BasicStatistics.cc:24-188, include/casm/monte/misc/math.hh:62-72
 */
#ifndef MONTEGPU_H
#define MONTEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_OK 0
#define MG_ERR_INVALID 1 /* invalid argument (reference: std::runtime_error) */
#define MG_ERR_CUDA 2    /* CUDA runtime error */
#define MG_ERR_DEVICE 4  /* a kernel reported an error status */
#define MG_ERR_FULL 5    /* admission refused: no free slot or arena space */

/* ---- library ---- */
const char* mg_last_error(void); /* thread-local message of the last failure */
int mg_version(void);            /* 100 * major + minor */
int mg_device_count(int* n);
int mg_device_sm_count(int* n);
/* free the device blocks that destroyed chain batches left in the library's cache (a batch
 * created later for a shape seen before reuses such a block instead of allocating; at most
 * 8 blocks and 1 GiB are kept per process) */
int mg_release_cached_memory(void);

/* ---- mt19937_64 engine (RandomNumberEngine; monte.cpp:469-513) ---- */
typedef struct mg_engine mg_engine;
/* seed_from_device != 0: seed from std::random_device (RandomNumberGenerator.hh:20-28) */
int mg_engine_create(int seed_from_device, mg_engine** out);
int mg_engine_destroy(mg_engine* e);
int mg_engine_seed(mg_engine* e, uint64_t value);
int mg_engine_seed_seq(mg_engine* e, const uint64_t* values, size_t n);
/* state as text in the std::mersenne_twister_engine stream format */
int mg_engine_dump(const mg_engine* e, char* buf, size_t len);
int mg_engine_load(mg_engine* e, const char* state);
/* RandomNumberGenerator::random_int (uniform_int_distribution, [0, max]) */
int mg_engine_random_int(mg_engine* e, uint64_t max, uint64_t* out);
/* RandomNumberGenerator::random_real (uniform_real_distribution, [0, max)) */
int mg_engine_random_real(mg_engine* e, double max, double* out);

/* ---- 2-D Ising semi-grand canonical serial replay (bit-exact with the reference) ----
 * n_chains independent chains of rows x cols sites (column-major, l = rows*j + i,
 * values +1/-1); per chain J, temperature [K], exchange potential mu and an mt19937_64
 * engine state (text).  use_nlist selects which reference formation-energy summation
 * (model.hh:259-290) the samples reproduce. */
typedef struct mg_ising_replay mg_ising_replay;
int mg_ising_replay_create(int rows, int cols, int n_chains, int use_nlist, const double* J,
                           const double* temperature, const double* mu, const int32_t* occ,
                           const char* const* engine_states, mg_ising_replay** out);
/* Run n_passes passes (each rows*cols steps).  After every pass whose running count is a
 * multiple of sample_period one sample is written per chain:
 * samples_out[chain][max_samples][2 + rows + cols] = {sum s, sum over bonds s_a s_b,
 * row dot products (rows), column dot products (cols)} (dots only when use_nlist == 0). */
int mg_ising_replay_run(mg_ising_replay* h, int n_passes, int sample_period,
                        long long* samples_out, int max_samples, int* n_samples_out);
/* occupation [n_chains][N], engine states (buffers of state_len bytes each), counters */
int mg_ising_replay_get_state(mg_ising_replay* h, int32_t* occ, char** engine_states,
                              size_t state_len, unsigned long long* n_accept,
                              unsigned long long* n_reject);
int mg_ising_replay_last_kernel_ms(mg_ising_replay* h, float* ms);
int mg_ising_replay_destroy(mg_ising_replay* h);

/* ---- FCC cluster expansion: model and coloured-sweep chain batch ----
 * basis_kind 0: binary occupation basis (species A,B); 1: ternary Chebyshev basis (A,B,C).
 * eci[n_classes]: one ECI per symmetrised cluster function in the library's class order
 * (empty, point, pairs 1-4NN, triplets, NN tetrahedron; decorated classes for ternary). */
typedef struct mg_ce_model mg_ce_model;
int mg_ce_model_create(int basis_kind, const double* eci, int n_eci, mg_ce_model** out);
int mg_ce_model_info(const mg_ce_model* m, int* n_classes, int* n_features, int* n_species);
/* per-class multiplicity (clusters per primitive cell) and scale prod(a_b) */
int mg_ce_model_classes(const mg_ce_model* m, long* multiplicity, double* scale);
int mg_ce_model_destroy(mg_ce_model* m);

typedef struct mg_ce_batch mg_ce_batch;
/* n_chains chains of an L0 x L1 x L2 primitive-cell supercell (l = i + L0*(j + L1*k)),
 * occ[n_chains][N] occupant indices, temperature[n_chains] (K),
 * mu[n_chains][n_species-1] exchange potentials conjugate to x_i = n(species i+1)/N,
 * seeds[n_chains] (Philox keys), chain_ids (Philox counter word, NULL = 0..n-1).
 * precision 0: FP64 acceptance decisions; 1: FP32 decisions (disagreements counted).
 * ctas_per_chain 0 = choose automatically; above 16 (more than one cluster holds) the
 * ternary word layout is swept by that many CTAs per chain on the whole grid (layout 4). */
int mg_ce_batch_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                       const double* temperature, const double* mu, const uint64_t* seeds,
                       const uint32_t* chain_ids, const int8_t* occ, int precision,
                       int ctas_per_chain, mg_ce_batch** out);
/* launch geometry: CTAs per chain, colours, threads per CTA, dynamic shared bytes */
int mg_ce_batch_info(const mg_ce_batch* b, int* ctas_per_chain, int* n_colors, int* threads,
                     size_t* smem_bytes);
int mg_ce_batch_colors(const mg_ce_batch* b, int32_t* color /* [N] */);
/* Shared-memory layout of the sweep: 0 = one site per byte (any basis and shape);
 * 1 = four sites per 32-bit word (either basis, L0 = 4Q with Q >= 4, colour(i+Q) =
 * colour(i); the ternary basis sums its energies from byte-parallel monomial counts);
 * 2 = layout 1 with the feature sums split around the phase barrier (binary basis; the
 * colourings generated for it: L0 a multiple of 16, L1/L2 multiples of 16/8); 3 = layout 2
 * with warp-specialised CTAs (one role prepares the next colour while the other decides the
 * current one; at most 384 words per CTA and colour); 4 = layout 1 of the ternary basis
 * swept by ctas_per_chain CTAs per chain on the whole grid (one cooperative launch, each
 * chain's word window in global memory, a grid barrier per chain between colours; default
 * CTA count: the resident CTAs shared between the chains; chosen by itself for ternary chains
 * whose word window does not fit a 16-CTA cluster or would give a CTA more than 1024 words of
 * one colour).  The grid sweep expects the device to itself while it runs: if other work
 * holds SMs long enough for a barrier wait to run out (over a second), the run is abandoned
 * with MG_ERR_DEVICE and the occupations are left as they were.  The best one that applies is
 * chosen automatically.  All give identical trajectories; set_layout rebuilds the site
 * lists (MG_ERR_INVALID where the layout does not apply). */
int mg_ce_batch_layout(const mg_ce_batch* b, int* layout);
/* The sweep's colouring of an L0 x L1 x L2 supercell (host only, no device needed):
 * writes color[N], returns the number of colours (or -status); word_layout (may be
 * NULL) receives 0, 1 or 2 (a batch of this shape uses that layout, or layout 3 where its
 * CTA split allows). */
int mg_ce_color_supercell(int basis_kind, int L0, int L1, int L2, int32_t* color, int* word_layout);
int mg_ce_batch_set_layout(mg_ce_batch* b, int layout);
/* Autotuner: times probe_passes passes of every layout that applies at every CTA count it
 * accepts, and the occupancy choice with rotation over two cluster sizes where the batch
 * has a rotation plan (runs of at least 4 n_chains passes, compared per pass), on the
 * batch's own chains, whose occupations and pass counters are restored after each trial, so
 * results do not change; keeps the fastest.  Reports the chosen layout, CTA count (the slow
 * slot's when rotating: mg_ce_batch_rotation tells) and milliseconds per pass (each may be
 * NULL). */
int mg_ce_batch_autotune(mg_ce_batch* b, int probe_passes, int* layout, int* ctas_per_chain, float* ms_per_pass);
/* Run n_passes passes.  out (host, may be NULL) receives [n_passes][n_chains][n_classes+2]
 * int64: slot 0 accepted proposals, slot f (1..n_classes-1) change of the integer
 * correlation sum of class f, slot n_classes proposals re-decided in FP64, slot
 * n_classes+1 FP32 decisions that differ from FP64. */
int mg_ce_batch_run(mg_ce_batch* b, int n_passes, long long* out);
/* device time of the sweep kernel(s) of the last run, from CUDA events on the batch's
 * stream */
int mg_ce_batch_last_kernel_ms(const mg_ce_batch* b, float* ms);
/* Rotation over two cluster sizes (layout 3 with the CTA count chosen by occupancy; no
 * counterpart in the reference, whose loop runs one chain on one host thread).  When
 * n_chains - 1 chains fit on the GPU at once on clusters of ctas_fast > ctas_per_chain CTAs
 * but n_chains do not, a run of at least 2 n_chains passes lets the chains take turns on one
 * cluster of ctas_per_chain CTAs (the slow slot) while the others sweep on clusters of
 * ctas_fast CTAs: chain c sweeps a_c passes fast, g passes in the slow slot (chains in
 * order) and the rest fast, with a_c and g set from the measured time ratio so that the slow
 * slot stays busy and every chain gets the run's passes.  A run rotates only when the
 * simulated rotated schedule (with the launch fixed cost measured by earlier rotated runs)
 * ends before one unrotated launch of the same passes; short runs stay unrotated.  Outputs
 * and occupations are identical to unrotated runs.  ctas_fast receives 0 when the batch does
 * not rotate; ratio the measured time per pass on ctas_fast CTAs over that on ctas_per_chain
 * CTAs.  set_rotation(b, mode): 0 turns it off for the batch, 1 re-plans it (the default),
 * 2 rotates every run of at least 2 n_chains passes even where it does not pay (to test
 * the rotated schedule).
 * last_launches: sweep kernels launched by the last run (1 unless it rotated). */
int mg_ce_batch_rotation(const mg_ce_batch* b, int* ctas_fast, double* ratio);
int mg_ce_batch_set_rotation(mg_ce_batch* b, int allowed);
int mg_ce_batch_last_launches(const mg_ce_batch* b, int* launches);
/* After a rotated run: ms[n_chains][6] = milliseconds from the run's start to each chain's
 * first fast sweep start and end, slow-slot sweep start and end, second fast sweep start and
 * end (a sweep of no passes starts and ends together). */
int mg_ce_batch_rotation_timeline(const mg_ce_batch* b, float* ms);

/* ---- FCC cluster expansion: canonical (fixed-composition) sweep ----
 * Replaces the canonical swap of include/casm/monte/events/OccEventProposal.hh:108-237
 * (propose_canonical_event) accepted by methods/metropolis.hh:26-35 inside the loop of
 * methods/occupation_metropolis.hh:114-150.  n_chains chains of an L0 x L1 x L2 supercell,
 * one CTA per chain (the supercell with a 2-site border must fit in one CTA's shared
 * memory: up to 56^3).  A pass proposes, colour by colour, a perfect matching of each colour
 * class (positions k and (d - k) mod n, d random per phase) and exchanges the occupants of
 * each pair by Metropolis; passes alternate between two colourings whose classes connect
 * every site, so atoms reach any site.  Composition is conserved exactly.  Same occupant,
 * temperature, seed, chain-id and precision conventions as mg_ce_batch_create; run's out has
 * the batch's layout with slot 0 = accepted swaps. */
typedef struct mg_ce_canon mg_ce_canon;
int mg_ce_canon_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                       const double* temperature, const uint64_t* seeds, const uint32_t* chain_ids,
                       const int8_t* occ, int precision, mg_ce_canon** out);
/* colours of the two colourings, threads per CTA, dynamic shared bytes */
int mg_ce_canon_info(const mg_ce_canon* h, int* n_colors_a, int* n_colors_b, int* threads,
                     size_t* smem_bytes);
/* colouring `which` (0: passes with even index, 1: odd) as color[N] */
int mg_ce_canon_colors(const mg_ce_canon* h, int which, int32_t* color);
/* the order of colouring `which`'s per-colour site lists (site_order[N], colour by colour):
 * the matching of a phase pairs positions k and (d - k) mod n of its colour's list */
int mg_ce_canon_class_order(const mg_ce_canon* h, int which, int32_t* site_order);
int mg_ce_canon_run(mg_ce_canon* h, int n_passes, long long* out);
int mg_ce_canon_last_kernel_ms(const mg_ce_canon* h, float* ms);
int mg_ce_canon_get_occ(mg_ce_canon* h, int8_t* occ);
/* integer correlation sums [n_chains][n_classes] from a full recompute */
int mg_ce_canon_corr(mg_ce_canon* h, long long* corr);
int mg_ce_canon_destroy(mg_ce_canon* h);

/* ---- FCC cluster expansion (binary basis): rejection-free (N-fold way) dynamics ----
 * An event selector for the loop of include/casm/monte/methods/nfold.hh:48-149 (which takes
 * the selector from the caller) run on the GPU for semi-grand canonical single-site flips:
 * rate of flipping site l = min(1, exp(-beta dE_l)), an event chosen with probability
 * rate / R, the residence time -ln(u) / R.  One CTA per chain (at most 32768 sites: the
 * rates and their sums live in shared memory; four chains share an SM up to 8192 sites).  A pass is N events; out receives per pass
 * and chain [2 + n_classes] doubles: the pass's time, the total rate at its end, and the
 * time-weighted sums of the integer correlation sums (time averages are these over the
 * time).  Same conventions as mg_ce_batch_create otherwise. */
typedef struct mg_ce_nfold mg_ce_nfold;
int mg_ce_nfold_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                       const double* temperature, const double* mu, const uint64_t* seeds,
                       const uint32_t* chain_ids, const int8_t* occ, mg_ce_nfold** out);
int mg_ce_nfold_run(mg_ce_nfold* h, int n_passes, double* out);
/* threads per chain, chains resident per SM (4 for supercells of at most 8192 sites, else 1),
 * dynamic shared bytes per chain */
int mg_ce_nfold_info(const mg_ce_nfold* h, int* threads, int* chains_per_sm, size_t* smem_bytes);
int mg_ce_nfold_last_kernel_ms(const mg_ce_nfold* h, float* ms);
int mg_ce_nfold_get_occ(mg_ce_nfold* h, int8_t* occ);
/* integer correlation sums [n_chains][n_classes]: tracked (recompute 0) or recomputed */
int mg_ce_nfold_corr(mg_ce_nfold* h, int recompute, long long* corr);
int mg_ce_nfold_destroy(mg_ce_nfold* h);
int mg_ce_batch_get_occ(mg_ce_batch* b, int8_t* occ);
int mg_ce_batch_set_occ(mg_ce_batch* b, const int8_t* occ);
/* full recompute of the integer correlation sums [n_chains][n_classes] */
int mg_ce_batch_corr(mg_ce_batch* b, long long* out);
/* per-proposal FP64 dE (formation + semi-grand canonical term) on the current state */
int mg_ce_batch_delta_e(mg_ce_batch* b, const int32_t* chain, const long long* sites,
                        const int8_t* new_occ, long long n, double* out);
int mg_ce_batch_destroy(mg_ce_batch* b);
/* how many chains of this supercell can sweep concurrently with ctas_per_chain CTAs each
 * (cudaOccupancyMaxActiveClusters on the sweep kernel); used by the autotuner */
int mg_ce_max_active_chains(const mg_ce_model* m, int L0, int L1, int L2, int ctas_per_chain,
                            int* n_chains);

/* ---- chain pool: many chains of any supercell shape, persistent kernel ----
 * The batched form of the reference's per-chain run (one `run` call per thermodynamic
 * state, basic_semigrand_canonical.hh:416-470): an HBM arena of arena_bytes holds the
 * occupations; chains are admitted while their occupation fits (MG_ERR_FULL otherwise)
 * and removed when done.  mg_ce_pool_run sweeps the given slots by n_passes each in one
 * launch of a persistent kernel (one CTA per chain, work queue largest first); every
 * chain keeps its own pass counter, so results do not depend on how runs are batched.
 * out (host, may be NULL): [n][n_passes][n_classes+2] in the order of `slots`, same slot
 * meaning as mg_ce_batch_run. */
typedef struct mg_ce_pool mg_ce_pool;
int mg_ce_pool_create(const mg_ce_model* m, long long arena_bytes, int max_chains, int precision,
                      mg_ce_pool** out);
int mg_ce_pool_add(mg_ce_pool* p, int L0, int L1, int L2, double temperature, const double* mu,
                   uint64_t seed, uint32_t chain_id, const int8_t* occ, int* slot);
/* admission of n chains in one call: dims [n][3], temperature [n], mu [n][n_species-1],
 * seeds [n], chain_ids [n], occ the n occupations back to back; slots [n] out.  Every
 * chain is checked first, then all are admitted or none (MG_ERR_FULL / MG_ERR_INVALID
 * leave the pool as it was); the same chains one mg_ce_pool_add each give the same slots
 * and trajectories.  The host-to-device copies are merged where the chains' arena spaces
 * are contiguous, with one stream synchronisation for the call. */
int mg_ce_pool_add_many(mg_ce_pool* p, int n, const int32_t* dims, const double* temperature,
                        const double* mu, const uint64_t* seeds, const uint32_t* chain_ids,
                        const int8_t* occ, int32_t* slots);
int mg_ce_pool_remove(mg_ce_pool* p, int slot);
/* build (and cache) the colouring and site lists of a supercell shape ahead of its first
 * chain; a geometry depends only on the shape, so servers prepare the shapes they expect */
int mg_ce_pool_prepare(mg_ce_pool* p, int L0, int L1, int L2);
int mg_ce_pool_info(const mg_ce_pool* p, long long* arena_free_bytes, long long* arena_bytes,
                    int* n_used, int* max_chains);
int mg_ce_pool_run(mg_ce_pool* p, const int32_t* slots, int n, int n_passes, long long* out);
int mg_ce_pool_last_kernel_ms(const mg_ce_pool* p, float* ms);
/* kernels the last mg_ce_pool_run launched (one per CTA class and layout with chains, plus
 * the series kernel when series are on) */
int mg_ce_pool_last_launches(const mg_ce_pool* p, int* n);
int mg_ce_pool_get_occ(mg_ce_pool* p, int slot, int8_t* occ);
/* colouring of the slot's supercell [N]; returns the number of colours (>0) or an error */
int mg_ce_pool_colors(const mg_ce_pool* p, int slot, int32_t* color);
int mg_ce_pool_corr(mg_ce_pool* p, int slot, long long* out);
/* Device-resident samples: after every pass each chain appends its potential energy per
 * site (E_f - mu . N x)/N to a series of up to max_samples values (call before adding
 * chains).  mg_ce_pool_check runs the reference's equilibration + convergence rule on one
 * component (EquilibrationCheck.cc:50-117 with the absolute precision, then
 * BasicStatisticsCalculator on the equilibrated tail, ConvergenceCheck.hh:74-90) on the
 * device for each slot: out[n][6] = {equilibrated, N_equilibration, N_statistics, mean,
 * calculated_precision, converged}. */
int mg_ce_pool_enable_series(mg_ce_pool* p, int max_samples);
int mg_ce_pool_series(mg_ce_pool* p, int slot, double* out, int max_n, int* n_samples);
int mg_ce_pool_check(mg_ce_pool* p, const int32_t* slots, int n, double abs_precision, double confidence,
                     double* out);
int mg_ce_pool_destroy(mg_ce_pool* p);

/* ---- serial replay of the reference's semi-grand canonical dynamics (cluster expansion) ----
 * Replaces, for an FCC cluster expansion on one asymmetric unit, the loop of
 * methods/occupation_metropolis.hh:114-150 with propose_semigrand_canonical_event
 * (events/OccEventProposal.hh:260-336), OccLocation::choose_mol / apply
 * (events/OccLocation.hh:257-261, OccLocation.cc:216-283) and metropolis_acceptance
 * (methods/metropolis.hh:26-35), consuming each chain's std::mt19937_64 exactly as the
 * reference's RandomNumberGenerator does (RandomNumberGenerator.hh:32-41): one warp per
 * chain, N = L0 L1 L2 steps per pass.  engine_states: the engines' text form (312 words and
 * the position, as operator<< writes it).  occ[n_chains][N] occupant indices; mu
 * [n_chains][n_species-1].  mg_ce_replay_run: out (optional) [n_passes][n_chains]
 * [n_classes+2] = {accepted steps of the pass, change of each integer correlation sum
 * (classes 1..n_classes-1), rejected steps of the pass, 0}.  mg_ce_replay_candidates: the
 * occupant lists (OccLocation::m_loc, one candidate per species) in list order, species by
 * species, with their sizes.  At most 200000 sites. */
typedef struct mg_ce_replay mg_ce_replay;
int mg_ce_replay_create(const mg_ce_model* m, int L0, int L1, int L2, int n_chains, const double* temperature,
                        const double* mu, const int8_t* occ, const char* const* engine_states,
                        mg_ce_replay** out);
int mg_ce_replay_run(mg_ce_replay* h, int n_passes, long long* out);
int mg_ce_replay_get_occ(mg_ce_replay* h, int8_t* occ);
int mg_ce_replay_engine_state(mg_ce_replay* h, int chain, char* buf, int buf_len);
int mg_ce_replay_candidates(mg_ce_replay* h, int chain, int32_t* sizes, int32_t* sites);
int mg_ce_replay_counts(mg_ce_replay* h, unsigned long long* n_accept, unsigned long long* n_reject);
int mg_ce_replay_last_kernel_ms(const mg_ce_replay* h, float* ms);
int mg_ce_replay_destroy(mg_ce_replay* h);

/* ---- allocation-free coloured sweep (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc (an embedding framework owns all device
 * memory, allocation is forbidden during a run, or the device is fully reserved): the
 * caller passes device pointers to the occupations d_occ[n_chains][N] (in/out; every code
 * in [0, n_species)) and the per-pass outputs d_out[n_passes][n_chains][n_classes+2]
 * (same meaning as mg_ce_batch_run), plus host arrays of temperatures, exchange
 * potentials and seeds.  The site lists, chain parameters and an occupant-check counter
 * go to a fixed file-scope device array of MG_NOALLOC_SCRATCH_BYTES, resident on every
 * device that loads the library until exit; no device memory is allocated after the
 * first call on a device (the colouring and site-list helpers use some host heap).
 * Sizes beyond MG_NOALLOC_MAX_SITES sites per chain or MG_NOALLOC_MAX_CHAINS chains are
 * rejected.  Occupant codes are checked on the device first; the call waits for that
 * check (it synchronises `stream`) and returns MG_ERR_INVALID, sweeping nothing, when a
 * code is out of range.  The sweep itself runs the byte-layout kernel (one site per byte),
 * the slowest layout of the batch API.  The first call on a device looks up the array's
 * address (do it before any stream capture).  Calls share the array: calls that overlap
 * on the GPU race, and host calls must not run concurrently.  The sweep is enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) after the check and not
 * synchronised; pass0 continues the Philox pass counter. */
#define MG_NOALLOC_MAX_SITES 262144
#define MG_NOALLOC_MAX_CHAINS 64
#define MG_NOALLOC_SCRATCH_BYTES 2162688
int mg_ce_sweep_noalloc(const mg_ce_model* m, int L0, int L1, int L2, int n_chains,
                        const double* temperature, const double* mu, const uint64_t* seeds,
                        int8_t* d_occ, long long pass0, int n_passes, long long* d_out,
                        int precision, void* stream);

/* ---- statistics (host numerics shared with the device convergence kernel) ---- */
/* _default_equilibration_check (EquilibrationCheck.cc:50-117) */
int mg_equilibration_check(const double* obs, long n, double prec, int* is_equilibrated,
                           long* n_samples_for_equilibration);
/* BasicStatisticsCalculator (BasicStatistics.cc:114-188); nw = 0 for unweighted */
int mg_basic_statistics(const double* obs, long n, const double* w, long nw, double confidence,
                        long method, long n_resamples, double* mean,
                        double* calculated_precision);
int mg_autocorrelation_factor(const double* obs, long n, double increment, double* out);
double mg_approx_erf_inv(double x);

#ifdef __cplusplus
}
#endif

#endif /* MONTEGPU_H */
