/*
 * paising.h -- C ABI of the GB300 population-annealing engine (2D +-J=1
 * ferromagnetic Ising model, periodic L x L lattice, no field).
 *
 * The reference (LevBarash/PAising) is two CUDA programs without a library
 * interface: its drop-in surface is the command line and the results file
 * (PAisingSSC.cu:367-404 flags, 670-692 output; PAisingMSC.cu:532-569,
 * 820-842).  The handle API below carries exactly those parameters and rows;
 * the stage entry points replace the reference's kernels one by one and are
 * what the parity tests call.
 *
 * Conventions: every function returns a pa_status (0 = success); no
 * exception or process exit crosses the boundary (the reference aborts with
 * exit() on any CUDA error, PAisingSSC.cu:80-88).  The library owns the
 * device memory of a handle; the caller owns every host buffer it passes.
 * Stage entry points take device pointers and a cudaStream_t passed as
 * void* (NULL = the legacy default stream) and synchronise that stream
 * before returning.  A handle is not thread-safe.
 */
#ifndef PAISING_H
#define PAISING_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PA_ABI_VERSION 1

#if defined(__GNUC__)
#define PA_API __attribute__((visibility("default")))
#else
#define PA_API
#endif

enum pa_status {
  PA_OK = 0,
  PA_ERR_ARG = 1,          /* invalid argument or unsupported size */
  PA_ERR_CUDA = 2,         /* a CUDA call failed (message in pa_last_error) */
  PA_ERR_CAPACITY = 3,     /* the population outgrew its preallocated buffer */
  PA_ERR_EXTINCT = 4,      /* resampling produced an empty population */
  PA_ERR_STATE = 5,        /* call out of order (e.g. rows before a run) */
  PA_ERR_TOO_MANY_STEPS = 6 /* schedule longer than nBmax = 10000 (PAisingSSC.cu:634-641) */
};

enum pa_coding { PA_CODING_SSC = 0, PA_CODING_MSC = 1 };
/* PA_RNG_NATIVE: the engine's own Philox streams.  PA_RNG_REFERENCE: every
 * random number is the Philox4x32-10 word the reference would draw at the
 * same (subsequence, counter) coordinates -- the injected test stream that
 * makes spins, energies and copy numbers bit-exact with the reference
 * programs built against the same stream. */
enum pa_rng_mode { PA_RNG_NATIVE = 0, PA_RNG_REFERENCE = 1 };
/* resampling weights: FP32 with compensated sums (default) or FP64 in the
 * reference's formulation (Emean shift) */
enum pa_weights { PA_WEIGHTS_FP32 = 0, PA_WEIGHTS_FP64 = 1 };

typedef struct pa_config {
  int L;             /* lattice size; #define L (PAisingSSC.cu:27), a runtime value here */
  int R;             /* initial population size, -R Rinit (PAisingSSC.cu:46,390) */
  int sweeps;        /* equilibration sweeps per temperature, -t (PAisingSSC.cu:35,391) */
  double dbeta;      /* inverse temperature step, -d (PAisingSSC.cu:39,392) */
  double beta_final; /* final inverse temperature, -f (PAisingSSC.cu:38,393) */
  int runs;          /* independent runs, -M (PAisingSSC.cu:48,394) */
  uint64_t seed;     /* -s RNGseed (PAisingSSC.cu:395) */
  int coding;        /* pa_coding: PAisingSSC or PAisingMSC */
  int rng_mode;      /* pa_rng_mode */
  int weights;       /* pa_weights */
  int graph;         /* 1: each run is one CUDA graph launch; 0: host steps every temperature */
  int device;        /* CUDA device ordinal */
  double capacity;   /* replica buffer = ceil(capacity * R) + 256; 0 selects 1.25 */
  int sweep_variant; /* MSC sweep kernel: 0 automatic, 1 one CTA per group, 2 or 4: a thread-block
                        cluster of that many CTAs per group (needed for L > 128; chosen automatically
                        for batches of 48 <= L <= 128, L % 8 == 0, with too few groups to fill the
                        GPU; above L = 128 automatically 4 when the groups need more than one and at
                        most eight waves of resident clusters of 2, else 2).  SSC: 0 automatic
                        (native stream: bit planes, 32 sites per word, where L packs into words at
                        least 3/4 full -- L = 8, 16, 24, 32, 48, 56, 64, 96, 112, 128, 144, 168, 192,
                        224, 240, 256 -- else int8), 1 int8 */
  int tile_groups;   /* MSC groups stacked into one work unit of the one-CTA sweep: 0 automatic,
                        1, 2, 4 or 8 (more than 1 needs L % 4 == 0 and at most 44 KB per tile).
                        SSC bit planes (native stream): replicas per tile, 0 automatic, else the
                        largest tile for L (pa_sweep_form) or a power-of-two fraction of it; the
                        whole batch then runs on bit planes */
  int adaptive;      /* 1: adaptive temperature step, the reference's AdaptiveStep build
                        (PAisingSSC.cu:23,306-334,644-660): after every temperature the next step is
                        the largest (grown by 1.1x, else bisected) whose energy-histogram overlap lies
                        in [min_overlap, max_overlap); dbeta is the first step.  Runs after the first
                        reuse the first run's schedule, as in the reference. */
  double min_overlap; /* MinOverlap (PAisingSSC.cu:42); 0 selects 0.85 */
  double max_overlap; /* MaxOverlap (PAisingSSC.cu:43); 0 selects 0.87 */
  int mhr;            /* 1: multi-histogram reweighting, the reference's MHR build (PAisingSSC.cu:22,
                         294-302,694-790): the energy histogram of every temperature of a run is
                         accumulated on the device and reweighted after the run (pa_get_mhr_rows,
                         PA_MHR_results_run_<r>.dat) */
  int store_energies; /* 1: keep the energies of every temperature, the reference's EnergiesPopStore
                         build (PAisingSSC.cu:24,563-578): pa_get_energies, PA_energies_<i>.dat */
  int family;         /* 1: family statistics at every temperature (no counterpart in the reference):
                         every replica carries the initial replica it descends from through the
                         resampling; pa_get_family_rows, PA_family_run_<r>.dat */
} pa_config;

/* One line of PA_results_run_<r>.dat (PAisingSSC.cu:679-690), per site. */
typedef struct pa_row {
  double beta, e, c, m, m2, m4, bf, s, r, lnq;
} pa_row;

typedef struct pa_handle pa_handle;

/* Fills cfg with the reference defaults: L=64, R=20000, 100 sweeps,
 * dbeta=0.005, beta_final=1, 1 run, seed 1, SSC, native RNG, FP32 weights,
 * graph mode (PAisingSSC.cu:27,35-50). */
PA_API int pa_config_init(pa_config* cfg);

/* Allocates the population buffers for cfg on cfg->device.  Replaces the
 * set-up part of main() (PAisingSSC.cu:438-479).  With the native stream,
 * cfg->runs > 1 independent runs (-M) are annealed concurrently as a batch
 * of populations with disjoint streams; with the reference stream they run
 * one after the other because each run continues the previous run's
 * subsequence counter (PAisingSSC.cu:481-486). */
PA_API int pa_create(const pa_config* cfg, pa_handle** out);

/* A batch of n independent populations, each with its own L, R, sweeps,
 * dbeta, beta_final and seed (runs must be 1; coding, rng_mode, weights,
 * graph and device must agree), annealed together: one persistent sweep
 * launch per temperature step serves every population, so small or uneven
 * populations fill the GPU.  Population k's rows are result set k.  No
 * counterpart in the reference, which runs one population per process. */
PA_API int pa_create_batch(const pa_config* cfgs, int n, pa_handle** out);

/* Runs the handle's anneals (beta from 0 while beta <= beta_final), the
 * population-annealing loop of main() (PAisingSSC.cu:481-664,
 * PAisingMSC.cu:640-814).  Each call is a new run: the subsequence counter
 * continues, and with the native stream the run number enters every sweep
 * draw's counter, so repeated calls give independent runs. */
PA_API int pa_run(pa_handle* h);

/* A run stepped from the host, for hosts that interleave their own work or
 * checkpoint long anneals: pa_run_begin sets up the run and its initial
 * population (temperature 0), pa_run_steps advances up to max_steps
 * temperatures (*done = 1 once every population has finished its schedule),
 * pa_run_end collects the rows like pa_run.  The same launches as the plain
 * mode; handles with one run (runs = 1, or a native batch).  No counterpart
 * in the reference, whose main() loop runs to the end. */
PA_API int pa_run_begin(pa_handle* h);
PA_API int pa_run_steps(pa_handle* h, int max_steps, int* done);
PA_API int pa_run_end(pa_handle* h);

/* Between the steps of a stepped run: the complete state of every
 * population (spins, energies, schedule, rows so far, stream positions,
 * MHR histogram, ancestors) to a binary file, and back into a handle created
 * with the same configurations, which then continues with pa_run_steps and
 * pa_run_end exactly as the original would have.  Runs that store their
 * energies are not checkpointed.
 *
 * pa_restore reads and checks the whole file before it writes to the device:
 * a file of another configuration, a truncated one, or one whose state lies
 * outside the handle's buffers (a population size beyond the capacity, a
 * buffer parity other than 0 or 1, a temperature index beyond the schedule,
 * a buffer of the wrong size) returns PA_ERR_ARG and leaves the handle as it
 * was.  Only a CUDA error while the buffers are being written leaves it
 * inconsistent; it then refuses to run (PA_ERR_STATE) until a restore
 * succeeds.  pa_checkpoint_verify makes the file-level checks alone, on the
 * host, without a handle or a device (message: pa_last_error(NULL)).  The
 * reference has no checkpoints (its state lives in one process). */
PA_API int pa_checkpoint(pa_handle* h, const char* path);
PA_API int pa_restore(pa_handle* h, const char* path);
PA_API int pa_checkpoint_verify(const char* path);

/* Autotuner of the sweep's tile shape and spins per word.  It times one
 * sweep launch of the handle's populations (freshly initialised, at the first
 * temperature) per candidate, keeps the fastest per spin-flip attempt and
 * rebuilds the launch plan (and graph):
 *   MSC, one CTA per work unit: for every lattice size, 1, 2, 4 or 8 groups
 *     of 32 replicas stacked per work unit, where valid; then, when every
 *     population has 48 <= L <= 128, L % 8 == 0 and leaves the form to the
 *     engine, that tuned form against clusters of 2 and of 4 CTAs per group
 *     for the whole batch.
 *   MSC, a lattice above L = 128 (clusters needed), every population leaving
 *     the form to the engine and able to take both: clusters of 2 CTAs of
 *     1024 threads against clusters of 4 of 512 for the whole batch.
 *   For MSC, results under the reference stream are unchanged by the choice
 *   (draws are keyed by group and site); the native stream's draws follow the
 *   form, as for SSC below.
 *   SSC, native stream, every L with a bit-plane layout and sweep_variant 0:
 *     for every lattice size the bit-plane tile (replicas per work unit), then
 *     for the whole batch the int8 sweep (4 sites of a replica per 32-bit
 *     word) or the bit-plane sweep (32 sites per word).  The forms and tiles
 *     draw different native streams (all with acceptance probability exactly
 *     T/2^32), so the choice changes the trajectory, not the statistics.
 * Must precede the first pa_run; the runs that follow start from the
 * configured state exactly as without it.  tiles[k] (k < n, may be null with
 * n = 0) receives population k's work-unit size (groups per tile for MSC,
 * replicas per tile for SSC); pa_sweep_form reports the whole form.  No
 * counterpart in the reference, whose launch shapes and MSbits are
 * compile-time constants (PAisingMSC.cu:34). */
PA_API int pa_autotune(pa_handle* h, int* tiles, int n);

/* The sweep form population `index` is annealed with. */
typedef struct pa_sweep_form_t {
  int spins_per_word;    /* spins held by one 32-bit word: SSC 4 (int8) or 32 (bit planes); MSC 32 */
  int replicas_per_word; /* SSC 1; MSC 32 (bit k = replica k of the group) */
  int tile;              /* work unit: MSC groups per tile, SSC replicas per tile */
  int cluster_ctas;      /* CTAs sweeping one MSC group together (1, 2 or 4); SSC 1 */
} pa_sweep_form_t;
PA_API int pa_sweep_form(const pa_handle* h, int index, pa_sweep_form_t* out);

/* Number of result sets a pa_run produces: one per population per
 * sequential run (PA_results_run_<set>.dat). */
PA_API int pa_num_sets(const pa_handle* h, int* n);

/* Longest number of rows of any result set (schedule length + 1). */
PA_API int pa_num_rows(const pa_handle* h, int* nrows);

/* Copies the rows of result set `set` (the contents of
 * PA_results_run_<set>.dat, PAisingSSC.cu:670-692) into rows[0..max_rows);
 * *nrows receives the number copied. */
PA_API int pa_get_rows(const pa_handle* h, int set, pa_row* rows, int max_rows, int* nrows);

/* Multi-histogram reweighting of result set `set` (config mhr = 1): 4
 * doubles per temperature, beta, E/N, C/N and betaF/N, the columns of the
 * reference's PA_MHR_results_run_<r>.dat (PAisingSSC.cu:694-786).  At most
 * max_rows rows are copied; *nrows receives the number available. */
PA_API int pa_get_mhr_rows(const pa_handle* h, int set, double* rows, int max_rows, int* nrows);

/* Energies of the population of result set `set` at temperature `step`
 * (config store_energies = 1; step 0 is the initial population), in the
 * reference's replica order (MSC: group-major, active replicas only): the
 * contents of PA_energies_<step>.dat (PAisingSSC.cu:563-578).  At most max
 * values are copied; *n receives the population size. */
PA_API int pa_get_energies(const pa_handle* h, int set, int step, int32_t* out, int max, int* n);

/* The reference's LatticePopStore build (PAisingSSC.cu:25,580-605): during the
 * handle's first run, after every temperature i >= 1 the population is
 * appended as text to dir/PA_lattice_<i>.dat ("i=..; beta=..; R=..;" and one
 * "P={{row},..};" line per replica, `precision` digits for beta).  The run is
 * then stepped from the host.  MSC populations (not in the reference) list
 * their active replicas group-major.  One population per handle; dir = NULL
 * switches the dumps off. */
PA_API int pa_set_lattice_dump(pa_handle* h, const char* dir, int precision);

/* Family statistics of result set `set` (config family = 1), 3 doubles per
 * temperature: the number of families (initial replicas with descendants),
 * rho_t = sum_f c_f^2 / R and the family entropy S_f = -sum_f (c_f/R)
 * ln(c_f/R), c_f the replicas descended from initial replica f.  No
 * counterpart in the reference. */
PA_API int pa_get_family_rows(const pa_handle* h, int set, double* rows, int max_rows, int* nrows);

/* Device time of the last pa_run in milliseconds (CUDA events around all
 * runs), and the reference's spin-flip attempt count
 * sweeps * N * sum_{i>=1} R_i over all runs (PAisingSSC.cu:632,806). */
PA_API int pa_get_timing(const pa_handle* h, double* ms, double* attempts);

/* Initial populations for the following pa_run calls instead of the random
 * initialisation (ReplicaInit, PAisingSSC.cu:150-157) -- e.g. to resume from
 * saved populations.  host holds, for every population of the handle in
 * order, its R replicas in the stage layout of the handle's coding (SSC: int8
 * [R][N]; MSC: uint32 [ceil(R/32)][N], bit k of group g = replica 32g+k).
 * The copies are complete when the call returns.  host = NULL restores the
 * random initialisation. */
PA_API int pa_set_population(pa_handle* h, const void* host);

/* Final population of population `pop` after the last pa_run, in the same
 * layout (MSC groups as stored: after resampling, replica s is at group
 * s / 32, bit s % 32 with the native stream, and at group s % rg, bit s / rg
 * with the reference stream, PAisingMSC.cu:413-414).  *R receives the
 * population size; bytes is the capacity of host. */
PA_API int pa_get_population(const pa_handle* h, int pop, void* host, size_t bytes, int* R);

/* Per-kernel device time of one run executed launch by launch with CUDA
 * events on the handle's stream around every kernel (serialised; for
 * profiling and rooflines, not for throughput).  Fills up to max entries. */
typedef struct pa_kernel_time {
  char name[24];
  int launches;
  double total_ms;
} pa_kernel_time;
PA_API int pa_profile_run(pa_handle* h, pa_kernel_time* out, int max, int* n);

/* Writes dir/PA_results_run_<r>.dat for every run with `precision`
 * significant digits (PAisingSSC.cu:670-692), PA_MHR_results_run_<r>.dat
 * where mhr is on, and PA_energies_<i>.dat (i >= 1, last run) where
 * store_energies is on and the handle holds one population. */
PA_API int pa_write_results(const pa_handle* h, const char* dir, int precision);

PA_API int pa_destroy(pa_handle* h);

PA_API const char* pa_status_string(int status);
/* Message of the last failure on this handle (or of the last failed
 * handle-less call when h is NULL). */
PA_API const char* pa_last_error(const pa_handle* h);
PA_API int pa_abi_version(void);

/* The inverse-temperature schedule of a run: betas[0] = 0 and
 * betas[i] = betas[i-1] + dbeta while betas[i] <= beta_final, accumulated in
 * FP64 exactly like the reference (PAisingSSC.cu:508-510,661), so
 * dbeta = 0.005 stops at 0.995 (200 rows).  Writes at most max entries;
 * *n receives the full length. */
PA_API int pa_schedule(double dbeta, double beta_final, double* betas, int max, int* n);

/* The random word the reference would draw as number ctr of the cuRAND
 * subsequence subseq under the injected stream (Philox4x32-10 keyed by seed,
 * counter (ctr >> 2, subseq), word ctr & 3).  Host-side, for checks. */
PA_API uint32_t pa_ref_word(uint64_t seed, uint64_t subseq, uint64_t ctr);

/* ------------------------------------------------------------------------
 * Stage entry points (device pointers).  Layouts:
 *   SSC spins : int8 [R][N], +-1, sublattice A (x+y even) then B, site (x,y)
 *               at y*L/2 + x/2 inside a sublattice (PAisingSSC.cu:70-77,169)
 *   MSC words : uint32 [rg][N], same split; bit k = replica k of the group,
 *               1 == +1 (PAisingMSC.cu:84-92); active: uint8 [rg*32]
 *   energies  : int32 E, M per replica (MSC: index 32*group + bit)
 * `iseq` is the reference's subsequence counter (initial_sequence,
 * PAisingSSC.cu:418) at the call; `step` keys the native stream.
 * ------------------------------------------------------------------------ */

/* ReplicaInit (PAisingSSC.cu:150-157): R random +-1 lattices. */
PA_API int pa_ssc_init(int8_t* spins, int L, int R, uint64_t seed, uint64_t iseq, void* stream);

/* checkKerALL + energyKer (PAisingSSC.cu:159-215): `sweeps` checkerboard
 * Metropolis sweeps at inverse temperature beta, then E and M per replica. */
PA_API int pa_ssc_sweep(int8_t* spins, int L, int R, int sweeps, double beta, int rng_mode, uint64_t seed,
                 uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream);

/* The same sweeps on bit planes (native stream only; no counterpart in the
 * reference): the population is packed to one bit per site in shared memory
 * (a sublattice row as words of up to 32 sites, or several replicas' rows per
 * word when a row has at most 16 sites), swept with the bitsliced adder and
 * the digit-serial acceptance, and unpacked.  Each site flips with
 * probability exactly min(1, T/2^32) like pa_ssc_sweep's native stream, from
 * another stream.  PA_ERR_ARG where L has no bit-plane layout. */
PA_API int pa_ssc_sweep_bits(int8_t* spins, int L, int R, int sweeps, double beta, uint64_t seed, int step,
                             int32_t* E, int32_t* M, void* stream);

/* ReplicaInit (PAisingMSC.cu:169-188): ceil(R/32) groups, active bits. */
PA_API int pa_msc_init(uint32_t* words, uint8_t* active, int L, int R, uint64_t seed, uint64_t iseq, void* stream);

/* checkKerALL + energyKer (PAisingMSC.cu:191-317) for rg groups. */
PA_API int pa_msc_sweep(uint32_t* words, const uint8_t* active, int L, int rg, int sweeps, double beta, int rng_mode,
                 uint64_t seed, uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream);

/* QKer + host lnQ + CalcTauKer + CalcParSum (PAisingSSC.cu:217-270,533;
 * PAisingMSC.cu:319-395): from the energies of the population before
 * resampling (n = R_prev for SSC, 32 * ceil(R_prev/32) slots with `active`
 * for MSC) computes copy numbers roff[n], their exclusive scan offs[n], the
 * gather map src[R_new] (new replica -> old linear index) and, in the HOST
 * array out[3], out[0] = lnQ, out[1] = q, out[2] = R_new.  e_ref is Emean for
 * FP64 weights and Emin for FP32 weights.  Uses internal scratch memory. */
PA_API int pa_resample_plan(const int32_t* E, const uint8_t* active, int coding, int R_prev, int Rinit, int Rcap,
                     double beta_prev, double beta, double e_ref, int weights, uint64_t seed, uint64_t iseq,
                     uint32_t* roff, uint32_t* offs, uint32_t* src, double* out, void* stream);

/* No counterpart in the reference.  pa_resample_plan for callers that cannot
 * allocate device memory -- e.g. a host framework that has reserved the
 * device's memory for its own allocator, or a latency-critical loop that
 * cannot afford the device-wide synchronisation cudaFree implies.  Same
 * arguments, kernels and results as pa_resample_plan, but it calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch is a
 * 32 KB array in the library's device memory, held by every GPU that loads
 * the library until the process exits.  Limit: at most 262144 replica slots
 * (SSC: R_prev; MSC: 32 * ceil(R_prev/32)); larger inputs return PA_ERR_ARG.
 * All calls share that one array, so calls whose GPU work overlaps (other
 * streams or host threads) race.  Every call looks up the array's address
 * on the current device (which allocates nothing); the first call on a
 * device may load the library's device code, so make it before any stream
 * capture. */
PA_API int pa_resample_plan_noalloc(const int32_t* E, const uint8_t* active, int coding, int R_prev, int Rinit,
                                    int Rcap, double beta_prev, double beta, double e_ref, int weights, uint64_t seed,
                                    uint64_t iseq, uint32_t* roff, uint32_t* offs, uint32_t* src, double* out,
                                    void* stream);

/* resampleKer (PAisingSSC.cu:272-280): new[s] = old[src[s]], s < R_new. */
PA_API int pa_ssc_resample(const int8_t* old_spins, int L, const uint32_t* src, int R_new, int8_t* new_spins, void* stream);

/* resampleKer (PAisingMSC.cu:397-435): new group j, bit k <- old replica
 * src[k*rg_new + j], rg_new = ceil(R_new/32); new_active filled. */
PA_API int pa_msc_resample(const uint32_t* old_words, int L, const uint32_t* src, int R_new, uint32_t* new_words,
                    uint8_t* new_active, void* stream);

/* The native stream's MSC gather (no counterpart in the reference): the
 * engine's own stream places offspring s at slot s (group s / 32, bit s % 32)
 * instead of the reference's s % rg_new, s / rg_new, so that a new word is
 * assembled from a few shifted old words.  new bit s <- old replica src[s],
 * s < R_new (src nondecreasing, values < R_old); old_words holds
 * ceil(R_old/32) groups; new_active filled. */
PA_API int pa_msc_resample_native(const uint32_t* old_words, int L, int R_old, const uint32_t* src, int R_new,
                                  uint32_t* new_words, uint8_t* new_active, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PAISING_H */
