// pa_state.h -- device state of the annealing engine.
//
// One PopDev lives in device memory per population; a BatchDev lists the
// populations that advance together.  Every kernel of a temperature step
// reads its sizes, buffer pointers and scalars from there, so a whole
// schedule is captured once as a CUDA graph: nothing the host learns only
// after a step (population sizes, the parity of the double buffer, lnQ, ...)
// is baked into launch arguments.
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace pa {

enum Coding : int { kSSC = 0, kMSC = 1 };
enum RngMode : int { kNative = 0, kRefCoords = 1 };
enum Weights : int { kFP32Kahan = 0, kFP64 = 1 };

constexpr int kMsb = 32;          // replicas per MSC word (MSbits, PAisingMSC.cu:34)
constexpr int kRefThreads = 128;  // EQthreads (PAisingSSC.cu:62): fixes the reference's draw layout
constexpr int kThrPerStep = 12;   // [0..9] SSC table thresholds, [10] T4, [11] T8
constexpr int kRowCols = 10;
constexpr int kResBlocksMax = 1024;
constexpr int kMaxPop = 1024;     // populations per batch
constexpr int kSweepThreads = 256;

struct PopDev {
  // ------------------------------------------------ configuration (constant)
  int L, N, coding, Rinit, Rcap, rgcap, sweeps, rng_mode, weights, pop_id, nsteps;
  int seg;  // SSC bit-plane sweep: sites per word segment (SweepGeom::seg)
  // sweep thread layout (see SweepGeom): words per row, rows per pass,
  // worker threads, passes, reference draws per thread per half sweep,
  // MSC groups per work unit (tile), and the reciprocals of L and Wr used
  // to split row and word indices without division
  int Wr, rpp, T, npass, kconst, gpt;
  unsigned int invL, invWr;
  unsigned long long seed;
  // ------------------------------------------------ buffers
  void* spins[2];      // SSC: int8 [Rcap][N] (+-1, sublattice A then B); MSC: uint32 [rgcap][N]
  int32_t* E;          // SSC [Rcap], MSC [rgcap*32]: energy of the current population
  int32_t* M;          // magnetisation, same indexing
  uint8_t* active[2];  // MSC: [rgcap*32] replica present (isActive, PAisingMSC.cu:91)
  uint32_t* roff;      // copy numbers of the previous population
  uint32_t* offs;      // exclusive scan of roff
  uint32_t* src;       // new linear replica index -> old linear replica index
  uint32_t* blk_tot;   // [kResBlocksMax] per-block sums of roff
  uint32_t* blk_off;   // [kResBlocksMax] exclusive scan of blk_tot
  double* qpart_d;     // [kResBlocksMax] FP64 partial sums of the weights
  float* qpart_f;      // [2*kResBlocksMax] FP32 (sum, compensation) partials
  double* rows;        // [(nsteps+1) * 10] output rows (columns of PA_results_run_<r>.dat)
  double* betas;       // [nsteps+1] (adaptive: [kNBmax], filled in as the run goes)
  uint32_t* thr;       // [(nsteps+1) * kThrPerStep], same
  uint32_t* hist;      // adaptive only: [N+1] energy histogram, bin (E + 2N) / 4
  const void* init_src;  // device copy of a caller-supplied initial population, or null (random init)
  // ------------------------------------------------ dynamic scalars
  int step;            // temperature index being computed (1..nsteps); nsteps+1 when done
  int R_prev;          // population size before resampling
  int R_cur;           // population size after resampling
  int parity;          // spins[parity] holds the current population
  int error;           // 0 ok, 1 capacity exceeded, 2 population extinct
  int Emin;            // minimum energy of the current population
  unsigned int ticket;     // last-block tickets of the resampling kernels
  int run;             // runs begun on this population before the current one (native stream key)
  unsigned long long iseq;  // reference subsequence counter (initial_sequence, PAisingSSC.cu:418)
  double Emean;        // <E> of the current population (Emean, PAisingSSC.cu:483,620)
  double sumlnQ;       // -sum of lnQ over the steps so far (PAisingSSC.cu:627)
  double lnQ;          // lnQ of the step being computed
  double q;            // sum of the resampling weights of the step being computed
  double bf0;          // -N ln 2, betaF at beta = 0 (PAisingSSC.cu:435), computed on the host
  // ------------------------------------------------ statistics accumulators
  long long sE, sE2, sM, sM2;
  unsigned long long sM4lo, sM4hi;
  int Emin_acc, pad3;
  // ------------------------------------------------ adaptive temperature step
  int adaptive;        // 1: the next beta is chosen after every temperature
  int pad4;
  double dbeta_cur;    // deltaBeta carried from step to step (PAisingSSC.cu:508,659)
  double min_ov, max_ov, beta_fin;
  // ------------------------------------------------ per-temperature records
  int rec;             // kRecMhr | kRecEnergies
  int last_rec;        // last temperature index recorded in this run (-1: none)
  int ring;            // temperatures the energy ring holds (slot = index % ring)
  int pad5;
  unsigned long long* mhr_hist;  // [N+1] energy histogram of all temperatures of the run
  int32_t* elog;       // [ring][units] energies of recorded temperatures
  uint8_t* alog;       // MSC: [ring][units] active flags of the same
  int* nlog;           // [ring] units recorded per slot
  // ------------------------------------------------ family statistics
  int family;          // 1: ancestors follow the replicas; statistics every temperature
  int last_fam;        // last temperature whose statistics are done in this run (-1: none)
  int32_t* anc[2];     // [units] initial replica each slot descends from, double-buffered like spins
  uint32_t* fam_cnt;   // [Rinit] replicas per family; zero between temperatures
  double* fam_rows;    // [rows][3] families, rho_t, S_f per temperature
  double* fam_part;    // [kResBlocksMax][3] per-block partial sums
  // ------------------------------------------------ MSC gather, native stream
  // (offspring s at slot s = 32 * group + bit): per new group the distinct
  // source shifts of its bits as (bit mask, shift) pairs, grouped by which
  // pair of window words they read, and their counts (msc_pairs_kernel)
  uint2* res_pairs;    // [rgcap][32]
  uint32_t* res_cnt;   // [rgcap]: pair counts n0 | n1 << 5 | n2 << 10 | k1 << 15 | k2 << 20 | k3 << 25,
                       // per-bit fallback << 31
};

constexpr int kRecMhr = 1, kRecEnergies = 2;

constexpr int kNBmax = 10000;  // nBmax, PAisingSSC.cu:57: rows of a schedule at most
// error codes in PopDev::error
constexpr int kErrCapacity = 1, kErrExtinct = 2, kErrTooManySteps = 3;
constexpr int kErrSweepForm = 4;  // a sweep kernel built for one lattice size met another (a host bug)

// Populations advancing together.  unit_prefix[p] .. unit_prefix[p+1]-1 are
// the sweep work units (SSC replicas, MSC groups) of population p in the
// current sweep launch; work_next hands them out to persistent CTAs.
struct BatchDev {
  int npop;
  unsigned int work_next;
  PopDev* pops;
  int unit_prefix[kMaxPop + 1];
  // the MSC resampling gather's work list: units of 32 new groups x 32 sites
  unsigned int res_next;
  int res_prefix[kMaxPop + 1];
  int grp_prefix[kMaxPop + 1];  // new groups of the populations before p (native-stream pair pass)
};

// A population takes part in the current temperature step.
__host__ __device__ inline bool pop_stepping(const PopDev* st) {
  return st->step >= 1 && st->step <= st->nsteps && !st->error;
}

}  // namespace pa
