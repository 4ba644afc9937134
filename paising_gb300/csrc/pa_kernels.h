// pa_kernels.h -- host-side launchers of the engine's CUDA kernels.
//
// All launchers work on a batch of populations: per-population kernels take
// the population from blockIdx.y (resampling) or blockIdx.x (bookkeeping);
// the sweep kernels are persistent and take work units of all populations
// from one queue (BatchDev::work_next).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pa_state.h"

namespace pa {

// Thread layout of a sweep over one lattice size (chosen on the host and
// stored per population in PopDev).
struct SweepGeom {
  int L, N, half;
  int Wr;      // 32-bit words per sublattice row (SSC: 4 sites/word -> L/8; MSC: 1 site/word -> L/2)
  int rpp;     // sublattice rows handled per pass
  int T;       // threads doing site work = Wr * rpp (<= kSweepThreads)
  int npass;   // ceil(L / rpp)
  int kconst;  // (N/2)/128 when 128 divides N/2 (draws per reference thread per half sweep), else 0
  int smem;    // dynamic shared memory bytes for one work unit
  int G = 1;   // MSC groups per work unit: G lattices stacked as G*L rows of one sweep
              // (SSC bit planes: replicas per work unit)
  int seg = 0; // SSC bit planes: sites of a sublattice row per word segment
};

// ceil(2^32 / d) for 2 <= d < 2^16: then __umulhi(n, recip32(d)) == n / d
// for every n < 2^16 (the rounding error n * (ceil - 2^32/d) / 2^32 < 2^-16 is
// smaller than the distance 1/d from n/d to the next integer).
inline unsigned int recip32(int d) {
  return (unsigned int)((0x100000000ull + (unsigned long long)d - 1) / (unsigned long long)d);
}

bool ssc_geom(int L, SweepGeom* g);
// tile: groups per work unit (0 automatic); groups: how many groups the
// sweep launches will hold and slots: resident CTAs of the persistent grid,
// which together drive the automatic choice (single-group tiles when either
// is 0)
bool msc_geom(int L, SweepGeom* g, int tile = 0, long long groups = 0, int slots = 0);
void geom_to_pop(const SweepGeom& g, PopDev* h);

// fixed_l of a launch whose populations include L = 96 with one group per
// work unit beside other sizes: the general MSC kernel with L = 96's
// compile-time form as well
constexpr int kWith96 = 1;
struct SweepLaunch {
  int grid, block, smem;
  int fixed_l;  // MSC, native stream: 96, kWith96 or 0 (see sweep_setup)
};
// Persistent grid for a sweep kernel with `smem` bytes of dynamic shared memory.
// fixed_l (MSC, native stream): 96 -- every population of the launch has
// L = 96 and one group per work unit, and a kernel built for that size alone
// is used; kWith96 -- some do, beside other sizes; 0 -- none.
cudaError_t sweep_setup(int coding, int rng_mode, int smem, SweepLaunch* out, int fixed_l = 0);
// The fixed_l for MSC populations of lattice size L and G groups per work unit
// (0 where no kernel is built for it).
int msc_fixed_l(int L, int G);

// Work plan of the next sweep launch: unit counts of the populations that
// take part (energy_only: populations at step 0), prefix sums, queue reset.
cudaError_t launch_plan(BatchDev* b, int npop, int energy_only, cudaStream_t s);
// `seed` keys the native sweep stream of the whole batch.
cudaError_t launch_sweep(BatchDev* b, int coding, int rng_mode, int energy_only, unsigned long long seed,
                         const SweepLaunch& sl, cudaStream_t s);

// Random (or caller-supplied) initial populations.
cudaError_t launch_init(PopDev* pops, int npop, int coding, cudaStream_t s);

// Resampling (both codings); `blocks` from res_blocks().
int res_blocks(long long max_units);
cudaError_t launch_q(PopDev* pops, int npop, int blocks, cudaStream_t s);
cudaError_t launch_copy_numbers(PopDev* pops, int npop, int blocks, cudaStream_t s);
cudaError_t launch_scatter(PopDev* pops, int npop, int blocks, cudaStream_t s);
// Gather of the resampled populations of the batch (a plan launch and a
// persistent gather launch taking units of every population from one queue).
cudaError_t launch_resample(BatchDev* b, int coding, int rng_mode, cudaStream_t s);

// Coding-specific launchers behind the generic ones above.
cudaError_t ssc_sweep_setup(int rng_mode, int smem, SweepLaunch* out);
cudaError_t msc_sweep_setup(int rng_mode, int smem, SweepLaunch* out, int fixed_l);
cudaError_t launch_ssc_sweep(BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                             const SweepLaunch& sl, cudaStream_t s);
cudaError_t launch_msc_sweep(BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                             const SweepLaunch& sl, cudaStream_t s);
cudaError_t launch_ssc_init(PopDev* pops, int npop, cudaStream_t s);
cudaError_t launch_msc_init(PopDev* pops, int npop, cudaStream_t s);
cudaError_t launch_ssc_resample(BatchDev* b, cudaStream_t s);
cudaError_t launch_msc_resample(BatchDev* b, int rng_mode, cudaStream_t s);

// SSC populations swept on bit planes (native stream): tiles of G replicas
// packed to one bit per site in shared memory, a sublattice row as Wr words
// of `seg` sites (several replicas' rows per word when a row is at most 16
// sites).  False where L has no such layout.  Replicas per tile: `tile` if
// given (the largest tile for L halved k times, else false), else the
// largest such tile that still leaves a tile for each of `slots` resident
// CTAs given the batch's replicas, else the largest tile (about 1024 words
// per plane).
bool ssc_bits_geom(int L, SweepGeom* g, int tile = 0, long long replicas = 0, int slots = 0);
// Fraction of the bits of the packed words that hold sites (1 at L = 16, 32,
// 64, 128, 256; 0.75 at L = 24, 48, 96; 0 where no bit-plane layout exists).
double ssc_bits_fill(int L);
cudaError_t ssc_bits_setup(int smem, SweepLaunch* out);
cudaError_t launch_ssc_bits_sweep(BatchDev* b, int energy_only, unsigned long long seed, const SweepLaunch& sl,
                                  cudaStream_t s);

// MSC sweep by thread-block clusters of cs = 2 or 4 CTAs (one horizontal
// stripe of the group per CTA), for lattices too large for one CTA.
bool msc_cluster_geom(int L, int cs, int threads, SweepGeom* g);
int msc_cluster_threads(int cs, int maxL);
cudaError_t msc_cluster_setup(int cs, int threads, int rng_mode, int smem, SweepLaunch* out);
cudaError_t launch_msc_cluster_sweep(int cs, int threads, BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                                     const SweepLaunch& sl, cudaStream_t s);

// Per-run / per-step bookkeeping.
cudaError_t launch_begin_run(PopDev* pops, int npop, cudaStream_t s);
cudaError_t launch_finish_step(PopDev* pops, int npop, cudaStream_t s);
// Populations with records: histogram / energy ring of the temperature just
// finished (after launch_finish_step); `blocks` from res_blocks().
cudaError_t launch_record(PopDev* pops, int npop, int blocks, cudaStream_t s);
// Family statistics: ancestors set at the initial population, carried by
// each resampling (after launch_resample), counted after launch_finish_step.
cudaError_t launch_family_init(PopDev* pops, int npop, int blocks, cudaStream_t s);
cudaError_t launch_family_resample(PopDev* pops, int npop, int blocks, cudaStream_t s);
cudaError_t launch_family_stats(PopDev* pops, int npop, int blocks, cudaStream_t s);
// Adaptive populations: choose the next temperature (after launch_finish_step).
cudaError_t launch_adapt(PopDev* pops, int npop, cudaStream_t s);

}  // namespace pa
