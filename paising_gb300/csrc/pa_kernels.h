// pa_kernels.h -- host-side launchers of the engine's CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pa_state.h"

namespace pa {

// Thread layout of a sweep kernel for one lattice size (chosen on the host).
struct SweepGeom {
  int L, N, half;
  int Wr;      // 32-bit words per sublattice row (SSC: 4 sites/word -> L/8; MSC: 1 site/word -> L/2)
  int rpp;     // sublattice rows handled per pass
  int T;       // threads doing site work = Wr * rpp
  int block;   // blockDim.x (T rounded up to a multiple of 32)
  int npass;   // ceil(L / rpp)
  int kconst;  // (N/2)/128 when 128 divides N/2 (draws per reference thread per half sweep), else 0
  int smem;    // dynamic shared memory bytes
  int grid;    // persistent grid size
};

bool ssc_geom(int L, int max_threads, SweepGeom* g);
bool msc_geom(int L, int max_threads, SweepGeom* g);

// Occupancy-derived persistent grid for the sweep kernels.
cudaError_t ssc_sweep_setup(SweepGeom* g, int rng_mode);
cudaError_t msc_sweep_setup(SweepGeom* g, int rng_mode);

// SSC (int8 spins)
cudaError_t launch_ssc_init(PopDev* st, const PopDev& h, cudaStream_t s);
cudaError_t launch_ssc_sweep(PopDev* st, const SweepGeom& g, int rng_mode, int sweeps, cudaStream_t s);
cudaError_t launch_ssc_resample(PopDev* st, const PopDev& h, cudaStream_t s);

// MSC (32 replicas per uint32 word)
cudaError_t launch_msc_init(PopDev* st, const PopDev& h, cudaStream_t s);
cudaError_t launch_msc_sweep(PopDev* st, const SweepGeom& g, int rng_mode, int sweeps, cudaStream_t s);
cudaError_t launch_msc_resample(PopDev* st, const PopDev& h, cudaStream_t s);

// Resampling (both codings)
int res_blocks(const PopDev& h);
cudaError_t launch_q(PopDev* st, const PopDev& h, cudaStream_t s);
cudaError_t launch_copy_numbers(PopDev* st, const PopDev& h, cudaStream_t s);
cudaError_t launch_scatter(PopDev* st, const PopDev& h, cudaStream_t s);
// initial statistics / per-step bookkeeping
cudaError_t launch_begin_run(PopDev* st, cudaStream_t s);
cudaError_t launch_finish_step(PopDev* st, cudaStream_t s);

}  // namespace pa
