// pa_stages.cu -- stage entry points of the C ABI: one reference kernel (or
// kernel group) each, on caller-owned device buffers.  They run the same
// kernels as the engine; a small PopDev describing the caller's buffers is
// placed in scratch device memory for the duration of the call.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "../../include/paising.h"
#include "pa_error.h"
#include "pa_kernels.h"

using namespace pa;

namespace {

int stage_fail(cudaError_t e, const char* what) {
  pa::g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return PA_ERR_CUDA;
}

// Scratch of one stage call: the PopDev plus betas/thresholds and the
// resampling partial-sum buffers.
struct Scratch {
  PopDev* st = nullptr;
  double* betas = nullptr;
  uint32_t* thr = nullptr;
  uint32_t* blk = nullptr;   // blk_tot | blk_off
  double* qd = nullptr;
  float* qf = nullptr;
  void* base = nullptr;
  cudaError_t alloc() {
    const size_t sz = 4096 + 2 * sizeof(double) + 2 * kThrPerStep * 4 + 2 * kResBlocksMax * 4 +
                      kResBlocksMax * 8 + 2 * kResBlocksMax * 4 + 256;
    cudaError_t e = cudaMalloc(&base, sz);
    if (e != cudaSuccess) return e;
    char* p = (char*)base;
    st = (PopDev*)p;
    p += 4096;
    betas = (double*)p;
    p += 2 * sizeof(double);
    thr = (uint32_t*)p;
    p += 2 * kThrPerStep * 4;
    blk = (uint32_t*)p;
    p += 2 * kResBlocksMax * 4;
    qd = (double*)(((uintptr_t)p + 7) & ~(uintptr_t)7);
    p = (char*)(qd + kResBlocksMax);
    qf = (float*)p;
    return cudaSuccess;
  }
  ~Scratch() {
    if (base) cudaFree(base);
  }
};

void fill_thr(double beta, uint32_t* t) {
  for (int i0 = 0; i0 <= 1; ++i0)
    for (int i1 = 0; i1 <= 4; ++i1) {
      double p = std::exp(-2 * (2 * i0 - 1) * (2 * i1 - 4) * beta);
      if (p > 1.0) p = 1.0;
      t[i0 + 2 * i1] = (uint32_t)(std::ceil(4294967296.0 * p) - 1.0);
    }
  const double t4 = std::ceil(4294967296.0 * std::exp(-4 * beta)), t8 = std::ceil(4294967296.0 * std::exp(-8 * beta));
  t[10] = t4 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t4;
  t[11] = t8 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t8;
}

PopDev base_state(int coding, int L) {
  PopDev h;
  std::memset(&h, 0, sizeof(h));
  h.coding = coding;
  h.L = L;
  h.N = L * L;
  h.Emin_acc = 0x7fffffff;
  return h;
}

int upload_and_sync(Scratch& S, const PopDev& h, const double* betas, const uint32_t* thr, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(S.st, &h, sizeof(PopDev), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && betas) e = cudaMemcpyAsync(S.betas, betas, 2 * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && thr) e = cudaMemcpyAsync(S.thr, thr, 2 * kThrPerStep * 4, cudaMemcpyHostToDevice, s);
  return e == cudaSuccess ? PA_OK : stage_fail(e, "upload");
}

}  // namespace

extern "C" {

int pa_ssc_init(int8_t* spins, int L, int R, uint64_t seed, uint64_t iseq, void* stream) {
  SweepGeom g;
  if (!spins || R < 1 || !ssc_geom(L, 256, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kSSC, L);
  h.spins[0] = spins;
  h.R_cur = h.Rinit = R;
  h.seed = seed;
  h.iseq = iseq;
  int rc = upload_and_sync(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  if ((e = launch_ssc_init(S.st, h, s)) != cudaSuccess) return stage_fail(e, "ssc_init");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "ssc_init");
  return PA_OK;
}

int pa_ssc_sweep(int8_t* spins, int L, int R, int sweeps, double beta, int rng_mode, uint64_t seed,
                 uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream) {
  SweepGeom g;
  if (!spins || !E || !M || R < 1 || sweeps < 0 || step < 0 || !ssc_geom(L, 256, &g)) return PA_ERR_ARG;
  if (rng_mode != PA_RNG_NATIVE && rng_mode != PA_RNG_REFERENCE) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = ssc_sweep_setup(&g, rng_mode);
  if (e != cudaSuccess) return stage_fail(e, "ssc setup");
  Scratch S;
  if ((e = S.alloc()) != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kSSC, L);
  h.spins[0] = spins;
  h.R_cur = h.Rinit = R;
  h.R_prev = 0;
  h.seed = seed;
  h.iseq = iseq;
  h.step = 1;
  h.pop_id = step;  // native stream key: (step, pop) -- the stage call folds both into pop_id
  h.E = E;
  h.M = M;
  h.betas = S.betas;
  h.thr = S.thr;
  double b[2] = {0.0, beta};
  uint32_t t[2 * kThrPerStep];
  fill_thr(0.0, t);
  fill_thr(beta, t + kThrPerStep);
  int rc = upload_and_sync(S, h, b, t, s);
  if (rc) return rc;
  if ((e = launch_ssc_sweep(S.st, g, rng_mode, sweeps, s)) != cudaSuccess) return stage_fail(e, "ssc_sweep");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "ssc_sweep");
  return PA_OK;
}

int pa_msc_init(uint32_t* words, uint8_t* active, int L, int R, uint64_t seed, uint64_t iseq, void* stream) {
  SweepGeom g;
  if (!words || !active || R < 1 || !msc_geom(L, 256, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kMSC, L);
  h.spins[0] = words;
  h.active[0] = active;
  h.R_cur = h.Rinit = R;
  h.seed = seed;
  h.iseq = iseq;
  int rc = upload_and_sync(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  if ((e = launch_msc_init(S.st, h, s)) != cudaSuccess) return stage_fail(e, "msc_init");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "msc_init");
  return PA_OK;
}

int pa_msc_sweep(uint32_t* words, const uint8_t* active, int L, int rg, int sweeps, double beta, int rng_mode,
                 uint64_t seed, uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream) {
  SweepGeom g;
  if (!words || !active || !E || !M || rg < 1 || sweeps < 0 || step < 0 || !msc_geom(L, 256, &g)) return PA_ERR_ARG;
  if (rng_mode != PA_RNG_NATIVE && rng_mode != PA_RNG_REFERENCE) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = msc_sweep_setup(&g, rng_mode);
  if (e != cudaSuccess) return stage_fail(e, "msc setup");
  Scratch S;
  if ((e = S.alloc()) != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kMSC, L);
  h.spins[0] = words;
  h.active[0] = const_cast<uint8_t*>(active);
  h.R_cur = h.Rinit = rg * kMsb;
  h.R_prev = 0;
  h.seed = seed;
  h.iseq = iseq;
  h.step = 1;
  h.pop_id = step;
  h.E = E;
  h.M = M;
  h.betas = S.betas;
  h.thr = S.thr;
  double b[2] = {0.0, beta};
  uint32_t t[2 * kThrPerStep];
  fill_thr(0.0, t);
  fill_thr(beta, t + kThrPerStep);
  int rc = upload_and_sync(S, h, b, t, s);
  if (rc) return rc;
  if ((e = launch_msc_sweep(S.st, g, rng_mode, sweeps, s)) != cudaSuccess) return stage_fail(e, "msc_sweep");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "msc_sweep");
  return PA_OK;
}

int pa_resample_plan(const int32_t* E, const uint8_t* active, int coding, int R_prev, int Rinit, int Rcap,
                     double beta_prev, double beta, double e_ref, int weights, uint64_t seed, uint64_t iseq,
                     uint32_t* roff, uint32_t* offs, uint32_t* src, double* out, void* stream) {
  if (!E || !roff || !offs || !src || !out || R_prev < 1 || Rinit < 1 || Rcap < 1) return PA_ERR_ARG;
  if (coding != PA_CODING_SSC && coding != PA_CODING_MSC) return PA_ERR_ARG;
  if (coding == PA_CODING_MSC && !active) return PA_ERR_ARG;
  if (weights != PA_WEIGHTS_FP32 && weights != PA_WEIGHTS_FP64) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(coding, 8);
  h.Rinit = Rinit;
  h.Rcap = Rcap;
  h.rgcap = (Rcap + kMsb - 1) / kMsb;
  h.R_prev = R_prev;
  h.R_cur = R_prev;
  h.step = 1;
  h.weights = weights;
  h.seed = seed;
  h.iseq = iseq;
  h.Emean = e_ref;
  h.Emin = (int)e_ref;
  h.E = const_cast<int32_t*>(E);
  h.active[0] = h.active[1] = const_cast<uint8_t*>(active);
  h.roff = roff;
  h.offs = offs;
  h.src = src;
  h.blk_tot = S.blk;
  h.blk_off = S.blk + kResBlocksMax;
  h.qpart_d = S.qd;
  h.qpart_f = S.qf;
  h.betas = S.betas;
  const long long units = coding == PA_CODING_MSC ? (long long)((R_prev + kMsb - 1) / kMsb) * kMsb : R_prev;
  // launch geometry follows the population that is resampled
  PopDev g = h;
  g.Rcap = (int)units;
  g.rgcap = (int)(units / kMsb + 1);
  double b[2] = {beta_prev, beta};
  int rc = upload_and_sync(S, h, b, nullptr, s);
  if (rc) return rc;
  if ((e = launch_q(S.st, g, s)) != cudaSuccess) return stage_fail(e, "q");
  if ((e = launch_copy_numbers(S.st, g, s)) != cudaSuccess) return stage_fail(e, "copy numbers");
  if ((e = launch_scatter(S.st, g, s)) != cudaSuccess) return stage_fail(e, "scatter");
  PopDev back;
  if ((e = cudaMemcpyAsync(&back, S.st, sizeof(PopDev), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return stage_fail(e, "readback");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "resample plan");
  out[0] = back.lnQ;
  out[1] = back.q;
  out[2] = back.error ? 0.0 : (double)back.R_cur;
  if (back.error == 1) return PA_ERR_CAPACITY;
  if (back.error == 2) return PA_ERR_EXTINCT;
  return PA_OK;
}

int pa_ssc_resample(const int8_t* old_spins, int L, const uint32_t* src, int R_new, int8_t* new_spins, void* stream) {
  SweepGeom g;
  if (!old_spins || !src || !new_spins || R_new < 1 || !ssc_geom(L, 256, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kSSC, L);
  h.spins[0] = new_spins;
  h.spins[1] = const_cast<int8_t*>(old_spins);
  h.R_cur = R_new;
  h.src = const_cast<uint32_t*>(src);
  int rc = upload_and_sync(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  if ((e = launch_ssc_resample(S.st, h, s)) != cudaSuccess) return stage_fail(e, "ssc_resample");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "ssc_resample");
  return PA_OK;
}

int pa_msc_resample(const uint32_t* old_words, int L, const uint32_t* src, int R_new, uint32_t* new_words,
                    uint8_t* new_active, void* stream) {
  SweepGeom g;
  if (!old_words || !src || !new_words || !new_active || R_new < 1 || !msc_geom(L, 256, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kMSC, L);
  h.spins[0] = new_words;
  h.spins[1] = const_cast<uint32_t*>(old_words);
  h.active[0] = new_active;
  h.R_cur = R_new;
  h.src = const_cast<uint32_t*>(src);
  int rc = upload_and_sync(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  if ((e = launch_msc_resample(S.st, h, s)) != cudaSuccess) return stage_fail(e, "msc_resample");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return stage_fail(e, "msc_resample");
  return PA_OK;
}

}  // extern "C"
