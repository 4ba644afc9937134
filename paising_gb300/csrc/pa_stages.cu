// pa_stages.cu -- stage entry points of the C ABI: one reference kernel (or
// kernel group) each, on caller-owned device buffers.  They run the same
// kernels as the engine on a batch of one population whose PopDev describes
// the caller's buffers; that descriptor and the reductions' partial sums live
// in scratch device memory allocated for the duration of the call.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "../../include/paising.h"
#include "pa_device.cuh"
#include "pa_error.h"
#include "pa_kernels.h"
#include "pa_thresholds.h"

using namespace pa;

namespace {

int stage_fail(cudaError_t e, const char* what) {
  pa::g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return PA_ERR_CUDA;
}

// Device scratch of one stage call.
struct Scratch {
  BatchDev* b = nullptr;
  PopDev* st = nullptr;
  double* betas = nullptr;
  uint32_t* thr = nullptr;
  uint32_t* blk = nullptr;  // blk_tot | blk_off
  double* qd = nullptr;
  float* qf = nullptr;
  void* base = nullptr;
  cudaError_t alloc() {
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_st = up(sizeof(BatchDev)), o_b = o_st + up(sizeof(PopDev)), o_t = o_b + 256,
                 o_k = o_t + up(2 * kThrPerStep * 4), o_qd = o_k + up(2 * kResBlocksMax * 4),
                 o_qf = o_qd + up(kResBlocksMax * 8), sz = o_qf + up(2 * kResBlocksMax * 4);
    cudaError_t e = cudaMalloc(&base, sz);
    if (e != cudaSuccess) return e;
    char* p = (char*)base;
    b = (BatchDev*)p;
    st = (PopDev*)(p + o_st);
    betas = (double*)(p + o_b);
    thr = (uint32_t*)(p + o_t);
    blk = (uint32_t*)(p + o_k);
    qd = (double*)(p + o_qd);
    qf = (float*)(p + o_qf);
    return cudaSuccess;
  }
  ~Scratch() {
    if (base) cudaFree(base);
  }
};

void fill_thr(double beta, uint32_t* t) { thresholds(beta, t); }

// A one-population state at temperature step 1 of a one-step schedule.
PopDev base_state(int coding, int L) {
  PopDev h;
  std::memset(&h, 0, sizeof(h));
  h.coding = coding;
  h.L = L;
  h.N = L * L;
  h.step = 1;
  h.nsteps = 1;
  h.Emin_acc = 0x7fffffff;
  SweepGeom g;
  if (coding == kMSC ? msc_geom(L, &g) : ssc_geom(L, &g)) geom_to_pop(g, &h);
  return h;
}

int upload(Scratch& S, const PopDev& h, const double* betas, const uint32_t* thr, cudaStream_t s) {
  BatchDev bd;
  std::memset(&bd, 0, sizeof(bd));
  bd.npop = 1;
  bd.pops = S.st;
  cudaError_t e = cudaMemcpyAsync(S.st, &h, sizeof(PopDev), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.b, &bd, sizeof(bd), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && betas) e = cudaMemcpyAsync(S.betas, betas, 2 * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && thr) e = cudaMemcpyAsync(S.thr, thr, 2 * kThrPerStep * 4, cudaMemcpyHostToDevice, s);
  return e == cudaSuccess ? PA_OK : stage_fail(e, "upload");
}

int finish(cudaError_t e, cudaStream_t s, const char* what) {
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? PA_OK : stage_fail(e, what);
}

// bits: the SSC bit-plane sweep (native stream only)
int sweep_stage(int coding, void* spins, uint8_t* active, int L, int units, int sweeps, double beta, int rng_mode,
                uint64_t seed, uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream, bool bits = false) {
  cudaStream_t s = (cudaStream_t)stream;
  SweepGeom g;
  if (bits ? !ssc_bits_geom(L, &g) : coding == kMSC ? !msc_geom(L, &g) : !ssc_geom(L, &g)) return PA_ERR_ARG;
  SweepLaunch sl;
  cudaError_t e = bits ? ssc_bits_setup(g.smem, &sl)
                       : sweep_setup(coding, rng_mode, g.smem, &sl,
                                     coding == kMSC && rng_mode == PA_RNG_NATIVE ? msc_fixed_l(g.L, g.G) : 0);
  if (e != cudaSuccess) return stage_fail(e, "sweep setup");
  Scratch S;
  if ((e = S.alloc()) != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(coding, L);
  h.spins[0] = spins;
  h.active[0] = active;
  h.R_cur = h.Rinit = coding == kMSC ? units * kMsb : units;
  h.sweeps = sweeps;
  h.rng_mode = rng_mode;
  h.seed = seed;
  h.iseq = iseq;
  h.pop_id = step;  // native stream key: the stage call folds (step, population) into pop_id
  h.E = E;
  h.M = M;
  h.betas = S.betas;
  h.thr = S.thr;
  double b[2] = {0.0, beta};
  uint32_t t[2 * kThrPerStep];
  fill_thr(0.0, t);
  fill_thr(beta, t + kThrPerStep);
  if (bits) geom_to_pop(g, &h);
  int rc = upload(S, h, b, t, s);
  if (rc) return rc;
  e = launch_plan(S.b, 1, 0, s);
  if (e == cudaSuccess)
    e = bits ? launch_ssc_bits_sweep(S.b, 0, seed, sl, s) : launch_sweep(S.b, coding, rng_mode, 0, seed, sl, s);
  return finish(e, s, "sweep");
}

}  // namespace

extern "C" {

int pa_ssc_init(int8_t* spins, int L, int R, uint64_t seed, uint64_t iseq, void* stream) {
  SweepGeom g;
  if (!spins || R < 1 || !ssc_geom(L, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kSSC, L);
  h.spins[0] = spins;
  h.R_cur = h.Rinit = R;
  h.seed = seed;
  h.iseq = iseq;
  int rc = upload(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  return finish(launch_init(S.st, 1, kSSC, s), s, "ssc_init");
}

int pa_ssc_sweep(int8_t* spins, int L, int R, int sweeps, double beta, int rng_mode, uint64_t seed,
                 uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream) {
  SweepGeom g;
  if (!spins || !E || !M || R < 1 || sweeps < 0 || step < 0 || !ssc_geom(L, &g)) return PA_ERR_ARG;
  if (rng_mode != PA_RNG_NATIVE && rng_mode != PA_RNG_REFERENCE) return PA_ERR_ARG;
  return sweep_stage(kSSC, spins, nullptr, L, R, sweeps, beta, rng_mode, seed, iseq, step, E, M, stream);
}

int pa_ssc_sweep_bits(int8_t* spins, int L, int R, int sweeps, double beta, uint64_t seed, int step, int32_t* E,
                      int32_t* M, void* stream) {
  SweepGeom g;
  if (!spins || !E || !M || R < 1 || sweeps < 0 || step < 0 || !ssc_bits_geom(L, &g)) return PA_ERR_ARG;
  return sweep_stage(kSSC, spins, nullptr, L, R, sweeps, beta, PA_RNG_NATIVE, seed, 0, step, E, M, stream, true);
}

int pa_msc_init(uint32_t* words, uint8_t* active, int L, int R, uint64_t seed, uint64_t iseq, void* stream) {
  SweepGeom g;
  if (!words || !active || R < 1 || !msc_geom(L, &g)) return PA_ERR_ARG;
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
  int rc = upload(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  return finish(launch_init(S.st, 1, kMSC, s), s, "msc_init");
}

int pa_msc_sweep(uint32_t* words, const uint8_t* active, int L, int rg, int sweeps, double beta, int rng_mode,
                 uint64_t seed, uint64_t iseq, int step, int32_t* E, int32_t* M, void* stream) {
  SweepGeom g;
  if (!words || !active || !E || !M || rg < 1 || sweeps < 0 || step < 0 || !msc_geom(L, &g)) return PA_ERR_ARG;
  if (rng_mode != PA_RNG_NATIVE && rng_mode != PA_RNG_REFERENCE) return PA_ERR_ARG;
  return sweep_stage(kMSC, words, const_cast<uint8_t*>(active), L, rg, sweeps, beta, rng_mode, seed, iseq, step, E,
                     M, stream);
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
  const int blocks = res_blocks(units);
  double b[2] = {beta_prev, beta};
  int rc = upload(S, h, b, nullptr, s);
  if (rc) return rc;
  if ((e = launch_q(S.st, 1, blocks, s)) != cudaSuccess) return stage_fail(e, "q");
  if ((e = launch_copy_numbers(S.st, 1, blocks, s)) != cudaSuccess) return stage_fail(e, "copy numbers");
  if ((e = launch_scatter(S.st, 1, blocks, s)) != cudaSuccess) return stage_fail(e, "scatter");
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
  if (!old_spins || !src || !new_spins || R_new < 1 || !ssc_geom(L, &g)) return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  PopDev h = base_state(kSSC, L);
  h.spins[0] = new_spins;
  h.spins[1] = const_cast<int8_t*>(old_spins);
  h.R_cur = R_new;
  h.src = const_cast<uint32_t*>(src);
  int rc = upload(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  return finish(launch_resample(S.b, kSSC, kRefCoords, s), s, "ssc_resample");
}

int pa_msc_resample(const uint32_t* old_words, int L, const uint32_t* src, int R_new, uint32_t* new_words,
                    uint8_t* new_active, void* stream) {
  SweepGeom g;
  if (!old_words || !src || !new_words || !new_active || R_new < 1 || !msc_geom(L, &g)) return PA_ERR_ARG;
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
  int rc = upload(S, h, nullptr, nullptr, s);
  if (rc) return rc;
  return finish(launch_resample(S.b, kMSC, kRefCoords, s), s, "msc_resample");
}

int pa_msc_resample_native(const uint32_t* old_words, int L, int R_old, const uint32_t* src, int R_new,
                           uint32_t* new_words, uint8_t* new_active, void* stream) {
  SweepGeom g;
  (void)g;
  if (!old_words || !src || !new_words || !new_active || R_old < 1 || R_new < 1 || L < 4 || L % 2 || L > 256)
    return PA_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Scratch S;
  cudaError_t e = S.alloc();
  if (e != cudaSuccess) return stage_fail(e, "scratch");
  const int rg_new = (R_new + kMsb - 1) / kMsb;
  void* pairs = nullptr;  // pair lists and counts of the new groups
  e = cudaMalloc(&pairs, (size_t)rg_new * (kMsb * sizeof(uint2) + sizeof(uint32_t)));
  if (e != cudaSuccess) return stage_fail(e, "pair scratch");
  PopDev h = base_state(kMSC, L);
  h.rng_mode = kNative;
  h.spins[0] = new_words;
  h.spins[1] = const_cast<uint32_t*>(old_words);
  h.active[0] = new_active;
  h.rgcap = (R_old + kMsb - 1) / kMsb;  // groups the old buffer holds
  h.R_cur = R_new;
  h.src = const_cast<uint32_t*>(src);
  h.res_pairs = static_cast<uint2*>(pairs);
  h.res_cnt = reinterpret_cast<uint32_t*>(static_cast<uint2*>(pairs) + (size_t)rg_new * kMsb);
  int rc = upload(S, h, nullptr, nullptr, s);
  if (rc == PA_OK) rc = finish(launch_resample(S.b, kMSC, kNative, s), s, "msc_resample_native");
  cudaFree(pairs);
  return rc;
}

}  // extern "C"
