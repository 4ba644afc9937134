// pa_engine.cu -- host driver of the population-annealing engine and the C
// ABI declared in include/paising.h.
//
// One handle = one population configuration on one GPU.  The temperature
// loop of the reference's main() (PAisingSSC.cu:481-664) becomes, per step,
//   q -> copy numbers -> scatter -> resample -> sweep(+energy) -> finish
// launched on the handle's stream with every size read from device memory.
// In graph mode the whole run (initialisation + all temperatures) is
// captured once and replayed as a single CUDA graph launch per run; in plain
// mode the host launches each step and synchronises after it, reading the
// step's output row like the reference's host loop reads its averages.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/paising.h"
#include "pa_device.cuh"
#include "pa_error.h"
#include "pa_kernels.h"

using namespace pa;

namespace {

struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 16);
    if (e == cudaSuccess) {
      ptrs.push_back(q);
      *p = (T*)q;
    }
    return e;
  }
};

constexpr int kNBmax = 10000;  // nBmax, PAisingSSC.cu:57

double ceil_thr(double p) { return std::ceil(4294967296.0 * p); }

// per-temperature acceptance thresholds (host exp, like the reference)
void thresholds(double beta, uint32_t* t) {
  // SSC Boltzmann table boltz[idxT0 + 2 idxT1] = min(1, exp(-2 s sum_nn beta))
  // (PAisingSSC.cu:512-516); a reference uniform (H+1)/2^32 is below p iff
  // H < ceil(2^32 p) - 1.
  for (int i0 = 0; i0 <= 1; ++i0)
    for (int i1 = 0; i1 <= 4; ++i1) {
      double p = std::exp(-2 * (2 * i0 - 1) * (2 * i1 - 4) * beta);
      if (p > 1.0) p = 1.0;
      t[i0 + 2 * i1] = (uint32_t)(ceil_thr(p) - 1.0);
    }
  // MSC integer thresholds (PAisingMSC.cu:674-675), also the native SSC ones
  const double t4 = ceil_thr(std::exp(-4 * beta)), t8 = ceil_thr(std::exp(-8 * beta));
  t[10] = t4 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t4;
  t[11] = t8 >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t8;
}

std::vector<double> schedule(double dbeta, double bfin) {
  std::vector<double> b{0.0};
  double x = b[0] + dbeta;  // B[i] = B[iprev] + deltaBeta (PAisingSSC.cu:508,661)
  while (x <= bfin && (int)b.size() < kNBmax + 1) {
    b.push_back(x);
    x = b.back() + dbeta;
  }
  return b;
}

}  // namespace

struct pa_handle {
  pa_config cfg{};
  PopDev h{};
  PopDev* d = nullptr;
  SweepGeom geom{};
  DevBuf buf;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<double> betas;
  std::vector<uint32_t> thr;
  int nsteps = 0;
  std::vector<double> rows;  // runs * (nsteps + 1) * 10
  int runs_done = 0;
  double ms = 0.0, attempts = 0.0;
  std::string err;
  void* staging = nullptr;  // device copy of a caller-supplied initial population

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return PA_ERR_CUDA;
  }

  // Optional per-kernel timing (pa_profile_run): CUDA events around every
  // launch on the handle's stream, synchronised per launch.
  struct Prof {
    cudaEvent_t a = nullptr, b = nullptr;
    std::vector<std::pair<std::string, std::pair<int, double>>> acc;
    void add(const char* name, double ms) {
      for (auto& x : acc)
        if (x.first == name) { x.second.first++; x.second.second += ms; return; }
      acc.push_back({name, {1, ms}});
    }
  };
  Prof* prof = nullptr;

  template <class F>
  cudaError_t launch(const char* name, F f) {
    if (!prof) return f();
    cudaError_t e = cudaEventRecord(prof->a, stream);
    if (e == cudaSuccess) e = f();
    if (e == cudaSuccess) e = cudaEventRecord(prof->b, stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(prof->b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, prof->a, prof->b);
    if (e == cudaSuccess) prof->add(name, ms);
    return e;
  }

  cudaError_t enqueue_init() {
    cudaError_t e;
    const bool msc = cfg.coding == PA_CODING_MSC;
    if ((e = launch("begin_run", [&] { return launch_begin_run(d, stream); })) != cudaSuccess) return e;
    e = launch(msc ? "msc_init" : "ssc_init",
               [&] { return msc ? launch_msc_init(d, h, stream) : launch_ssc_init(d, h, stream); });
    if (e != cudaSuccess) return e;
    e = launch(msc ? "msc_energy" : "ssc_energy", [&] {
      return msc ? launch_msc_sweep(d, geom, cfg.rng_mode, 0, stream) : launch_ssc_sweep(d, geom, cfg.rng_mode, 0, stream);
    });
    if (e != cudaSuccess) return e;
    return launch("finish_step", [&] { return launch_finish_step(d, stream); });
  }

  cudaError_t enqueue_step() {
    cudaError_t e;
    const bool msc = cfg.coding == PA_CODING_MSC;
    if ((e = launch("q", [&] { return launch_q(d, h, stream); })) != cudaSuccess) return e;
    if ((e = launch("copy_numbers", [&] { return launch_copy_numbers(d, h, stream); })) != cudaSuccess) return e;
    if ((e = launch("scatter", [&] { return launch_scatter(d, h, stream); })) != cudaSuccess) return e;
    e = launch(msc ? "msc_resample" : "ssc_resample",
               [&] { return msc ? launch_msc_resample(d, h, stream) : launch_ssc_resample(d, h, stream); });
    if (e != cudaSuccess) return e;
    e = launch(msc ? "msc_sweep" : "ssc_sweep", [&] {
      return msc ? launch_msc_sweep(d, geom, cfg.rng_mode, cfg.sweeps, stream)
                 : launch_ssc_sweep(d, geom, cfg.rng_mode, cfg.sweeps, stream);
    });
    if (e != cudaSuccess) return e;
    return launch("finish_step", [&] { return launch_finish_step(d, stream); });
  }

  ~pa_handle() {
    if (staging) cudaFree(staging);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int pa_abi_version(void) { return PA_ABI_VERSION; }

int pa_schedule(double dbeta, double beta_final, double* betas, int max, int* n) {
  if (!(dbeta > 0) || !(beta_final > 0) || max < 0 || (max > 0 && !betas)) return PA_ERR_ARG;
  const std::vector<double> b = schedule(dbeta, beta_final);
  for (int i = 0; i < max && i < (int)b.size(); ++i) betas[i] = b[i];
  if (n) *n = (int)b.size();
  return (int)b.size() > kNBmax - 1 ? PA_ERR_TOO_MANY_STEPS : PA_OK;
}

uint32_t pa_ref_word(uint64_t seed, uint64_t subseq, uint64_t ctr) { return ref_word(seed, subseq, ctr); }

const char* pa_status_string(int s) {
  switch (s) {
    case PA_OK: return "ok";
    case PA_ERR_ARG: return "invalid argument";
    case PA_ERR_CUDA: return "CUDA error";
    case PA_ERR_CAPACITY: return "population exceeded its buffer capacity";
    case PA_ERR_EXTINCT: return "population became empty";
    case PA_ERR_STATE: return "call out of order";
    case PA_ERR_TOO_MANY_STEPS: return "number of temperature steps exceeds nBmax=10000";
    default: return "unknown status";
  }
}

const char* pa_last_error(const pa_handle* h) { return h ? h->err.c_str() : pa::g_last_error.c_str(); }

int pa_config_init(pa_config* c) {
  if (!c) return PA_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  c->L = 64;
  c->R = 20000;
  c->sweeps = 100;
  c->dbeta = 0.005;
  c->beta_final = 1.0;
  c->runs = 1;
  c->seed = 1;
  c->coding = PA_CODING_SSC;
  c->rng_mode = PA_RNG_NATIVE;
  c->weights = PA_WEIGHTS_FP32;
  c->graph = 1;
  c->device = 0;
  c->capacity = 1.25;
  return PA_OK;
}

int pa_create(const pa_config* cfg, pa_handle** out) {
  if (!cfg || !out) return PA_ERR_ARG;
  *out = nullptr;
  pa_handle* H = new (std::nothrow) pa_handle();
  if (!H) return PA_ERR_ARG;
  H->cfg = *cfg;
  pa_config& c = H->cfg;
  auto bad = [&](const char* m) {
    pa::g_last_error = m;
    delete H;
    return PA_ERR_ARG;
  };
  if (c.coding != PA_CODING_SSC && c.coding != PA_CODING_MSC) return bad("coding must be SSC or MSC");
  if (c.rng_mode != PA_RNG_NATIVE && c.rng_mode != PA_RNG_REFERENCE) return bad("bad rng_mode");
  if (c.weights != PA_WEIGHTS_FP32 && c.weights != PA_WEIGHTS_FP64) return bad("bad weights");
  if (c.R < 1 || c.sweeps < 0 || c.runs < 1 || !(c.dbeta > 0) || !(c.beta_final > 0)) return bad("R, sweeps, runs, dbeta, beta_final out of range");
  if (c.capacity <= 0) c.capacity = 1.25;
  if (c.capacity < 1.0) return bad("capacity must be >= 1");
  bool okg = c.coding == PA_CODING_MSC ? msc_geom(c.L, 256, &H->geom) : ssc_geom(c.L, 256, &H->geom);
  if (!okg) return bad(c.coding == PA_CODING_MSC ? "MSC needs even L in [8, 128]" : "SSC needs L % 8 == 0, 8 <= L <= 256");

  H->betas = schedule(c.dbeta, c.beta_final);
  H->nsteps = (int)H->betas.size() - 1;
  if ((int)H->betas.size() > kNBmax - 1) {
    pa::g_last_error = "number of temperature steps exceeds nBmax=10000";
    delete H;
    return PA_ERR_TOO_MANY_STEPS;
  }
  H->thr.assign(H->betas.size() * kThrPerStep, 0u);
  for (size_t i = 0; i < H->betas.size(); ++i) thresholds(H->betas[i], &H->thr[i * kThrPerStep]);

  cudaError_t e = cudaSetDevice(c.device);
  if (e != cudaSuccess) { pa::g_last_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e); delete H; return PA_ERR_CUDA; }
  e = c.coding == PA_CODING_MSC ? msc_sweep_setup(&H->geom, c.rng_mode) : ssc_sweep_setup(&H->geom, c.rng_mode);
  if (e != cudaSuccess) { pa::g_last_error = std::string("sweep setup: ") + cudaGetErrorString(e); delete H; return PA_ERR_CUDA; }

  PopDev& h = H->h;
  const int L = c.L, N = L * L;
  const long long Rcap = (long long)std::ceil(c.capacity * c.R) + 256;
  const long long rgcap = (Rcap + kMsb - 1) / kMsb;
  if (Rcap * (long long)(c.coding == PA_CODING_MSC ? 4 : 1) * N > (1ll << 40)) return bad("population too large");
  h.L = L;
  h.N = N;
  h.coding = c.coding;
  h.Rinit = c.R;
  h.Rcap = (int)Rcap;
  h.rgcap = (int)rgcap;
  h.sweeps = c.sweeps;
  h.rng_mode = c.rng_mode;
  h.weights = c.weights;
  h.pop_id = 0;
  h.nsteps = H->nsteps;
  h.seed = c.seed;
  h.bf0 = -N * std::log(2.0);
  const size_t units = c.coding == PA_CODING_MSC ? (size_t)rgcap * kMsb : (size_t)Rcap;
  DevBuf& B = H->buf;
  auto chk = [&](cudaError_t err, const char* what) { if (err != cudaSuccess && e == cudaSuccess) { e = err; H->err = what; } };
  if (c.coding == PA_CODING_MSC) {
    uint32_t *a, *b;
    chk(B.alloc(&a, (size_t)rgcap * N), "spins");
    chk(B.alloc(&b, (size_t)rgcap * N), "spins");
    h.spins[0] = a;
    h.spins[1] = b;
    chk(B.alloc(&h.active[0], units), "active");
    chk(B.alloc(&h.active[1], units), "active");
  } else {
    int8_t *a, *b;
    chk(B.alloc(&a, (size_t)Rcap * N), "spins");
    chk(B.alloc(&b, (size_t)Rcap * N), "spins");
    h.spins[0] = a;
    h.spins[1] = b;
    h.active[0] = h.active[1] = nullptr;
  }
  chk(B.alloc(&h.E, units), "E");
  chk(B.alloc(&h.M, units), "M");
  chk(B.alloc(&h.roff, units), "roff");
  chk(B.alloc(&h.offs, units), "offs");
  chk(B.alloc(&h.src, (size_t)Rcap), "src");
  chk(B.alloc(&h.blk_tot, kResBlocksMax), "scratch");
  chk(B.alloc(&h.blk_off, kResBlocksMax), "scratch");
  chk(B.alloc(&h.qpart_d, kResBlocksMax), "scratch");
  chk(B.alloc(&h.qpart_f, 2 * kResBlocksMax), "scratch");
  double* rows;
  chk(B.alloc(&rows, H->betas.size() * kRowCols), "rows");
  h.rows = rows;
  double* bet;
  chk(B.alloc(&bet, H->betas.size()), "betas");
  h.betas = bet;
  uint32_t* th;
  chk(B.alloc(&th, H->thr.size()), "thresholds");
  h.thr = th;
  chk(B.alloc(&H->d, 1), "state");
  if (e != cudaSuccess) {
    pa::g_last_error = std::string("cudaMalloc (") + H->err + "): " + cudaGetErrorString(e);
    delete H;
    return PA_ERR_CUDA;
  }
  h.iseq = 0;  // initial_sequence = 0 (PAisingSSC.cu:418), continues across runs
  chk(cudaMemcpy(bet, H->betas.data(), H->betas.size() * sizeof(double), cudaMemcpyHostToDevice), "betas");
  chk(cudaMemcpy(th, H->thr.data(), H->thr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "thr");
  chk(cudaMemcpy(H->d, &h, sizeof(PopDev), cudaMemcpyHostToDevice), "state");
  chk(cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking), "stream");
  chk(cudaEventCreate(&H->ev0), "event");
  chk(cudaEventCreate(&H->ev1), "event");
  if (e == cudaSuccess && c.graph) {
    chk(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal), "capture");
    if (e == cudaSuccess) {
      cudaError_t e1 = H->enqueue_init();
      for (int i = 1; i <= H->nsteps && e1 == cudaSuccess; ++i) e1 = H->enqueue_step();
      cudaError_t e2 = cudaStreamEndCapture(H->stream, &H->graph);
      chk(e1, "capture launches");
      chk(e2, "end capture");
      if (e == cudaSuccess) chk(cudaGraphInstantiate(&H->exec, H->graph, 0), "graph instantiate");
    }
  }
  if (e != cudaSuccess) {
    pa::g_last_error = std::string(H->err) + ": " + cudaGetErrorString(e);
    delete H;
    return PA_ERR_CUDA;
  }
  *out = H;
  return PA_OK;
}

int pa_run(pa_handle* H) {
  if (!H) return PA_ERR_ARG;
  const pa_config& c = H->cfg;
  const size_t nrow = H->betas.size();
  H->rows.assign((size_t)c.runs * nrow * kRowCols, 0.0);
  H->runs_done = 0;
  H->attempts = 0;
  cudaError_t e = cudaEventRecord(H->ev0, H->stream);
  if (e != cudaSuccess) return H->cuda_fail(e, "event");
  int status = PA_OK;
  for (int r = 0; r < c.runs && status == PA_OK; ++r) {
    if (c.graph) {
      e = cudaGraphLaunch(H->exec, H->stream);
      if (e != cudaSuccess) return H->cuda_fail(e, "graph launch");
    } else {
      e = H->enqueue_init();
      if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
      for (int i = 1; i <= H->nsteps && e == cudaSuccess; ++i) {
        e = H->enqueue_step();
        if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
        double row[kRowCols];
        if (e == cudaSuccess)
          e = cudaMemcpy(row, H->h.rows + (size_t)i * kRowCols, sizeof(row), cudaMemcpyDeviceToHost);
      }
      if (e != cudaSuccess) return H->cuda_fail(e, "plain step");
    }
    double* dst = H->rows.data() + (size_t)r * nrow * kRowCols;
    e = cudaMemcpyAsync(dst, H->h.rows, nrow * kRowCols * sizeof(double), cudaMemcpyDeviceToHost, H->stream);
    int err_flag = 0;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&err_flag, &H->d->error, sizeof(int), cudaMemcpyDeviceToHost, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return H->cuda_fail(e, "run");
    if (err_flag) {
      status = err_flag == 2 ? PA_ERR_EXTINCT : PA_ERR_CAPACITY;
      H->err = err_flag == 2 ? "resampling produced an empty population"
                             : "population exceeded its buffer capacity (raise pa_config.capacity)";
      break;
    }
    for (size_t i = 1; i < nrow; ++i) H->attempts += (double)c.sweeps * (double)H->h.N * dst[i * kRowCols + 8];
    H->runs_done = r + 1;
  }
  e = cudaEventRecord(H->ev1, H->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(H->ev1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, H->ev0, H->ev1);
  if (e != cudaSuccess) return H->cuda_fail(e, "timing");
  H->ms = ms;
  return status;
}

static size_t population_bytes(const pa_config& c, int R) {
  const size_t N = (size_t)c.L * c.L;
  return c.coding == PA_CODING_MSC ? (size_t)((R + kMsb - 1) / kMsb) * N * 4 : (size_t)R * N;
}

int pa_set_population(pa_handle* H, const void* host) {
  if (!H) return PA_ERR_ARG;
  cudaError_t e = cudaSuccess;
  const void* dev = nullptr;
  if (host) {
    const size_t bytes = population_bytes(H->cfg, H->cfg.R);
    if (!H->staging) e = cudaMalloc(&H->staging, bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(H->staging, host, bytes, cudaMemcpyHostToDevice, H->stream);
    dev = H->staging;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&H->d->init_src, &dev, sizeof(dev), cudaMemcpyHostToDevice, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);  // `dev` lives on this stack frame
  if (e != cudaSuccess) return H->cuda_fail(e, "set population");
  H->h.init_src = dev;
  return PA_OK;
}

int pa_get_population(const pa_handle* H, void* host, size_t bytes, int* R) {
  if (!H || !host) return PA_ERR_ARG;
  if (H->runs_done == 0) return PA_ERR_STATE;
  PopDev st;
  cudaError_t e = cudaMemcpy(&st, H->d, sizeof(PopDev), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return PA_ERR_CUDA;
  const size_t need = population_bytes(H->cfg, st.R_cur);
  if (R) *R = st.R_cur;
  if (bytes < need) return PA_ERR_ARG;
  e = cudaMemcpy(host, st.spins[st.parity], need, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

int pa_profile_run(pa_handle* H, pa_kernel_time* out, int max, int* n) {
  if (!H || (max > 0 && !out)) return PA_ERR_ARG;
  pa_handle::Prof P;
  cudaError_t e = cudaEventCreate(&P.a);
  if (e == cudaSuccess) e = cudaEventCreate(&P.b);
  H->prof = &P;
  if (e == cudaSuccess) e = H->enqueue_init();
  for (int i = 1; i <= H->nsteps && e == cudaSuccess; ++i) e = H->enqueue_step();
  H->prof = nullptr;
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (P.a) cudaEventDestroy(P.a);
  if (P.b) cudaEventDestroy(P.b);
  if (e != cudaSuccess) return H->cuda_fail(e, "profile run");
  int k = 0;
  for (auto& x : P.acc) {
    if (k < max) {
      std::snprintf(out[k].name, sizeof(out[k].name), "%s", x.first.c_str());
      out[k].launches = x.second.first;
      out[k].total_ms = x.second.second;
    }
    ++k;
  }
  if (n) *n = k;
  return PA_OK;
}

int pa_num_rows(const pa_handle* H, int* n) {
  if (!H || !n) return PA_ERR_ARG;
  *n = (int)H->betas.size();
  return PA_OK;
}

int pa_get_rows(const pa_handle* H, int run, pa_row* rows, int max_rows, int* nrows) {
  if (!H || !rows) return PA_ERR_ARG;
  if (run < 0 || run >= H->runs_done) return PA_ERR_STATE;
  const int n = (int)H->betas.size();
  const int m = n < max_rows ? n : max_rows;
  const double* src = H->rows.data() + (size_t)run * n * kRowCols;
  for (int i = 0; i < m; ++i) std::memcpy(&rows[i], src + (size_t)i * kRowCols, sizeof(pa_row));
  if (nrows) *nrows = m;
  return PA_OK;
}

int pa_get_timing(const pa_handle* H, double* ms, double* attempts) {
  if (!H) return PA_ERR_ARG;
  if (ms) *ms = H->ms;
  if (attempts) *attempts = H->attempts;
  return PA_OK;
}

int pa_write_results(const pa_handle* H, const char* dir, int precision) {
  if (!H || !dir) return PA_ERR_ARG;
  if (H->runs_done == 0) return PA_ERR_STATE;
  const int n = (int)H->betas.size();
  for (int r = 0; r < H->runs_done; ++r) {
    std::string path = std::string(dir);
    if (!path.empty() && path.back() != '/') path += '/';
    path += "PA_results_run_" + std::to_string(r) + ".dat";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return PA_ERR_ARG;
    const double* o = H->rows.data() + (size_t)r * n * kRowCols;
    for (int i = 0; i < n; ++i) {
      const double* w = o + (size_t)i * kRowCols;
      for (int k = 0; k < 8; ++k) std::fprintf(f, "%.*g ", precision, w[k]);
      std::fprintf(f, "%d %.*g\n", (int)w[8], precision, w[9]);
    }
    std::fclose(f);
  }
  return PA_OK;
}

int pa_destroy(pa_handle* H) {
  delete H;
  return PA_OK;
}

}  // extern "C"
