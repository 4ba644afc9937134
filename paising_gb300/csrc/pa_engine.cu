// pa_engine.cu -- host driver of the population-annealing engine and the C
// ABI declared in include/paising.h.
//
// A handle holds a batch of populations on one GPU (one population for a
// plain run; several identical ones for concurrent independent runs; uneven
// ones from pa_create_batch).  The temperature loop of the reference's main()
// (PAisingSSC.cu:481-664) becomes, per temperature step of the batch,
//   q -> copy numbers -> scatter -> resample -> plan -> sweep(+energy) -> finish
// with every population handled by the same launches and every size read
// from device memory.  In graph mode a whole run of the batch is captured
// once and replayed as one CUDA graph launch; in plain mode the host launches
// each step and synchronises after it, reading the step's rows like the
// reference's host loop reads its averages.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/paising.h"
#include "pa_device.cuh"
#include "pa_error.h"
#include "pa_kernels.h"
#include "pa_thresholds.h"

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

constexpr double kMinOverlap = 0.85, kMaxOverlap = 0.87;  // PAisingSSC.cu:42-43

std::vector<double> schedule(double dbeta, double bfin) {
  std::vector<double> b{0.0};
  double x = b[0] + dbeta;  // B[i] = B[iprev] + deltaBeta (PAisingSSC.cu:508,661)
  while (x <= bfin && (int)b.size() < kNBmax + 1) {
    b.push_back(x);
    x = b.back() + dbeta;
  }
  return b;
}

// Multi-histogram reweighting of one run: the single-iteration estimate the
// reference's MHR build writes (PAisingSSC.cu:694-767 with MHR_Niter = 1),
// written from the weighted-histogram equations.  Population i (inverse
// temperature b_i, R_i replicas, free energy f_i = betaF_i, Z_i = e^{-f_i})
// samples energy level E with probability Omega(E) e^{-b_i E} / Z_i, so the
// pooled histogram H(E) of all temperatures estimates
//     Omega(E) = H(E) / D(E),   D(E) = sum_i R_i e^{f_i - b_i E},
// and at every b_j the reweighted ensemble is Omega(E) e^{-b_j E}:
//     Z_j = sum_E Omega e^{-b_j E},  <E>_j,  C_j = b_j^2 var_j(E),
//     betaF_j = -ln Z_j.
// Logarithms of sums are taken relative to their largest exponent.  The f_i
// are recomputed from the rows' lnQ column in the order the reference
// accumulates them (f_i = -N ln 2 + sum_{j<=i} -lnQ_j); every sum runs over
// temperatures and energy levels in ascending order.  Returns 4 doubles per
// temperature: beta, E/N, C/N, betaF/N.
std::vector<double> mhr_analysis(int N, const std::vector<double>& rows, const std::vector<unsigned long long>& hist) {
  const int nT = (int)(rows.size() / kRowCols);
  std::vector<double> beta(nT), f(nT), pop(nT);
  double acc = 0.0;
  for (int i = 0; i < nT; ++i) {
    const double* r = &rows[(size_t)i * kRowCols];
    beta[i] = r[0];
    pop[i] = r[8];
    if (i > 0) acc -= r[9];
    f[i] = -N * std::log(2.0) + acc;
  }
  // energy levels the anneal visited (the others carry no information)
  std::vector<int> level;
  std::vector<double> energy, ln_omega;
  for (int k = 0; k <= N; ++k) {
    if (hist[k] == 0) continue;
    const double E = 4.0 * k - 2.0 * N;
    double top = f[0] - beta[0] * E;
    for (int i = 1; i < nT; ++i) top = std::max(top, f[i] - beta[i] * E);
    double d = 0.0;  // D(E) e^{-top}
    for (int i = 0; i < nT; ++i) d += pop[i] * std::exp(f[i] - beta[i] * E - top);
    if (d == 0.0) continue;
    level.push_back(k);
    energy.push_back(E);
    ln_omega.push_back(std::log((double)hist[k]) - top - std::log(d));
  }
  const size_t nL = level.size();
  std::vector<double> out((size_t)nT * 4, 0.0), w(nL);
  for (int j = 0; j < nT; ++j) {
    double top = -HUGE_VAL;
    for (size_t l = 0; l < nL; ++l) top = std::max(top, ln_omega[l] - beta[j] * energy[l]);
    double z = 0.0, e1 = 0.0;  // Z_j e^{-top}, sum E Omega e^{-b_j E - top}
    for (size_t l = 0; l < nL; ++l) {
      w[l] = std::exp(ln_omega[l] - beta[j] * energy[l] - top);
      z += w[l];
    }
    for (size_t l = 0; l < nL; ++l) e1 += energy[l] * w[l];
    const double mean = e1 / z;
    double var = 0.0;
    for (size_t l = 0; l < nL; ++l) var += (energy[l] - mean) * (energy[l] - mean) * w[l];
    var /= z;
    out[(size_t)j * 4 + 0] = beta[j];
    out[(size_t)j * 4 + 1] = mean / N;
    out[(size_t)j * 4 + 2] = beta[j] * beta[j] * var / N;
    out[(size_t)j * 4 + 3] = -(top + std::log(z)) / N;
  }
  return out;
}

// Appends the population of temperature i to dir/PA_lattice_<i>.dat in the
// reference's LatticePopStore text (PAisingSSC.cu:580-605): a header line
// "i=..; beta=..; R=..;", then per replica "P={{..},{..},..};" with the L rows
// of the lattice in x order (A and B sites interleaved, A first on even rows),
// and an empty line.  MSC populations (no counterpart in the reference) list
// their active replicas group-major.  spins: the coding's layout; act: MSC
// active flags.
int write_lattice(const std::string& dir, int i, double beta, int precision, int coding, int L, int R,
                  const void* spins, const uint8_t* act, int units) {
  std::string path = dir;
  if (!path.empty() && path.back() != '/') path += '/';
  path += "PA_lattice_" + std::to_string(i) + ".dat";
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return PA_ERR_ARG;
  std::fprintf(f, "i=%d; beta=%.*g; R=%d;\n", i, precision, beta, R);
  const int N = L * L, h = N / 2, W = L / 2;
  std::vector<int> s(N);
  auto emit = [&]() {  // s: sublattice A then B, +-1
    std::string line = "P={";
    int ab = 0;
    for (int k = 0; k < h; ++k) {
      if (k % W == 0) {
        line += '{';
        ab = 1 - ab;
      }
      const int a = s[k], b = s[h + k];
      line += std::to_string(ab ? a : b) + "," + std::to_string(ab ? b : a);
      if ((k + 1) % W == 0) {
        line += '}';
        if (k + 1 < h) line += ',';
      } else {
        line += ',';
      }
    }
    line += "};\n";
    std::fputs(line.c_str(), f);
  };
  if (coding == PA_CODING_SSC) {
    const int8_t* p = (const int8_t*)spins;
    for (int j = 0; j < R; ++j) {
      for (int x = 0; x < N; ++x) s[x] = p[(size_t)j * N + x];
      emit();
    }
  } else {
    const uint32_t* w = (const uint32_t*)spins;
    for (int j = 0; j < units; ++j) {
      if (!act[j]) continue;
      const int g = j / 32, b = j % 32;
      for (int x = 0; x < N; ++x) s[x] = (w[(size_t)g * N + x] >> b) & 1u ? 1 : -1;
      emit();
    }
  }
  std::fputs("\n", f);
  std::fclose(f);
  return PA_OK;
}

size_t population_bytes(int coding, int L, int R) {
  const size_t N = (size_t)L * L;
  return coding == PA_CODING_MSC ? (size_t)((R + kMsb - 1) / kMsb) * N * 4 : (size_t)R * N;
}

// Host view of one population of a batch.
struct PopHost {
  pa_config cfg{};
  PopDev h{};
  SweepGeom geom{};
  std::vector<double> betas;  // the schedule (adaptive: its first two temperatures)
  std::vector<uint32_t> thr;
  int nsteps = 0;             // steps of the schedule (adaptive: the most the buffers allow)
  int cap = 0;                // rows the device buffers hold
  int user_index = 0;
};

}  // namespace

struct pa_handle {
  std::vector<PopHost> pops;  // device order: descending work per sweep unit
  int npop = 0;
  int coding = 0, rng_mode = 0, graph = 1, device = 0;
  int seq_runs = 1;  // sequential runs of a single population (reference stream, runs > 1)
  int max_steps = 0;
  int rblocks = 1;
  int cs = 1;  // CTAs per MSC group in the sweep (1, or a cluster of 2 / 4)
  int cthreads = 256;  // threads per CTA of a cluster (msc_cluster_threads)
  bool ssc_bits = false;  // SSC swept on bit planes (pa_ssc_bits.cu)
  bool adaptive = false;  // some population chooses its temperatures as it goes
  static constexpr int kChunk = 16;  // adaptive runs: steps per graph launch between host checks
  cudaGraph_t chunk_t = nullptr;
  cudaGraphExec_t chunk_exec = nullptr;
  unsigned long long stream_seed = 0;  // key of the native sweep stream (seed of the first population)
  SweepLaunch sweep{};
  PopDev* d_pops = nullptr;
  BatchDev* d_batch = nullptr;
  DevBuf buf;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraph_t graph_t = nullptr;
  cudaGraphExec_t exec = nullptr;
  // rows[set] = rows of one population in one run; set = run * npop + user population index
  std::vector<std::vector<double>> rows;
  int sets_done = 0;
  bool ran = false;  // pa_run has been called
  int runs_done = 0;  // completed runs: the first one chooses adaptive schedules, the others replay them
  bool records = false;  // some population keeps an MHR histogram or its energies
  bool family = false;   // some population keeps family statistics
  std::string lattice_dir;  // pa_set_lattice_dump: per-temperature population text of the first run
  int lattice_prec = 11;
  bool lattice_failed = false;
  int step_run = -1;  // stepped run in progress (pa_run_begin .. pa_run_end): its index, else -1
  bool unusable = false;  // a restore failed after writing device buffers: runs refused until one succeeds
  int step_i = 0;     // temperatures done in it
  std::vector<std::vector<double>> fam;  // per set: rows of (families, rho_t, S_f)
  std::vector<std::vector<double>> mhr;                    // per set: rows of (beta, E/N, C/N, betaF/N)
  std::vector<std::vector<std::vector<int32_t>>> energies;  // per set, per temperature: energies
  std::vector<int> drained;                                 // per population: last temperature read back
  double ms = 0.0, attempts = 0.0;
  std::string err;
  std::vector<void*> staging;  // per population: device copy of a caller-supplied initial population

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

  cudaError_t sweep_launch(int energy_only) {
    if (ssc_bits) return launch_ssc_bits_sweep(d_batch, energy_only, stream_seed, sweep, stream);
    return cs > 1 ? launch_msc_cluster_sweep(cs, cthreads, d_batch, rng_mode, energy_only, stream_seed, sweep, stream)
                  : launch_sweep(d_batch, coding, rng_mode, energy_only, stream_seed, sweep, stream);
  }

  // after finish_step: energy records and family statistics of the temperature just finished
  cudaError_t enqueue_record() {
    cudaError_t e = cudaSuccess;
    if (records) e = launch("record", [&] { return launch_record(d_pops, npop, rblocks, stream); });
    if (e == cudaSuccess && family) e = launch("family", [&] { return launch_family_stats(d_pops, npop, rblocks, stream); });
    return e;
  }

  cudaError_t enqueue_init() {
    cudaError_t e;
    const bool msc = coding == PA_CODING_MSC;
    for (const auto& P : pops)  // the run's MHR histogram starts empty (PAisingSSC.cu:497-499)
      if (P.h.mhr_hist &&
          (e = cudaMemsetAsync(P.h.mhr_hist, 0, sizeof(unsigned long long) * (P.h.N + 1), stream)) != cudaSuccess)
        return e;
    if ((e = launch("begin_run", [&] { return launch_begin_run(d_pops, npop, stream); })) != cudaSuccess) return e;
    if ((e = launch(msc ? "msc_init" : "ssc_init", [&] { return launch_init(d_pops, npop, coding, stream); })) != cudaSuccess)
      return e;
    if (family && (e = launch("family_init", [&] { return launch_family_init(d_pops, npop, rblocks, stream); })) !=
                      cudaSuccess)
      return e;
    if ((e = launch("plan", [&] { return launch_plan(d_batch, npop, 1, stream); })) != cudaSuccess) return e;
    e = launch(msc ? "msc_energy" : "ssc_energy", [&] { return sweep_launch(1); });
    if (e != cudaSuccess) return e;
    e = launch("finish_step", [&] { return launch_finish_step(d_pops, npop, stream); });
    return e != cudaSuccess ? e : enqueue_record();
  }

  cudaError_t enqueue_step() {
    cudaError_t e;
    const bool msc = coding == PA_CODING_MSC;
    if ((e = launch("q", [&] { return launch_q(d_pops, npop, rblocks, stream); })) != cudaSuccess) return e;
    if ((e = launch("copy_numbers", [&] { return launch_copy_numbers(d_pops, npop, rblocks, stream); })) != cudaSuccess)
      return e;
    if ((e = launch("scatter", [&] { return launch_scatter(d_pops, npop, rblocks, stream); })) != cudaSuccess) return e;
    e = launch(msc ? "msc_resample" : "ssc_resample", [&] { return launch_resample(d_batch, coding, rng_mode, stream); });
    if (e != cudaSuccess) return e;
    if (family && (e = launch("family_resample", [&] { return launch_family_resample(d_pops, npop, rblocks, stream); })) !=
                      cudaSuccess)
      return e;
    if ((e = launch("plan", [&] { return launch_plan(d_batch, npop, 0, stream); })) != cudaSuccess) return e;
    e = launch(msc ? "msc_sweep" : "ssc_sweep", [&] { return sweep_launch(0); });
    if (e != cudaSuccess) return e;
    e = launch("finish_step", [&] { return launch_finish_step(d_pops, npop, stream); });
    if (e == cudaSuccess) e = enqueue_record();
    if (e != cudaSuccess || !adaptive) return e;
    return launch("adapt", [&] { return launch_adapt(d_pops, npop, stream); });
  }

  // Energies of the temperatures recorded since the last call, from the
  // device ring into energies[r * npop + population] (active replicas only,
  // in the reference's replica order).
  cudaError_t drain(int r) {
    if (!records) return cudaSuccess;
    std::vector<PopDev> st(npop);
    cudaError_t e = cudaMemcpyAsync(st.data(), d_pops, sizeof(PopDev) * npop, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    std::vector<int32_t> ev;
    std::vector<uint8_t> av;
    for (int k = 0; k < npop && e == cudaSuccess; ++k) {
      const PopDev& h = pops[k].h;
      if (!(h.rec & kRecEnergies)) continue;
      auto& dst = energies[(size_t)r * npop + pops[k].user_index];
      const size_t stride = h.coding == PA_CODING_MSC ? (size_t)h.rgcap * kMsb : (size_t)h.Rcap;
      for (int s = drained[k] + 1; s <= st[k].last_rec && e == cudaSuccess; ++s) {
        const int slot = s % h.ring;
        int n = 0;
        e = cudaMemcpy(&n, h.nlog + slot, sizeof(int), cudaMemcpyDeviceToHost);
        ev.resize((size_t)n);
        av.assign((size_t)n, 1);
        if (e == cudaSuccess && n > 0)
          e = cudaMemcpy(ev.data(), h.elog + slot * stride, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && n > 0 && h.alog)
          e = cudaMemcpy(av.data(), h.alog + slot * stride, (size_t)n, cudaMemcpyDeviceToHost);
        if ((int)dst.size() <= s) dst.resize((size_t)s + 1);
        dst[s].clear();
        for (int j = 0; j < n; ++j)
          if (av[j]) dst[s].push_back(ev[j]);
      }
      drained[k] = std::max(drained[k], st[k].last_rec);
    }
    return e;
  }

  // A whole run as one launch sequence (fixed schedules: the graph of a run).
  cudaError_t enqueue_run() {
    cudaError_t e = enqueue_init();
    for (int i = 1; i <= max_steps && e == cudaSuccess; ++i) e = enqueue_step();
    return e;
  }

  // Adaptive schedules end when the device says so: every population has
  // passed its last step or stopped with an error.
  cudaError_t all_done(bool* done) {
    std::vector<PopDev> st(npop);
    cudaError_t e = cudaMemcpyAsync(st.data(), d_pops, sizeof(PopDev) * npop, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    *done = true;
    for (const auto& s : st)
      if (!s.error && s.step <= s.nsteps) *done = false;
    return e;
  }

  // The device values of the adaptive-step switch and step bound that a run
  // starts from: the handle's first run chooses its temperatures, every later
  // run (of the same or a later pa_run) replays that schedule, as the
  // reference's runs after the first do (PAisingSSC.cu:644,662).
  cudaError_t set_adaptive(bool first_run) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < npop && e == cudaSuccess; ++k) {
      if (!pops[k].cfg.adaptive) continue;
      const int on = first_run ? 1 : 0;
      e = cudaMemcpy(&d_pops[k].adaptive, &on, sizeof(int), cudaMemcpyHostToDevice);
      if (e == cudaSuccess && first_run)
        e = cudaMemcpy(&d_pops[k].nsteps, &pops[k].nsteps, sizeof(int), cudaMemcpyHostToDevice);
      if (e == cudaSuccess && first_run)
        e = cudaMemcpy(&d_pops[k].dbeta_cur, &pops[k].cfg.dbeta, sizeof(double), cudaMemcpyHostToDevice);
    }
    return e;
  }

  // The population of population k after temperature i to the lattice files
  // (only when it did advance to i).
  cudaError_t dump_lattice(int k, int i, double beta) {
    PopDev st;
    cudaError_t e = cudaMemcpy(&st, d_pops + k, sizeof(PopDev), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess || st.error || st.step - 1 != i) return e;
    const int units = st.coding == PA_CODING_MSC ? (st.R_cur + kMsb - 1) / kMsb * kMsb : st.R_cur;
    std::vector<uint8_t> sp(population_bytes(st.coding, st.L, st.R_cur));
    std::vector<uint8_t> act(st.coding == PA_CODING_MSC ? (size_t)units : 0);
    e = cudaMemcpy(sp.data(), st.spins[st.parity], sp.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && !act.empty())
      e = cudaMemcpy(act.data(), st.active[st.parity], act.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess &&
        write_lattice(lattice_dir, i, beta, lattice_prec, st.coding, st.L, st.R_cur, sp.data(), act.data(), units))
      lattice_failed = true;
    return e;
  }

  // Run r, on the stream: graph replays or host-stepped launches.  Recorded
  // energies are read back whenever the device ring may be about to wrap.
  cudaError_t run_once(int r) {
    cudaError_t e;
    drained.assign(npop, -1);
    const bool lattices = !lattice_dir.empty() && runs_done == 0 && r == 0;  // the first run, as the reference
    if (graph && !lattices) {
      e = cudaGraphLaunch(exec, stream);
      while (adaptive && e == cudaSuccess) {
        bool done = false;
        e = drain(r);
        if (e == cudaSuccess) e = all_done(&done);
        if (e != cudaSuccess || done) break;
        e = cudaGraphLaunch(chunk_exec, stream);
      }
      return e == cudaSuccess ? drain(r) : e;
    }
    e = plain_begin(r);
    bool done = false;
    for (int i = 1; e == cudaSuccess && !done; ++i) e = plain_step(r, i, lattices, &done);
    return e;
  }

  // Host-stepped pieces of run r (plain mode and the stepping entry points):
  // the set-up and initial population ...
  cudaError_t plain_begin(int r) {
    drained.assign(npop, -1);
    cudaError_t e = enqueue_init();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) e = drain(r);
    return e;
  }

  // ... and temperature i; *done once every population is through its schedule
  cudaError_t plain_step(int r, int i, bool lattices, bool* done) {
    cudaError_t e = enqueue_step();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    // the host reads every step's result, like the reference's host loop
    for (int k = 0; k < npop && e == cudaSuccess; ++k) {
      if (i >= pops[k].cap) continue;
      double row[kRowCols];
      e = cudaMemcpy(row, pops[k].h.rows + (size_t)i * kRowCols, sizeof(row), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && lattices) e = dump_lattice(k, i, row[0]);
    }
    if (e == cudaSuccess) e = drain(r);
    *done = i >= max_steps;
    if (adaptive && e == cudaSuccess) e = all_done(done);
    return e;
  }

  // After run r: its rows, statistics and status into result sets r*npop + k.
  int collect_run(int r) {
    int status = PA_OK;
    std::vector<PopDev> back(npop);
    cudaError_t e = cudaMemcpyAsync(back.data(), d_pops, sizeof(PopDev) * npop, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    for (int k = 0; k < npop && e == cudaSuccess; ++k) {
      // rows of the schedule the run followed (adaptive: as long as the device made it)
      const PopHost& P = pops[k];
      const int nrows = std::min(back[k].nsteps + 1, P.cap);
      std::vector<double>& dst = rows[(size_t)r * npop + P.user_index];
      dst.assign((size_t)nrows * kRowCols, 0.0);
      e = cudaMemcpyAsync(dst.data(), P.h.rows, dst.size() * sizeof(double), cudaMemcpyDeviceToHost, stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "run");
    for (int k = 0; k < npop; ++k) {
      if (back[k].error) {
        switch (back[k].error) {
          case kErrExtinct:
            status = PA_ERR_EXTINCT;
            err = "resampling produced an empty population";
            break;
          case kErrTooManySteps:
            status = PA_ERR_TOO_MANY_STEPS;
            err = "number of temperature steps exceeds nBmax=10000 (raise R or lower min_overlap)";
            break;
          case kErrSweepForm:
            status = PA_ERR_STATE;
            err = "sweep kernel built for another lattice size";
            break;
          default:
            status = PA_ERR_CAPACITY;
            err = "population exceeded its buffer capacity (raise pa_config.capacity)";
        }
      }
      const PopHost& P = pops[k];
      const std::vector<double>& rw = rows[(size_t)r * npop + P.user_index];
      for (size_t i = 1; i < rw.size() / kRowCols; ++i)
        attempts += (double)P.cfg.sweeps * (double)P.h.N * rw[i * kRowCols + 8];
      if (P.h.mhr_hist && !back[k].error) {
        std::vector<unsigned long long> hist((size_t)P.h.N + 1);
        e = cudaMemcpy(hist.data(), P.h.mhr_hist, sizeof(unsigned long long) * hist.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "MHR histogram");
        mhr[(size_t)r * npop + P.user_index] = mhr_analysis(P.h.N, rw, hist);
      }
      if (P.h.family && !back[k].error) {
        std::vector<double>& f = fam[(size_t)r * npop + P.user_index];
        f.assign(rw.size() / kRowCols * 3, 0.0);
        e = cudaMemcpy(f.data(), P.h.fam_rows, sizeof(double) * f.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "family statistics");
      }
    }
    if (status == PA_OK) {
      sets_done = (r + 1) * npop;
      ++runs_done;
    }
    return status;
  }

  // Result containers for a new pa_run (or stepped run).
  void reset_results() {
    rows.assign((size_t)npop * seq_runs, {});
    mhr.assign((size_t)npop * seq_runs, {});
    energies.assign((size_t)npop * seq_runs, {});
    fam.assign((size_t)npop * seq_runs, {});
    sets_done = 0;
    attempts = 0;
    ran = true;
  }

  // Persistent sweep grid for the populations' current geometry and, in
  // graph mode, the run captured as one graph (again, after a re-tune).
  // The lattice size of a sweep kernel built for one size, when every
  // population of the handle can use it (MSC, one group per work unit, one
  // L); kWith96 when only some can (the general kernel with that size's form).
  int fixed_l(const std::vector<SweepGeom>& geo) const {
    if (coding != PA_CODING_MSC || cs != 1 || rng_mode != PA_RNG_NATIVE || geo.empty()) return 0;
    int n = 0;
    for (const auto& g : geo) n += msc_fixed_l(g.L, g.G) == 96;
    return n == (int)geo.size() ? 96 : n > 0 ? kWith96 : 0;
  }

  cudaError_t setup_launches() {
    int max_smem = 0;
    std::vector<SweepGeom> geo;
    for (const auto& P : pops) {
      max_smem = std::max(max_smem, P.geom.smem);
      geo.push_back(P.geom);
    }
    cudaError_t e = ssc_bits ? ssc_bits_setup(max_smem, &sweep)
                    : cs > 1 ? msc_cluster_setup(cs, cthreads, rng_mode, max_smem, &sweep)
                             : sweep_setup(coding, rng_mode, max_smem, &sweep, fixed_l(geo));
    if (e != cudaSuccess || !graph) return e;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph_t) cudaGraphDestroy(graph_t);
    if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
    if (chunk_t) cudaGraphDestroy(chunk_t);
    exec = chunk_exec = nullptr;
    graph_t = chunk_t = nullptr;
    // fixed schedules: one graph per run; adaptive: the set-up plus a first
    // chunk of steps, then chunks of kChunk steps until the device is done
    auto capture = [&](int steps, bool with_init, cudaGraph_t* g, cudaGraphExec_t* x) {
      cudaError_t c = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
      if (c != cudaSuccess) return c;
      cudaError_t e1 = with_init ? enqueue_init() : cudaSuccess;
      for (int i = 1; i <= steps && e1 == cudaSuccess; ++i) e1 = enqueue_step();
      cudaError_t e2 = cudaStreamEndCapture(stream, g);
      if (e1 != cudaSuccess) return e1;
      if (e2 != cudaSuccess) return e2;
      return cudaGraphInstantiate(x, *g, 0);
    };
    if (!adaptive) return capture(max_steps, true, &graph_t, &exec);
    e = capture(kChunk, true, &graph_t, &exec);
    if (e == cudaSuccess) e = capture(kChunk, false, &chunk_t, &chunk_exec);
    return e;
  }

  cudaError_t upload_pops(const std::vector<PopDev>& hp) {
    return cudaMemcpy(d_pops, hp.data(), sizeof(PopDev) * npop, cudaMemcpyHostToDevice);
  }

  // Device time per spin-flip attempt of one sweep launch over the
  // populations flagged in `part` (the others are marked finished), with
  // geometry geo[k] for population k (SSC: `bits` selects the bit-plane
  // sweep); the population state is the one left on the device by the caller
  // (an initialised population at step 1).
  // cs > 1: the MSC cluster sweep with clusters of cs CTAs of cluster_threads
  cudaError_t time_sweep(const std::vector<PopDev>& state, const std::vector<char>& part,
                         const std::vector<SweepGeom>& geo, bool bits, double* ns_per_attempt, int tcs = 1,
                         int cluster_threads = 256) {
    std::vector<PopDev> hp = state;
    double attempts = 0;
    int smem = 0;
    for (int k = 0; k < npop; ++k) {
      if (part[k]) {
        geom_to_pop(geo[k], &hp[k]);
        smem = std::max(smem, geo[k].smem);
        if (pop_stepping(&hp[k])) attempts += (double)pops[k].cfg.sweeps * hp[k].N * (double)hp[k].R_cur;
      } else {
        hp[k].step = hp[k].nsteps + 1;
      }
    }
    cudaError_t e = upload_pops(hp);
    SweepLaunch sl{};
    if (e == cudaSuccess)
      e = bits ? ssc_bits_setup(smem, &sl)
               : tcs > 1 ? msc_cluster_setup(tcs, cluster_threads, rng_mode, smem, &sl)
                         : sweep_setup(coding, rng_mode, smem, &sl, fixed_l(geo));
    float best = 0.f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {  // the first launch warms up
      e = launch_plan(d_batch, npop, 0, stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev0, stream);
      if (e == cudaSuccess)
        e = bits ? launch_ssc_bits_sweep(d_batch, 0, stream_seed, sl, stream)
                 : tcs > 1 ? launch_msc_cluster_sweep(tcs, cluster_threads, d_batch, rng_mode, 0, stream_seed, sl,
                                                      stream)
                           : launch_sweep(d_batch, coding, rng_mode, 0, stream_seed, sl, stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev1, stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
      if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    *ns_per_attempt = attempts > 0 ? best * 1e6 / attempts : 0.0;
    return e;
  }

  ~pa_handle() {
    for (void* p : staging)
      if (p) cudaFree(p);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph_t) cudaGraphDestroy(graph_t);
    if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
    if (chunk_t) cudaGraphDestroy(chunk_t);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

// CTAs per MSC group: the requested variant, or automatically one CTA when
// the group (4 N bytes) fits its shared memory and a cluster of 2 otherwise.
int msc_variant(int requested, int L) { return requested ? requested : (L > 128 ? 2 : 1); }

// Automatic sweep form of an MSC batch whose populations all leave the form
// to the engine (sweep_variant 0, tile_groups 0) and have 48 <= L <= 128,
// L % 8 == 0: a batch with too few groups to keep the resident one-CTA sweep
// slots busy runs each group on a cluster of 4 or 2 CTAs of 256 threads,
// so that more SMs take part and the last wave is finer.  The thresholds
// (groups as fractions of the slots, 608 on a GB300) come from the measured
// crossovers of whole single-population anneals on a GB300: L=64 (compile-time
// cluster form for clusters of 2) clusters of 4 up to ~110 groups, of 2 up
// to ~700; L=128 (compile-time forms for both; its one-CTA form fits three
// CTAs per SM) 4 up to ~550, 2 up to ~2000; other sizes 4 up to ~200, 2 up to
// ~400.  Smaller lattices keep stacked tiles, which serve them better.
int msc_auto_clusters(const std::vector<pa_config>& cfgs, int cs, long long groups, int slots) {
  if (cs != 1) return cs;
  int L0 = 0;
  bool same_L = true;
  for (const auto& c : cfgs) {
    if (c.coding != PA_CODING_MSC || c.sweep_variant != 0 || c.tile_groups != 0 || c.L < 48 || c.L > 128 ||
        c.L % 8 != 0)
      return cs;
    if (L0 && c.L != L0) same_L = false;
    L0 = c.L;
  }
  // per mille of the slots: clusters of 4 up to t4, of 2 up to t2
  long long t4 = 330, t2 = 660;
  if (same_L && L0 == 64) t4 = 180, t2 = 1150;
  if (same_L && L0 == 128) t4 = 900, t2 = 3300;
  if (groups * 1000 <= t4 * slots) return 4;
  if (groups * 1000 <= t2 * slots) return 2;
  return 1;
}

// Automatic cluster size of an MSC batch that holds a lattice above L = 128
// (which needs a cluster) and leaves the form to the engine: clusters of 4
// CTAs of 512 threads from just over one resident wave of clusters of 2 (1024
// threads, one CTA per SM) up to eight such waves, clusters of 2 otherwise.
// Measured on whole anneals at L = 144..256 on a GB300:
// with at most one wave the larger halo share and cluster barriers of
// clusters of 4 cost more than they spread; just past one wave clusters of 2
// run a nearly empty second wave (L=256, clusters of 2 vs 4: 63 groups 4095
// vs 3897 attempts/ns, 82 groups 2723 vs 3599); from about eight waves on
// both fill the GPU and clusters of 2 do slightly less work per site.
int msc_auto_large_clusters(const std::vector<pa_config>& cfgs, int cs, long long groups, int rng_mode) {
  if (cs != 2) return cs;
  int maxL = 0, smem = 0;
  for (const auto& c : cfgs) {
    SweepGeom g2, g4;
    if (c.coding != PA_CODING_MSC || c.sweep_variant != 0 || c.tile_groups != 0 ||
        !msc_cluster_geom(c.L, 2, 1024, &g2) || !msc_cluster_geom(c.L, 4, 512, &g4))
      return cs;
    maxL = std::max(maxL, c.L);
    smem = std::max(smem, g2.smem);
  }
  if (maxL <= 128) return cs;
  SweepLaunch sl{};
  if (msc_cluster_setup(2, 1024, rng_mode, smem, &sl) != cudaSuccess) {
    cudaGetLastError();
    return cs;
  }
  const long long wave2 = sl.grid / 2;  // resident clusters of 2
  return groups > wave2 && groups <= 8 * wave2 ? 4 : 2;
}

int validate(const pa_config& c) {
  auto bad = [](const char* m) {
    pa::g_last_error = m;
    return PA_ERR_ARG;
  };
  if (c.coding != PA_CODING_SSC && c.coding != PA_CODING_MSC) return bad("coding must be SSC or MSC");
  if (c.rng_mode != PA_RNG_NATIVE && c.rng_mode != PA_RNG_REFERENCE) return bad("bad rng_mode");
  if (c.weights != PA_WEIGHTS_FP32 && c.weights != PA_WEIGHTS_FP64) return bad("bad weights");
  if (c.R < 1 || c.sweeps < 0 || c.runs < 1 || !(c.dbeta > 0) || !(c.beta_final > 0))
    return bad("R, sweeps, runs, dbeta, beta_final out of range");
  if (c.capacity != 0 && c.capacity < 1.0) return bad("capacity must be >= 1");
  // replica indices and slot counts are 32-bit on the device
  if ((c.capacity > 0 ? c.capacity : 1.25) * (double)c.R + 256.0 > 2147483647.0 - kMsb)
    return bad("R * capacity must stay below 2^31 replica slots");
  if (c.sweep_variant != 0 && c.sweep_variant != 1 && c.sweep_variant != 2 && c.sweep_variant != 4)
    return bad("sweep_variant must be 0, 1, 2 or 4");
  if (c.coding == PA_CODING_SSC && c.sweep_variant > 1) return bad("cluster sweeps exist for MSC only");
  SweepGeom g;
  if (c.coding == PA_CODING_SSC && c.tile_groups != 0) {
    // replicas per tile of the bit-plane sweep
    if (c.rng_mode != PA_RNG_NATIVE || c.sweep_variant == 1 || !ssc_bits_geom(c.L, &g, c.tile_groups))
      return bad("SSC tile_groups: replicas per bit-plane tile (native stream), the largest tile for L or a "
                 "power-of-two fraction of it");
  } else {
    if (c.tile_groups != 0 && c.tile_groups != 1 && c.tile_groups != 2 && c.tile_groups != 4 && c.tile_groups != 8)
      return bad("tile_groups must be 0, 1, 2, 4 or 8");
    if (c.tile_groups > 1 && msc_variant(c.sweep_variant, c.L) > 1)
      return bad("tiles of several groups exist for the one-CTA MSC sweep only");
  }
  if (c.coding == PA_CODING_MSC) {
    const int cs = msc_variant(c.sweep_variant, c.L);
    if (cs == 1 && c.tile_groups > 1 && !msc_geom(c.L, &g, c.tile_groups))
      return bad("tile_groups > 1 needs L % 4 == 0 and at most 44 KB of spins per tile");
    const bool ok = cs == 1 ? msc_geom(c.L, &g) : msc_cluster_geom(c.L, cs, msc_cluster_threads(cs, c.L), &g);
    if (!ok) return bad("MSC needs even L in [8, 128] (one CTA per group) or L % 4 == 0 up to 256 (clusters)");
  } else if (!ssc_geom(c.L, &g)) {
    return bad("SSC needs L % 8 == 0, 8 <= L <= 256");
  }
  if (c.adaptive != 0 && c.adaptive != 1) return bad("adaptive must be 0 or 1");
  if ((c.mhr != 0 && c.mhr != 1) || (c.store_energies != 0 && c.store_energies != 1) ||
      (c.family != 0 && c.family != 1))
    return bad("mhr, store_energies and family must be 0 or 1");
  if (c.adaptive) {
    const double lo = c.min_overlap > 0 ? c.min_overlap : kMinOverlap;
    const double hi = c.max_overlap > 0 ? c.max_overlap : kMaxOverlap;
    if (!(lo > 0 && lo < hi && hi < 1)) return bad("adaptive step needs 0 < min_overlap < max_overlap < 1");
  } else if ((int)schedule(c.dbeta, c.beta_final).size() > kNBmax - 1) {
    pa::g_last_error = "number of temperature steps exceeds nBmax=10000";
    return PA_ERR_TOO_MANY_STEPS;
  }
  return PA_OK;
}

// Builds a handle from per-population configurations (already validated and
// sharing coding, rng_mode, weights, graph, device).
int build_handle(const std::vector<pa_config>& cfgs, int seq_runs, pa_handle** out) {
  pa_handle* H = new (std::nothrow) pa_handle();
  if (!H) return PA_ERR_ARG;
  auto fail = [&](int code, const std::string& m) {
    pa::g_last_error = m;
    delete H;
    return code;
  };
  const pa_config& c0 = cfgs[0];
  H->coding = c0.coding;
  H->rng_mode = c0.rng_mode;
  H->graph = c0.graph;
  H->device = c0.device;
  H->seq_runs = seq_runs;
  H->npop = (int)cfgs.size();
  H->stream_seed = c0.seed;
  cudaError_t e = cudaSetDevice(c0.device);
  if (e != cudaSuccess) return fail(PA_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));

  // one sweep kernel serves the whole batch: clusters if any population needs them
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c0.device);
  const int slots = 4 * nsm;  // resident one-CTA sweep CTAs (four per SM, register-bound)
  H->cs = 1;
  long long batch_groups = 0;  // work available to the one-CTA sweep: bounds automatic tile sizes
  int maxL = 0;
  if (H->coding == PA_CODING_MSC)
    for (const auto& c : cfgs) {
      H->cs = std::max(H->cs, msc_variant(c.sweep_variant, c.L));
      batch_groups += (c.R + kMsb - 1) / kMsb;
      maxL = std::max(maxL, c.L);
    }
  H->cs = msc_auto_clusters(cfgs, H->cs, batch_groups, slots);
  H->cs = msc_auto_large_clusters(cfgs, H->cs, batch_groups, H->rng_mode);
  H->cthreads = msc_cluster_threads(H->cs, maxL);
  // SSC with the native stream: bit-plane sweep when every lattice packs
  // into words at least 3/4 full (sweep_variant 1 keeps the int8 sweep;
  // pa_autotune may also choose a sparser bit-plane layout by timing)
  H->ssc_bits = H->coding == PA_CODING_SSC && H->rng_mode == PA_RNG_NATIVE;
  long long batch_replicas = 0;  // work of the bit-plane sweep: bounds its tile sizes
  bool ssc_tiles = false;        // a population asks for a bit-plane tile size
  for (const auto& c : cfgs) {
    if (c.sweep_variant == 1 || ssc_bits_fill(c.L) < 0.75) H->ssc_bits = false;
    batch_replicas += c.R;
    ssc_tiles = ssc_tiles || (c.coding == PA_CODING_SSC && c.tile_groups > 0);
  }
  if (ssc_tiles) {  // every population of the batch then needs a bit-plane layout
    H->ssc_bits = true;
    for (const auto& c : cfgs) {
      SweepGeom gb;
      if (c.sweep_variant == 1 || !ssc_bits_geom(c.L, &gb)) return fail(PA_ERR_ARG, "SSC tile_groups needs every "
                                                                      "population of the batch on bit planes");
    }
  }
  H->pops.resize(cfgs.size());
  for (size_t k = 0; k < cfgs.size(); ++k) {
    PopHost& P = H->pops[k];
    P.cfg = cfgs[k];
    P.user_index = (int)k;
    if (P.cfg.capacity <= 0) P.cfg.capacity = 1.25;
    bool okg;
    if (P.cfg.coding == PA_CODING_SSC)
      okg = H->ssc_bits ? ssc_bits_geom(P.cfg.L, &P.geom, P.cfg.tile_groups, batch_replicas, slots)
                        : ssc_geom(P.cfg.L, &P.geom);
    else if (H->cs == 1) okg = msc_geom(P.cfg.L, &P.geom, P.cfg.tile_groups, batch_groups, slots);
    else okg = msc_cluster_geom(P.cfg.L, H->cs, H->cthreads, &P.geom);
    if (!okg) return fail(PA_ERR_ARG, "L=" + std::to_string(P.cfg.L) + " cannot join a batch swept by clusters of " +
                                          std::to_string(H->cs) + " CTAs");
    if (P.cfg.adaptive) {
      // the first step is dbeta; the device chooses the others (at most the
      // rows nBmax allows) and ends the schedule at beta_final
      P.betas = {0.0};
      if (P.cfg.dbeta <= P.cfg.beta_final) P.betas.push_back(P.cfg.dbeta);
      P.nsteps = P.betas.size() > 1 ? kNBmax - 1 : 0;
      P.cap = kNBmax;
      H->adaptive = true;
    } else {
      P.betas = schedule(P.cfg.dbeta, P.cfg.beta_final);
      P.nsteps = (int)P.betas.size() - 1;
      P.cap = (int)P.betas.size();
    }
    P.thr.assign(P.betas.size() * kThrPerStep, 0u);
    for (size_t i = 0; i < P.betas.size(); ++i) thresholds(P.betas[i], &P.thr[i * kThrPerStep]);
  }
  // longest work units first: persistent CTAs then finish the batch together
  std::stable_sort(H->pops.begin(), H->pops.end(), [](const PopHost& a, const PopHost& b) {
    return (long long)a.cfg.L * a.cfg.L * a.cfg.sweeps > (long long)b.cfg.L * b.cfg.L * b.cfg.sweeps;
  });

  long long max_units = 1;
  DevBuf& B = H->buf;
  auto chk = [&](cudaError_t err) {
    if (err != cudaSuccess && e == cudaSuccess) e = err;
  };
  for (int k = 0; k < H->npop; ++k) {
    PopHost& P = H->pops[k];
    const pa_config& c = P.cfg;
    PopDev& h = P.h;
    std::memset(&h, 0, sizeof(h));
    const int L = c.L, N = L * L;
    const long long Rcap = (long long)std::ceil(c.capacity * c.R) + 256;
    const long long rgcap = (Rcap + kMsb - 1) / kMsb;
    h.L = L;
    h.N = N;
    h.coding = c.coding;
    h.Rinit = c.R;
    h.Rcap = (int)Rcap;
    h.rgcap = (int)rgcap;
    h.sweeps = c.sweeps;
    h.rng_mode = c.rng_mode;
    h.weights = c.weights;
    h.pop_id = P.user_index;
    h.run = -1;  // begin_run_kernel numbers the runs from 0
    h.nsteps = P.nsteps;
    h.seed = c.seed;
    h.bf0 = -N * std::log(2.0);
    geom_to_pop(P.geom, &h);
    // reference stream: every population starts at initial_sequence = 0 like a
    // separate run of the reference program; native stream: disjoint ranges
    h.iseq = c.rng_mode == PA_RNG_REFERENCE ? 0ull : (unsigned long long)P.user_index << 40;
    const size_t units = c.coding == PA_CODING_MSC ? (size_t)rgcap * kMsb : (size_t)Rcap;
    max_units = std::max(max_units, (long long)units);
    if (c.coding == PA_CODING_MSC) {
      uint32_t *a = nullptr, *b2 = nullptr;
      chk(B.alloc(&a, (size_t)rgcap * N));
      chk(B.alloc(&b2, (size_t)rgcap * N));
      h.spins[0] = a;
      h.spins[1] = b2;
      chk(B.alloc(&h.active[0], units));
      chk(B.alloc(&h.active[1], units));
      if (c.rng_mode == PA_RNG_NATIVE) {  // the native stream's word-level gather
        chk(B.alloc(&h.res_pairs, units));
        chk(B.alloc(&h.res_cnt, (size_t)rgcap));
      }
    } else {
      int8_t *a = nullptr, *b2 = nullptr;
      chk(B.alloc(&a, (size_t)Rcap * N));
      chk(B.alloc(&b2, (size_t)Rcap * N));
      h.spins[0] = a;
      h.spins[1] = b2;
    }
    chk(B.alloc(&h.E, units));
    chk(B.alloc(&h.M, units));
    chk(B.alloc(&h.roff, units));
    chk(B.alloc(&h.offs, units));
    chk(B.alloc(&h.src, (size_t)Rcap));
    chk(B.alloc(&h.blk_tot, kResBlocksMax));
    chk(B.alloc(&h.blk_off, kResBlocksMax));
    chk(B.alloc(&h.qpart_d, kResBlocksMax));
    chk(B.alloc(&h.qpart_f, 2 * kResBlocksMax));
    double* rows = nullptr;
    chk(B.alloc(&rows, (size_t)P.cap * kRowCols));
    h.rows = rows;
    double* bet = nullptr;
    chk(B.alloc(&bet, (size_t)P.cap));
    h.betas = bet;
    uint32_t* th = nullptr;
    chk(B.alloc(&th, (size_t)P.cap * kThrPerStep));
    h.thr = th;
    if (c.mhr) {
      chk(B.alloc(&h.mhr_hist, (size_t)N + 1));
      h.rec |= kRecMhr;
    }
    if (c.store_energies) {
      // fixed schedules: every temperature of a run; adaptive: one graph
      // chunk (plus the set-up) between read-backs
      h.ring = c.adaptive ? pa_handle::kChunk + 1 : P.nsteps + 1;
      chk(B.alloc(&h.elog, (size_t)h.ring * units));
      if (c.coding == PA_CODING_MSC) chk(B.alloc(&h.alog, (size_t)h.ring * units));
      chk(B.alloc(&h.nlog, (size_t)h.ring));
      h.rec |= kRecEnergies;
    }
    if (h.rec) H->records = true;
    if (c.family) {
      chk(B.alloc(&h.anc[0], units));
      chk(B.alloc(&h.anc[1], units));
      chk(B.alloc(&h.fam_cnt, (size_t)c.R));
      chk(B.alloc(&h.fam_rows, (size_t)P.cap * 3));
      chk(B.alloc(&h.fam_part, (size_t)kResBlocksMax * 3));
      if (e == cudaSuccess) chk(cudaMemset(h.fam_cnt, 0, sizeof(uint32_t) * (size_t)c.R));
      h.family = 1;
      H->family = true;
    }
    if (c.adaptive) {
      chk(B.alloc(&h.hist, (size_t)N + 1));
      h.adaptive = 1;
      h.dbeta_cur = c.dbeta;  // deltaBeta = dBinit (PAisingSSC.cu:508)
      h.min_ov = c.min_overlap > 0 ? c.min_overlap : kMinOverlap;
      h.max_ov = c.max_overlap > 0 ? c.max_overlap : kMaxOverlap;
      h.beta_fin = c.beta_final;
    }
    if (e != cudaSuccess) break;
    chk(cudaMemcpy(bet, P.betas.data(), P.betas.size() * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(th, P.thr.data(), P.thr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    H->max_steps = std::max(H->max_steps, P.nsteps);
  }
  if (e != cudaSuccess) return fail(PA_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  H->rblocks = res_blocks(max_units);
  chk(B.alloc(&H->d_pops, (size_t)H->npop));
  chk(B.alloc(&H->d_batch, 1));
  if (e != cudaSuccess) return fail(PA_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e));
  std::vector<PopDev> hp(H->npop);
  for (int k = 0; k < H->npop; ++k) hp[k] = H->pops[k].h;
  chk(cudaMemcpy(H->d_pops, hp.data(), sizeof(PopDev) * H->npop, cudaMemcpyHostToDevice));
  BatchDev bd;
  std::memset(&bd, 0, sizeof(bd));
  bd.npop = H->npop;
  bd.pops = H->d_pops;
  chk(cudaMemcpy(H->d_batch, &bd, sizeof(bd), cudaMemcpyHostToDevice));
  chk(cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking));
  chk(cudaEventCreate(&H->ev0));
  chk(cudaEventCreate(&H->ev1));
  H->staging.assign(H->npop, nullptr);
  if (e == cudaSuccess) chk(H->setup_launches());
  if (e != cudaSuccess) return fail(PA_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e));
  *out = H;
  return PA_OK;
}

}  // namespace

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
  int rc = validate(*cfg);
  if (rc) return rc;
  // independent runs: concurrent populations with disjoint native streams; with
  // the reference stream they must run one after the other, because each run
  // continues the subsequence counter of the previous one (PAisingSSC.cu:481-486);
  // with the adaptive step too, because later runs replay the first run's
  // schedule (PAisingSSC.cu:644,662)
  if (cfg->rng_mode == PA_RNG_REFERENCE || cfg->runs == 1 || cfg->adaptive) {
    pa_config c = *cfg;
    return build_handle({c}, cfg->runs, out);
  }
  std::vector<pa_config> cs(cfg->runs, *cfg);
  for (auto& c : cs) c.runs = 1;
  return build_handle(cs, 1, out);
}

int pa_create_batch(const pa_config* cfgs, int n, pa_handle** out) {
  if (!cfgs || !out || n < 1 || n > kMaxPop) return PA_ERR_ARG;
  *out = nullptr;
  std::vector<pa_config> cs(cfgs, cfgs + n);
  for (auto& c : cs) {
    int rc = validate(c);
    if (rc) return rc;
    if (c.runs != 1 || c.coding != cs[0].coding || c.rng_mode != cs[0].rng_mode || c.weights != cs[0].weights ||
        c.graph != cs[0].graph || c.device != cs[0].device) {
      pa::g_last_error = "batch members need runs=1 and one coding, rng_mode, weights, graph and device";
      return PA_ERR_ARG;
    }
  }
  return build_handle(cs, 1, out);
}

int pa_num_sets(const pa_handle* H, int* n) {
  if (!H || !n) return PA_ERR_ARG;
  *n = H->npop * H->seq_runs;
  return PA_OK;
}

int pa_run(pa_handle* H) {
  if (!H) return PA_ERR_ARG;
  if (H->unusable) {
    H->err = "a failed restore left this handle inconsistent: restore again or destroy it";
    return PA_ERR_STATE;
  }
  if (H->step_run >= 0) {
    H->err = "a stepped run is in progress (pa_run_end first)";
    return PA_ERR_STATE;
  }
  H->reset_results();
  cudaError_t e = cudaEventRecord(H->ev0, H->stream);
  if (e != cudaSuccess) return H->cuda_fail(e, "event");
  int status = PA_OK;
  for (int r = 0; r < H->seq_runs && status == PA_OK; ++r) {
    if (H->adaptive) {
      e = H->set_adaptive(H->runs_done == 0);
      if (e != cudaSuccess) return H->cuda_fail(e, "adaptive set-up");
    }
    H->lattice_failed = false;
    e = H->run_once(r);
    if (e != cudaSuccess) return H->cuda_fail(e, H->graph ? "graph launch" : "plain step");
    if (H->lattice_failed) {
      H->err = "cannot append to the lattice files in " + H->lattice_dir;
      return PA_ERR_ARG;
    }
    status = H->collect_run(r);
    if (status == PA_ERR_CUDA) return status;
  }
  e = cudaEventRecord(H->ev1, H->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(H->ev1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, H->ev0, H->ev1);
  if (e != cudaSuccess) return H->cuda_fail(e, "timing");
  H->ms = ms;
  return status;
}

int pa_run_begin(pa_handle* H) {
  if (!H) return PA_ERR_ARG;
  if (H->unusable) {
    H->err = "a failed restore left this handle inconsistent: restore again or destroy it";
    return PA_ERR_STATE;
  }
  if (H->step_run >= 0 || H->seq_runs != 1) {
    H->err = H->seq_runs != 1 ? "stepped runs need one run per handle (runs = 1 or a native batch)"
                              : "a stepped run is already in progress";
    return PA_ERR_STATE;
  }
  H->reset_results();
  cudaError_t e = H->adaptive ? H->set_adaptive(H->runs_done == 0) : cudaSuccess;
  if (e == cudaSuccess) e = H->plain_begin(0);
  if (e != cudaSuccess) return H->cuda_fail(e, "run begin");
  H->step_run = 0;
  H->step_i = 0;
  return PA_OK;
}

int pa_run_steps(pa_handle* H, int max_steps, int* done) {
  if (!H || max_steps < 0) return PA_ERR_ARG;
  if (H->step_run < 0) {
    H->err = "no stepped run in progress (pa_run_begin first)";
    return PA_ERR_STATE;
  }
  bool fin = false;
  cudaError_t e = H->all_done(&fin);
  const bool lattices = !H->lattice_dir.empty() && H->runs_done == 0;
  for (int k = 0; k < max_steps && e == cudaSuccess && !fin; ++k) e = H->plain_step(0, ++H->step_i, lattices, &fin);
  if (e != cudaSuccess) return H->cuda_fail(e, "run steps");
  if (H->lattice_failed) {
    H->err = "cannot append to the lattice files in " + H->lattice_dir;
    return PA_ERR_ARG;
  }
  if (done) *done = fin ? 1 : 0;
  return PA_OK;
}

int pa_run_end(pa_handle* H) {
  if (!H) return PA_ERR_ARG;
  if (H->step_run < 0) return PA_ERR_STATE;
  const int status = H->collect_run(0);
  H->step_run = -1;
  return status;
}

// ---------------------------------------------------------------- checkpoint
// File (version 2, little-endian, every field naturally aligned):
//   "PAGB300C", int32 {version, populations, coding, temperatures done,
//   runs completed}; then per population (device order) CkptPop (the shape
//   it was written for), CkptScalars (the dynamic scalars of its PopDev) and
//   its stateful buffers as (uint64 bytes, bytes) in ckpt_buffer_sizes'
//   order.  Device addresses and the configuration fields of PopDev are not
//   stored: a restore takes them from the handle.
namespace {
constexpr char kCkptMagic[8] = {'P', 'A', 'G', 'B', '3', '0', '0', 'C'};
constexpr int32_t kCkptVersion = 2;

struct CkptPop {
  int32_t L, R, Rcap, rgcap, cap, gpt, coding, rec, family;
};

struct CkptScalars {
  int32_t nsteps, step, R_prev, R_cur, parity, error, Emin, run, Emin_acc, last_rec, last_fam, pad;
  uint64_t iseq, sM4lo, sM4hi;
  int64_t sE, sE2, sM, sM2;
  double Emean, sumlnQ, lnQ, q, dbeta_cur;
};
static_assert(sizeof(CkptPop) == 36 && sizeof(CkptScalars) == 144, "checkpoint records are packed");

CkptScalars scalars_of(const PopDev& st) {
  CkptScalars c{};
  c.nsteps = st.nsteps; c.step = st.step; c.R_prev = st.R_prev; c.R_cur = st.R_cur; c.parity = st.parity;
  c.error = st.error; c.Emin = st.Emin; c.run = st.run; c.Emin_acc = st.Emin_acc; c.last_rec = st.last_rec;
  c.last_fam = st.last_fam; c.iseq = st.iseq; c.sM4lo = st.sM4lo; c.sM4hi = st.sM4hi; c.sE = st.sE;
  c.sE2 = st.sE2; c.sM = st.sM; c.sM2 = st.sM2; c.Emean = st.Emean; c.sumlnQ = st.sumlnQ; c.lnQ = st.lnQ;
  c.q = st.q; c.dbeta_cur = st.dbeta_cur;
  return c;
}

void apply_scalars(const CkptScalars& c, PopDev* st) {
  st->nsteps = c.nsteps; st->step = c.step; st->R_prev = c.R_prev; st->R_cur = c.R_cur; st->parity = c.parity;
  st->error = c.error; st->Emin = c.Emin; st->run = c.run; st->Emin_acc = c.Emin_acc; st->last_rec = c.last_rec;
  st->last_fam = c.last_fam; st->iseq = c.iseq; st->sM4lo = c.sM4lo; st->sM4hi = c.sM4hi; st->sE = c.sE;
  st->sE2 = c.sE2; st->sM = c.sM; st->sM2 = c.sM2; st->Emean = c.Emean; st->sumlnQ = c.sumlnQ; st->lnQ = c.lnQ;
  st->q = c.q; st->dbeta_cur = c.dbeta_cur;
  st->ticket = 0;
}

// Bytes of every stateful buffer of a population of shape cp holding R_cur
// replicas: current spins, MSC active flags, E, M, rows, betas, thresholds,
// MHR histogram (rec & kRecMhr), ancestors and family rows (family).
std::vector<size_t> ckpt_buffer_sizes(const CkptPop& cp, int R_cur) {
  const size_t units = cp.coding == PA_CODING_MSC ? (size_t)cp.rgcap * kMsb : (size_t)cp.Rcap;
  std::vector<size_t> b;
  b.push_back(population_bytes(cp.coding, cp.L, R_cur));
  if (cp.coding == PA_CODING_MSC) b.push_back(units);
  b.push_back(units * sizeof(int32_t));
  b.push_back(units * sizeof(int32_t));
  b.push_back((size_t)cp.cap * kRowCols * sizeof(double));
  b.push_back((size_t)cp.cap * sizeof(double));
  b.push_back((size_t)cp.cap * kThrPerStep * sizeof(uint32_t));
  if (cp.rec & kRecMhr) b.push_back(((size_t)cp.L * cp.L + 1) * sizeof(unsigned long long));
  if (cp.family) {
    b.push_back(units * sizeof(int32_t));
    b.push_back((size_t)cp.cap * 3 * sizeof(double));
  }
  return b;
}

// The same buffers of population st on the device (current half of the
// double buffers), in the same order.
std::vector<void*> state_buffers(const PopDev& st) {
  std::vector<void*> b;
  b.push_back(st.spins[st.parity]);
  if (st.coding == PA_CODING_MSC) b.push_back(st.active[st.parity]);
  b.push_back(st.E);
  b.push_back(st.M);
  b.push_back(st.rows);
  b.push_back(st.betas);
  b.push_back(st.thr);
  if (st.rec & kRecMhr) b.push_back(st.mhr_hist);
  if (st.family) {
    b.push_back(st.anc[st.parity]);
    b.push_back(st.fam_rows);
  }
  return b;
}

CkptPop shape_of(const PopHost& P) {
  return CkptPop{P.h.L, P.cfg.R, P.h.Rcap, P.h.rgcap, P.cap, P.h.gpt, P.h.coding, P.h.rec, P.h.family};
}

// A checkpoint file read into host memory.
struct CkptFile {
  int32_t head[5] = {0, 0, 0, 0, 0};
  struct Pop {
    CkptPop shape{};
    CkptScalars sc{};
    std::vector<std::vector<uint8_t>> bufs;
  };
  std::vector<Pop> pops;
};

// Reads and checks a whole checkpoint file before anything is written to a
// device: the header, every population's shape and scalars (sizes within the
// capacity, parity 0 or 1, step within the schedule) and every buffer's size
// against what that shape and population size need.  Returns "" or what is
// wrong.
std::string read_checkpoint(const char* path, CkptFile* out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return "cannot read the file";
  struct Closer {
    FILE* f;
    ~Closer() { std::fclose(f); }
  } closer{f};
  // the file's length bounds every buffer before anything is allocated for it
  if (std::fseek(f, 0, SEEK_END) != 0) return "cannot read the file";
  const long fsize = std::ftell(f);
  if (fsize < 0 || std::fseek(f, 0, SEEK_SET) != 0) return "cannot read the file";
  char magic[8];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kCkptMagic, 8) != 0) return "not a checkpoint";
  int32_t* head = out->head;
  if (std::fread(head, sizeof(int32_t), 5, f) != 5) return "truncated header";
  if (head[0] != kCkptVersion) return "unknown version";
  if (head[1] < 1 || head[1] > kMaxPop) return "population count out of range";
  if (head[2] != PA_CODING_SSC && head[2] != PA_CODING_MSC) return "unknown coding";
  if (head[3] < 0 || head[3] >= kNBmax || head[4] < 0) return "temperature or run count out of range";
  out->pops.resize(head[1]);
  for (int k = 0; k < head[1]; ++k) {
    CkptFile::Pop& p = out->pops[k];
    if (std::fread(&p.shape, sizeof(p.shape), 1, f) != 1 || std::fread(&p.sc, sizeof(p.sc), 1, f) != 1)
      return "truncated";
    const CkptPop& cp = p.shape;
    const CkptScalars& c = p.sc;
    if (cp.coding != head[2] || cp.L < 2 || cp.L > 4096 || cp.R < 1 || cp.Rcap < cp.R ||
        cp.rgcap != (int)(((long long)cp.Rcap + kMsb - 1) / kMsb) || cp.cap < 1 || cp.cap > kNBmax)
      return "population shape out of range";
    if (c.parity != 0 && c.parity != 1) return "buffer parity is not 0 or 1";
    if (c.R_cur < 0 || c.R_cur > cp.Rcap || c.R_prev < 0 || c.R_prev > cp.Rcap)
      return "population size beyond the capacity";
    if (c.nsteps < 0 || c.nsteps >= cp.cap || c.step < 0 || c.step > c.nsteps + 1)
      return "temperature index beyond the schedule";
    if (c.error < 0 || c.error > kErrSweepForm || c.run < -1 || c.last_rec < -1 || c.last_rec > cp.cap ||
        c.last_fam < -1 || c.last_fam > cp.cap)
      return "state field out of range";
    for (size_t want : ckpt_buffer_sizes(cp, c.R_cur)) {
      uint64_t n = 0;
      if (std::fread(&n, sizeof(n), 1, f) != 1) return "truncated";
      if (n != want) return "buffer size does not match the population";
      const long at = std::ftell(f);
      if (at < 0 || n > (uint64_t)(fsize - at)) return "truncated";
      try {
        p.bufs.emplace_back(n);
      } catch (const std::bad_alloc&) {
        return "buffer too large for host memory";
      }
      if (std::fread(p.bufs.back().data(), 1, n, f) != n) return "truncated";
    }
  }
  if (std::fgetc(f) != EOF) return "trailing bytes";
  return "";
}
}  // namespace

int pa_checkpoint(pa_handle* H, const char* path) {
  if (!H || !path) return PA_ERR_ARG;
  if (H->unusable) {
    H->err = "a failed restore left this handle inconsistent: restore again or destroy it";
    return PA_ERR_STATE;
  }
  if (H->step_run < 0) {
    H->err = "checkpoints are taken between the steps of a stepped run";
    return PA_ERR_STATE;
  }
  for (const auto& P : H->pops)
    if (P.h.rec & kRecEnergies) {
      H->err = "a run that stores its energies cannot be checkpointed";
      return PA_ERR_STATE;
    }
  std::vector<PopDev> st(H->npop);
  cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e == cudaSuccess) e = cudaMemcpy(st.data(), H->d_pops, sizeof(PopDev) * H->npop, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return H->cuda_fail(e, "checkpoint");
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    H->err = std::string("cannot write ") + path;
    return PA_ERR_ARG;
  }
  bool ok = std::fwrite(kCkptMagic, 1, 8, f) == 8;
  const int32_t head[5] = {kCkptVersion, H->npop, H->coding, H->step_i, H->runs_done};
  ok = ok && std::fwrite(head, sizeof(head), 1, f) == 1;
  std::vector<uint8_t> buf;
  for (int k = 0; k < H->npop && ok; ++k) {
    const CkptPop cp = shape_of(H->pops[k]);
    const CkptScalars sc = scalars_of(st[k]);
    ok = std::fwrite(&cp, sizeof(cp), 1, f) == 1 && std::fwrite(&sc, sizeof(sc), 1, f) == 1;
    const std::vector<size_t> sizes = ckpt_buffer_sizes(cp, sc.R_cur);
    const std::vector<void*> ptrs = state_buffers(st[k]);
    for (size_t j = 0; j < sizes.size() && ok; ++j) {
      buf.resize(sizes[j]);
      e = cudaMemcpy(buf.data(), ptrs[j], sizes[j], cudaMemcpyDeviceToHost);
      const uint64_t n = sizes[j];
      ok = e == cudaSuccess && std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(buf.data(), 1, n, f) == n;
    }
  }
  ok = (std::fclose(f) == 0) && ok;
  if (e != cudaSuccess) return H->cuda_fail(e, "checkpoint");
  if (!ok) {
    H->err = std::string("cannot write ") + path;
    return PA_ERR_ARG;
  }
  return PA_OK;
}

int pa_checkpoint_verify(const char* path) {
  if (!path) return PA_ERR_ARG;
  CkptFile cf;
  const std::string why = read_checkpoint(path, &cf);
  if (!why.empty()) {
    pa::g_last_error = std::string(path) + ": " + why;
    return PA_ERR_ARG;
  }
  return PA_OK;
}

int pa_restore(pa_handle* H, const char* path) {
  if (!H || !path) return PA_ERR_ARG;
  if (H->step_run >= 0) {
    H->err = "a stepped run is in progress";
    return PA_ERR_STATE;
  }
  // the whole file is read and checked first: a bad file changes nothing
  CkptFile cf;
  std::string why = read_checkpoint(path, &cf);
  if (why.empty() && (cf.head[1] != H->npop || cf.head[2] != H->coding))
    why = "written by a handle of another configuration";
  for (int k = 0; k < H->npop && why.empty(); ++k) {
    const PopHost& P = H->pops[k];
    const CkptPop want = shape_of(P);
    const CkptFile::Pop& p = cf.pops[k];
    if (std::memcmp(&p.shape, &want, sizeof(want)) != 0) why = "written by a handle of another configuration";
    else if (P.h.adaptive ? p.sc.nsteps > P.h.nsteps : p.sc.nsteps != P.h.nsteps)
      why = "schedule length differs from the handle's";
  }
  if (!why.empty()) {
    H->err = std::string(path) + ": " + why;
    return PA_ERR_ARG;
  }
  std::vector<PopDev> cur(H->npop);
  cudaError_t e = cudaMemcpy(cur.data(), H->d_pops, sizeof(PopDev) * H->npop, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return H->cuda_fail(e, "restore");
  // from here on a failure leaves device buffers half written
  for (int k = 0; k < H->npop && e == cudaSuccess; ++k) {
    apply_scalars(cf.pops[k].sc, &cur[k]);  // the handle's own configuration and buffers
    const std::vector<void*> ptrs = state_buffers(cur[k]);
    for (size_t j = 0; j < ptrs.size() && e == cudaSuccess; ++j)
      e = cudaMemcpy(ptrs[j], cf.pops[k].bufs[j].data(), cf.pops[k].bufs[j].size(), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(H->d_pops, cur.data(), sizeof(PopDev) * H->npop, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    H->unusable = true;
    return H->cuda_fail(e, "restore (the handle is unusable until a restore succeeds)");
  }
  H->unusable = false;
  H->reset_results();
  H->runs_done = cf.head[4];
  H->drained.assign(H->npop, -1);
  H->step_run = 0;
  H->step_i = cf.head[3];
  return PA_OK;
}

int pa_autotune(pa_handle* H, int* tiles, int n) {
  if (!H || (n > 0 && !tiles)) return PA_ERR_ARG;
  if (H->ran) {
    H->err = "pa_autotune must precede the first pa_run";
    return PA_ERR_STATE;
  }
  // MSC: groups per tile of the one-CTA sweep for every lattice size and,
  // where every population allows it (48 <= L <= 128, L % 8 == 0, form left
  // to the engine), clusters of 2 or 4 CTAs per group: the fastest form of
  // the batch is kept
  // Above L = 128 (clusters needed, form left to the engine): clusters of 2
  // CTAs of 1024 threads against clusters of 4 of 512.
  bool msc_tiles = H->coding == PA_CODING_MSC, msc_clusters = H->coding == PA_CODING_MSC;
  bool msc_large = H->coding == PA_CODING_MSC;
  int maxL = 0;
  for (const auto& P : H->pops) {
    SweepGeom g2, g4;
    maxL = std::max(maxL, P.cfg.L);
    if (P.cfg.L > 128 || P.cfg.sweep_variant > 1) msc_tiles = false;
    if (P.cfg.sweep_variant != 0 || P.cfg.tile_groups != 0 || P.cfg.L < 48 || P.cfg.L > 128 || P.cfg.L % 8 != 0)
      msc_clusters = false;
    if (P.cfg.sweep_variant != 0 || P.cfg.tile_groups != 0 || !msc_cluster_geom(P.cfg.L, 2, 1024, &g2) ||
        !msc_cluster_geom(P.cfg.L, 4, 512, &g4))
      msc_large = false;
  }
  msc_large = msc_large && maxL > 128;
  // SSC, native stream: int8 (4 sites per word) or bit planes (32 sites per
  // word) for the whole batch, when every population allows both and asks
  // for neither
  bool ssc_forms = H->coding == PA_CODING_SSC && H->rng_mode == PA_RNG_NATIVE;
  for (const auto& P : H->pops) {
    SweepGeom gb;
    if (P.cfg.sweep_variant != 0 || !ssc_bits_geom(P.cfg.L, &gb)) ssc_forms = false;
  }
  if (msc_tiles || ssc_forms || msc_large) {
    // an initialised population (step 1, random spins) to sweep
    cudaError_t e = H->enqueue_init();
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    std::vector<PopDev> state(H->npop);
    if (e == cudaSuccess) e = cudaMemcpy(state.data(), H->d_pops, sizeof(PopDev) * H->npop, cudaMemcpyDeviceToHost);
    if (msc_tiles) {  // groups per tile, per lattice size
      std::vector<int> done(H->npop, 0);
      for (int k = 0; k < H->npop && e == cudaSuccess; ++k) {
        if (done[k]) continue;
        const int L = H->pops[k].cfg.L;
        std::vector<char> part(H->npop, 0);
        for (int j = 0; j < H->npop; ++j) part[j] = H->pops[j].cfg.L == L;
        int best_G = 1;
        double best = 0;
        for (int G = 1; G <= 8 && e == cudaSuccess; G *= 2) {
          SweepGeom g;
          if (!msc_geom(L, &g, G)) continue;
          double t = 0;
          e = H->time_sweep(state, part, std::vector<SweepGeom>(H->npop, g), false, &t);
          if (e == cudaSuccess && t > 0 && (best == 0 || t < best)) {
            best = t;
            best_G = G;
          }
        }
        for (int j = 0; j < H->npop; ++j)
          if (part[j]) {
            done[j] = 1;
            PopHost& P = H->pops[j];
            msc_geom(L, &P.geom, best_G);
            geom_to_pop(P.geom, &P.h);
          }
      }
      H->cs = 1;
      if (msc_clusters && e == cudaSuccess) {  // the tuned one-CTA form against clusters of 2 and 4
        std::vector<char> all(H->npop, 1);
        std::vector<SweepGeom> g1(H->npop);
        for (int k = 0; k < H->npop; ++k) g1[k] = H->pops[k].geom;
        double best = 0;
        e = H->time_sweep(state, all, g1, false, &best);
        for (int tcs = 2; tcs <= 4 && e == cudaSuccess; tcs *= 2) {
          std::vector<SweepGeom> gc(H->npop);
          bool ok = true;
          for (int k = 0; k < H->npop; ++k) ok = ok && msc_cluster_geom(H->pops[k].cfg.L, tcs, 256, &gc[k]);
          if (!ok) continue;
          double t = 0;
          e = H->time_sweep(state, all, gc, false, &t, tcs, 256);
          if (e == cudaSuccess && t > 0 && (best == 0 || t < best)) {
            best = t;
            H->cs = tcs;
            for (int k = 0; k < H->npop; ++k) {
              H->pops[k].geom = gc[k];
              geom_to_pop(gc[k], &H->pops[k].h);
            }
          }
        }
        H->cthreads = 256;
      }
    } else if (msc_large) {  // clusters of 2 against clusters of 4
      std::vector<char> all(H->npop, 1);
      double best = 0;
      for (int tcs = 2; tcs <= 4 && e == cudaSuccess; tcs *= 2) {
        const int th = msc_cluster_threads(tcs, maxL);
        std::vector<SweepGeom> gc(H->npop);
        for (int k = 0; k < H->npop; ++k) msc_cluster_geom(H->pops[k].cfg.L, tcs, th, &gc[k]);
        double t = 0;
        e = H->time_sweep(state, all, gc, false, &t, tcs, th);
        if (e == cudaSuccess && t > 0 && (best == 0 || t < best)) {
          best = t;
          H->cs = tcs;
          H->cthreads = th;
          for (int k = 0; k < H->npop; ++k) {
            H->pops[k].geom = gc[k];
            geom_to_pop(gc[k], &H->pops[k].h);
          }
        }
      }
    } else {  // SSC: bit-plane replicas per tile for every lattice size, then the form of the batch
      std::vector<char> all(H->npop, 1);
      std::vector<SweepGeom> g8(H->npop), gb(H->npop);
      for (int k = 0; k < H->npop; ++k) ssc_geom(H->pops[k].cfg.L, &g8[k]);
      std::vector<int> done(H->npop, 0);
      for (int k = 0; k < H->npop && e == cudaSuccess; ++k) {
        if (done[k]) continue;
        const int L = H->pops[k].cfg.L;
        std::vector<char> part(H->npop, 0);
        for (int j = 0; j < H->npop; ++j) part[j] = H->pops[j].cfg.L == L;
        SweepGeom best_g;
        ssc_bits_geom(L, &best_g);  // the largest tile
        double best = 0;
        for (int t = best_g.G; t >= 1 && e == cudaSuccess; t /= 2) {
          SweepGeom g;
          if (!ssc_bits_geom(L, &g, t)) continue;
          double tt = 0;
          e = H->time_sweep(state, part, std::vector<SweepGeom>(H->npop, g), true, &tt);
          if (e == cudaSuccess && tt > 0 && (best == 0 || tt < best)) {
            best = tt;
            best_g = g;
          }
        }
        for (int j = 0; j < H->npop; ++j)
          if (part[j]) {
            done[j] = 1;
            gb[j] = best_g;
          }
      }
      double t8 = 0, tb = 0;
      if (e == cudaSuccess) e = H->time_sweep(state, all, g8, false, &t8);
      if (e == cudaSuccess) e = H->time_sweep(state, all, gb, true, &tb);
      if (e == cudaSuccess) {
        H->ssc_bits = tb > 0 && (t8 <= 0 || tb <= t8);
        for (int k = 0; k < H->npop; ++k) {
          PopHost& P = H->pops[k];
          P.geom = H->ssc_bits ? gb[k] : g8[k];
          geom_to_pop(P.geom, &P.h);
        }
      }
    }
    // the run starts from the configured state again (stream positions included)
    std::vector<PopDev> hp(H->npop);
    for (int k = 0; k < H->npop; ++k) hp[k] = H->pops[k].h;
    if (e == cudaSuccess) e = H->upload_pops(hp);
    if (e == cudaSuccess) e = H->setup_launches();
    if (e != cudaSuccess) return H->cuda_fail(e, "autotune");
  }
  for (int k = 0; k < H->npop; ++k)
    if (H->pops[k].user_index < n) tiles[H->pops[k].user_index] = H->pops[k].geom.G;
  return PA_OK;
}

int pa_sweep_form(const pa_handle* H, int index, pa_sweep_form_t* out) {
  if (!H || !out) return PA_ERR_ARG;
  for (const auto& P : H->pops)
    if (P.user_index == index) {
      const bool msc = P.cfg.coding == PA_CODING_MSC;
      out->spins_per_word = msc ? kMsb : (H->ssc_bits ? 32 : 4);
      out->replicas_per_word = msc ? kMsb : 1;
      out->tile = P.geom.G;
      out->cluster_ctas = msc ? H->cs : 1;
      return PA_OK;
    }
  return PA_ERR_ARG;
}

int pa_num_rows(const pa_handle* H, int* n) {
  if (!H || !n) return PA_ERR_ARG;
  int m = 0;
  if (H->sets_done > 0) {  // rows of the last run (adaptive schedules are known only then)
    for (int s = 0; s < H->sets_done; ++s) m = std::max(m, (int)(H->rows[s].size() / kRowCols));
  } else {
    for (const auto& P : H->pops) m = std::max(m, P.cfg.adaptive ? P.cap : (int)P.betas.size());
  }
  *n = m;
  return PA_OK;
}

int pa_get_rows(const pa_handle* H, int set, pa_row* rows, int max_rows, int* nrows) {
  if (!H || !rows) return PA_ERR_ARG;
  if (set < 0 || set >= H->sets_done) return PA_ERR_STATE;
  const std::vector<double>& src = H->rows[set];
  const int n = (int)(src.size() / kRowCols);
  const int m = n < max_rows ? n : max_rows;
  for (int i = 0; i < m; ++i) std::memcpy(&rows[i], src.data() + (size_t)i * kRowCols, sizeof(pa_row));
  if (nrows) *nrows = m;
  return PA_OK;
}

int pa_get_mhr_rows(const pa_handle* H, int set, double* rows, int max_rows, int* nrows) {
  if (!H || (max_rows > 0 && !rows)) return PA_ERR_ARG;
  if (set < 0 || set >= H->sets_done || H->mhr[set].empty()) return PA_ERR_STATE;
  const std::vector<double>& src = H->mhr[set];
  const int n = (int)(src.size() / 4), m = std::min(n, max_rows);
  if (m > 0) std::memcpy(rows, src.data(), sizeof(double) * 4 * (size_t)m);
  if (nrows) *nrows = n;
  return PA_OK;
}

int pa_set_lattice_dump(pa_handle* H, const char* dir, int precision) {
  if (!H) return PA_ERR_ARG;
  if (dir && H->npop != 1) {
    H->err = "lattice dumps need a handle with one population";
    return PA_ERR_ARG;
  }
  H->lattice_dir = dir ? dir : "";
  H->lattice_prec = precision > 0 ? precision : 11;
  return PA_OK;
}

int pa_get_family_rows(const pa_handle* H, int set, double* rows, int max_rows, int* nrows) {
  if (!H || (max_rows > 0 && !rows)) return PA_ERR_ARG;
  if (set < 0 || set >= H->sets_done || H->fam[set].empty()) return PA_ERR_STATE;
  const std::vector<double>& src = H->fam[set];
  const int n = (int)(src.size() / 3), m = std::min(n, max_rows);
  if (m > 0) std::memcpy(rows, src.data(), sizeof(double) * 3 * (size_t)m);
  if (nrows) *nrows = n;
  return PA_OK;
}

int pa_get_energies(const pa_handle* H, int set, int step, int32_t* out, int max, int* n) {
  if (!H || (max > 0 && !out)) return PA_ERR_ARG;
  if (set < 0 || set >= H->sets_done) return PA_ERR_STATE;
  const auto& per = H->energies[set];
  if (step < 0 || step >= (int)per.size()) return per.empty() ? PA_ERR_STATE : PA_ERR_ARG;
  const std::vector<int32_t>& e = per[step];
  const int k = std::min((int)e.size(), max);
  if (k > 0) std::memcpy(out, e.data(), sizeof(int32_t) * (size_t)k);
  if (n) *n = (int)e.size();
  return PA_OK;
}

int pa_get_timing(const pa_handle* H, double* ms, double* attempts) {
  if (!H) return PA_ERR_ARG;
  if (ms) *ms = H->ms;
  if (attempts) *attempts = H->attempts;
  return PA_OK;
}

int pa_set_population(pa_handle* H, const void* host) {
  if (!H) return PA_ERR_ARG;
  cudaError_t e = cudaSuccess;
  const char* src = (const char*)host;
  for (int u = 0; u < H->npop && e == cudaSuccess; ++u) {  // populations in user order
    int k = 0;
    while (H->pops[k].user_index != u) ++k;
    PopHost& P = H->pops[k];
    const void* dev = nullptr;
    if (host) {
      const size_t bytes = population_bytes(H->coding, P.cfg.L, P.cfg.R);
      if (!H->staging[k]) e = cudaMalloc(&H->staging[k], bytes);
      if (e == cudaSuccess) e = cudaMemcpyAsync(H->staging[k], src, bytes, cudaMemcpyHostToDevice, H->stream);
      src += bytes;
      dev = H->staging[k];
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&H->d_pops[k].init_src, &dev, sizeof(dev), cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);  // `dev` lives on this stack frame
    P.h.init_src = dev;
  }
  if (e != cudaSuccess) return H->cuda_fail(e, "set population");
  return PA_OK;
}

int pa_get_population(const pa_handle* H, int pop, void* host, size_t bytes, int* R) {
  if (!H || !host || pop < 0 || pop >= H->npop) return PA_ERR_ARG;
  if (H->sets_done == 0) return PA_ERR_STATE;
  int k = 0;
  while (H->pops[k].user_index != pop) ++k;
  PopDev st;
  cudaError_t e = cudaMemcpy(&st, H->d_pops + k, sizeof(PopDev), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return PA_ERR_CUDA;
  const size_t need = population_bytes(H->coding, st.L, st.R_cur);
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
  if (e == cudaSuccess) e = H->enqueue_run();
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

int pa_write_results(const pa_handle* H, const char* dir, int precision) {
  if (!H || !dir) return PA_ERR_ARG;
  if (H->sets_done == 0) return PA_ERR_STATE;
  for (int r = 0; r < H->sets_done; ++r) {
    std::string path = std::string(dir);
    if (!path.empty() && path.back() != '/') path += '/';
    path += "PA_results_run_" + std::to_string(r) + ".dat";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return PA_ERR_ARG;
    const std::vector<double>& o = H->rows[r];
    const int n = (int)(o.size() / kRowCols);
    for (int i = 0; i < n; ++i) {
      const double* w = o.data() + (size_t)i * kRowCols;
      for (int k = 0; k < 8; ++k) std::fprintf(f, "%.*g ", precision, w[k]);
      std::fprintf(f, "%d %.*g\n", (int)w[8], precision, w[9]);
    }
    std::fclose(f);
    // PA_MHR_results_run_<r>.dat: beta E/N C/N betaF/N (PAisingSSC.cu:768-786)
    if (!H->mhr[r].empty()) {
      std::string mp = path.substr(0, path.rfind('/') + 1) + "PA_MHR_results_run_" + std::to_string(r) + ".dat";
      FILE* g = std::fopen(mp.c_str(), "w");
      if (!g) return PA_ERR_ARG;
      const std::vector<double>& m = H->mhr[r];
      for (size_t i = 0; i < m.size() / 4; ++i) {
        for (int k = 0; k < 4; ++k) std::fprintf(g, "%.*g ", precision, m[i * 4 + k]);
        std::fprintf(g, "\n");
      }
      std::fclose(g);
    }
    // PA_family_run_<r>.dat: beta, families, rho_t, S_f (no reference counterpart)
    if (!H->fam[r].empty()) {
      std::string fp = path.substr(0, path.rfind('/') + 1) + "PA_family_run_" + std::to_string(r) + ".dat";
      FILE* g = std::fopen(fp.c_str(), "w");
      if (!g) return PA_ERR_ARG;
      const std::vector<double>& fr = H->fam[r];
      for (size_t i = 0; i < fr.size() / 3; ++i)
        std::fprintf(g, "%.*g %d %.*g %.*g\n", precision, o[i * kRowCols], (int)fr[i * 3], precision, fr[i * 3 + 1],
                     precision, fr[i * 3 + 2]);
      std::fclose(g);
    }
  }
  // PA_energies_<i>.dat: energies of temperature i >= 1, space separated, of
  // the last run (each run overwrites them, PAisingSSC.cu:563-578); one
  // population per handle, as the files carry no population index
  if (H->npop == 1 && !H->energies[H->sets_done - 1].empty()) {
    const auto& per = H->energies[H->sets_done - 1];
    for (size_t i = 1; i < per.size(); ++i) {
      std::string ep = std::string(dir);
      if (!ep.empty() && ep.back() != '/') ep += '/';
      ep += "PA_energies_" + std::to_string(i) + ".dat";
      FILE* g = std::fopen(ep.c_str(), "w");
      if (!g) return PA_ERR_ARG;
      for (int32_t v : per[i]) std::fprintf(g, "%d ", (int)v);
      std::fclose(g);
    }
  }
  return PA_OK;
}

int pa_destroy(pa_handle* H) {
  delete H;
  return PA_OK;
}

}  // extern "C"
