// pa_resample.cu -- resampling of the populations on the device, no host
// round trip, the per-temperature bookkeeping, and the batch launchers.
//
// Replaces, from the reference (both codings):
//   QKer        (PAisingSSC.cu:217-234, PAisingMSC.cu:319-345) + host lnQ
//               (PAisingSSC.cu:533)                  -> q_kernel
//   CalcTauKer  (PAisingSSC.cu:236-254, PAisingMSC.cu:347-360)
//   + CalcParSum block totals                        -> copy_numbers_kernel
//   CalcParSum  (PAisingSSC.cu:256-270, PAisingMSC.cu:362-395)
//                                                    -> scatter_kernel (exclusive
//               scan + map new replica -> old replica, consumed by the gathers)
//   CalcAverages + host observables (PAisingSSC.cu:282-292, 614-630)
//                                                    -> finish_step_kernel (sums
//               are accumulated exactly in integers by the sweep kernels)
//
// Population p of a batch is handled by the blocks with blockIdx.y == p.
// Every multi-block reduction ends with the last-block pattern: each block
// publishes its partial result, takes a ticket, and the block that draws the
// last ticket combines the partials in block order.  Results therefore do not
// depend on block scheduling, and no block ever waits for another.
#include <cfloat>
#include <climits>
#include <cmath>

#include "pa_device.cuh"
#include "pa_kernels.h"
#include "pa_thresholds.h"

namespace pa {

namespace {

constexpr int kResThreads = 256;

__device__ __forceinline__ int pop_units(const PopDev* st, int R) {
  return st->coding == kMSC ? ((R + kMsb - 1) / kMsb) * kMsb : R;
}

// Neumaier's variant of Kahan compensated summation, FP32.
struct Comp32 {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    if (fabsf(s) >= fabsf(x))
      c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, t), x));
    else
      c = __fadd_rn(c, __fadd_rn(__fsub_rn(x, t), s));
    s = t;
  }
};

// resampling weight of one replica in FP32: exp(-dbeta (E - Emin)) <= 1
__device__ __forceinline__ float weight32(float dBf, int E, int Emin) {
  return expf(-dBf * (float)(E - Emin));
}

// last-block ticket: returns true in every thread of the block that finished
// last among the gridDim.x blocks of its population
__device__ __forceinline__ bool last_block(unsigned int* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  return s_last;
}

// contiguous chunk of [0, n) owned by this block, a whole number of tiles
__device__ __forceinline__ void block_chunk(int n, int& lo, int& hi) {
  const int per = (n + gridDim.x - 1) / gridDim.x;
  const int c = (per + blockDim.x - 1) / blockDim.x * blockDim.x;
  lo = min(n, (int)blockIdx.x * c);
  hi = min(n, lo + c);
}

}  // namespace

// ------------------------------------------------------------------------ Q
// q = sum_j w_j over the population before resampling, then
//   lnQ = -dbeta E_ref + ln q - ln R_prev            (PAisingSSC.cu:533)
// FP64 weights: w = exp(-dbeta (E - Emean)), E_ref = Emean (the reference's
// choice, PAisingSSC.cu:222).  FP32 weights: w = exp(-dbeta (E - Emin)) <= 1,
// compensated sums, E_ref = Emin; lnQ itself is formed in FP64.
__global__ void __launch_bounds__(kResThreads) q_kernel(PopDev* pops) {
  __shared__ double s_d[33];
  __shared__ float s_f[2][kResThreads];
  PopDev* st = pops + blockIdx.y;
  if (!pop_stepping(st)) return;
  const int step = st->step, Rp = st->R_prev, n = pop_units(st, Rp);
  const double dB = st->betas[step] - st->betas[step - 1];
  const uint8_t* act = st->coding == kMSC ? st->active[st->parity] : nullptr;
  const int32_t* E = st->E;
  const int tid = threadIdx.x;
  if (st->weights == kFP64) {
    const double Em = st->Emean;
    double v = 0.0;
    for (int j = blockIdx.x * blockDim.x + tid; j < n; j += gridDim.x * blockDim.x)
      if (!act || act[j]) v += exp(-dB * (E[j] - Em));
    v = block_sum(v, s_d);
    if (tid == 0) st->qpart_d[blockIdx.x] = v;
    if (last_block(&st->ticket)) {
      double a = 0.0;
      for (int bb = tid; bb < (int)gridDim.x; bb += blockDim.x) a += ((volatile double*)st->qpart_d)[bb];
      a = block_sum(a, s_d);
      if (tid == 0) {
        st->q = a;
        st->lnQ = -(st->betas[step] - st->betas[step - 1]) * Em + log(a) - log((double)Rp);
        st->ticket = 0;
      }
    }
  } else {
    const int Emin = st->Emin;
    const float dBf = (float)dB;
    Comp32 acc;
    for (int j = blockIdx.x * blockDim.x + tid; j < n; j += gridDim.x * blockDim.x)
      if (!act || act[j]) acc.add(weight32(dBf, E[j], Emin));
    s_f[0][tid] = acc.s;
    s_f[1][tid] = acc.c;
    __syncthreads();
    if (tid == 0) {
      Comp32 bsum;
      float c = 0.f;
      for (int i = 0; i < (int)blockDim.x; ++i) { bsum.add(s_f[0][i]); c = __fadd_rn(c, s_f[1][i]); }
      st->qpart_f[2 * blockIdx.x] = bsum.s;
      st->qpart_f[2 * blockIdx.x + 1] = __fadd_rn(bsum.c, c);
    }
    if (last_block(&st->ticket)) {
      // thread t sums the partials of blocks t, t + 256, ... (all loads in
      // flight at once), thread 0 then the 256 thread sums in thread order:
      // a fixed order, so the result does not depend on block scheduling
      Comp32 t;
      float c = 0.f;
      const volatile float* qp = st->qpart_f;
      for (int bb = tid; bb < (int)gridDim.x; bb += blockDim.x) {
        t.add(qp[2 * bb]);
        c = __fadd_rn(c, qp[2 * bb + 1]);
      }
      __syncthreads();  // the block sums above are done with s_f
      s_f[0][tid] = t.s;
      s_f[1][tid] = __fadd_rn(t.c, c);
      __syncthreads();
      if (tid == 0) {
        Comp32 u;
        float cc = 0.f;
        for (int i = 0; i < (int)blockDim.x; ++i) { u.add(s_f[0][i]); cc = __fadd_rn(cc, s_f[1][i]); }
        const float q = __fadd_rn(u.s, __fadd_rn(u.c, cc));
        st->q = (double)q;
        st->lnQ = -dB * (double)Emin + log((double)q) - log((double)Rp);
        st->ticket = 0;
      }
    }
  }
}

// ------------------------------------------------------------ copy numbers
// Nearest-integer resampling (PAisingSSC.cu:242-247):
//   mu_j = R_init / R_prev * exp(-dbeta E_j - lnQ),
//   roff_j = floor(mu_j) + [U_j < mu_j - floor(mu_j)],
// U_j the reference's draw 0 of subsequence iseq + j (j = linear replica
// index; for MSC j = 32 * group + bit, PAisingMSC.cu:355).  Block totals are
// scanned by the last block, which also publishes the new population size
// and flips the double buffer.
__global__ void __launch_bounds__(kResThreads) copy_numbers_kernel(PopDev* pops) {
  __shared__ uint32_t s_u[33];
  __shared__ uint32_t s_run;
  PopDev* st = pops + blockIdx.y;
  if (!pop_stepping(st)) return;
  const int step = st->step, Rp = st->R_prev, n = pop_units(st, Rp), Rinit = st->Rinit;
  const double dB = st->betas[step] - st->betas[step - 1], lnQ = st->lnQ;
  const uint8_t* act = st->coding == kMSC ? st->active[st->parity] : nullptr;
  const int32_t* E = st->E;
  const unsigned long long seed = st->seed, iseq = st->iseq;
  const bool fp64 = st->weights == kFP64;
  const float dBf = (float)dB, qf = (float)st->q, Rf = (float)Rinit;
  const int Emin = st->Emin;
  int lo, hi;
  block_chunk(n, lo, hi);
  uint32_t tot = 0;
  for (int base = lo; base < hi; base += blockDim.x) {
    const int j = base + threadIdx.x;
    uint32_t r = 0;
    if (j < hi && (!act || act[j])) {
      const double U = ref_uniform(ref_word(seed, iseq + (unsigned long long)j, 0));
      if (fp64) {
        const double mu = ((double)Rinit) / Rp * exp(-dB * (double)E[j] - lnQ);
        const double fl = floor(mu);
        r = (uint32_t)(U < (mu - fl) ? fl + 1 : fl);
      } else {
        const float mu = Rf * weight32(dBf, E[j], Emin) / qf;
        const float fl = floorf(mu);
        r = (uint32_t)fl + (U < (double)(mu - fl) ? 1u : 0u);
      }
    }
    if (j < hi) st->roff[j] = r;
    tot += block_sum(r, s_u);
  }
  if (threadIdx.x == 0) st->blk_tot[blockIdx.x] = tot;
  if (last_block(&st->ticket)) {
    // exclusive scan of the block totals, in block order
    if (threadIdx.x == 0) s_run = 0;
    __syncthreads();
    for (int b0 = 0; b0 < (int)gridDim.x; b0 += blockDim.x) {
      const int bb = b0 + threadIdx.x;
      const uint32_t v = bb < (int)gridDim.x ? ((volatile uint32_t*)st->blk_tot)[bb] : 0u;
      uint32_t total;
      const uint32_t ex = block_exscan(v, s_u, &total);
      if (bb < (int)gridDim.x) st->blk_off[bb] = s_run + ex;
      __syncthreads();
      if (threadIdx.x == 0) s_run += total;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const unsigned int Rn = s_run;
      if (Rn == 0u || Rn > (unsigned int)st->Rcap) {
        st->error = Rn == 0u ? 2 : 1;
        st->R_cur = 0;
      } else {
        st->R_cur = (int)Rn;
      }
      st->parity ^= 1;
      st->ticket = 0;
    }
  }
}

// ------------------------------------------------------------------ scatter
// offs_j = exclusive prefix of roff; src[offs_j + p] = j for p < roff_j.
// The new replicas of a tile of 256 old ones are filled by the whole block,
// new index i taking the last old replica of the tile whose offset is <= i
// (a binary search over the tile's offsets in shared memory): one old
// replica with thousands of copies -- a large dbeta against the energy
// spread makes them -- costs the block a few passes instead of leaving one
// thread to write them all.
__global__ void __launch_bounds__(kResThreads) scatter_kernel(PopDev* pops) {
  __shared__ uint32_t s_u[33];
  __shared__ uint32_t s_off[kResThreads + 1];
  PopDev* st = pops + blockIdx.y;
  if (!pop_stepping(st)) return;
  const int n = pop_units(st, st->R_prev);
  int lo, hi;
  block_chunk(n, lo, hi);
  uint32_t run = st->blk_off[blockIdx.x];
  const int nt = blockDim.x;
  for (int base = lo; base < hi; base += nt) {
    const int j = base + threadIdx.x;
    const uint32_t r = j < hi ? st->roff[j] : 0u;
    uint32_t total;
    const uint32_t off = run + block_exscan(r, s_u, &total);
    if (j < hi) st->offs[j] = off;
    s_off[threadIdx.x] = off;  // non-decreasing; equal to run + total past hi
    if (threadIdx.x == 0) s_off[nt] = run + total;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < total; t += nt) {
      const uint32_t i = run + t;
      // last k with s_off[k] <= i: s_off[0] = run <= i < s_off[nt]
      int a = 0, b = nt;
      while (b - a > 1) {
        const int m = (a + b) >> 1;
        if (s_off[m] <= i) a = m;
        else b = m;
      }
      st->src[i] = (uint32_t)(base + a);
    }
    __syncthreads();
    run += total;
  }
}

// ------------------------------------------------------------- sweep plan
// Unit counts of the populations that take part in the next sweep launch,
// their exclusive prefix sums, and a fresh work queue.
__global__ void __launch_bounds__(1024) plan_kernel(BatchDev* b, int energy_only) {
  __shared__ uint32_t s_u[33];
  const int p = threadIdx.x, np = b->npop;
  uint32_t units = 0;
  if (p < np) {
    const PopDev* st = b->pops + p;
    const bool part = energy_only ? (st->step == 0) : pop_stepping(st);
    if (part) {
      const int gpt = st->gpt > 0 ? st->gpt : 1;
      units = st->coding == kMSC ? (uint32_t)(((st->R_cur + kMsb - 1) / kMsb + gpt - 1) / gpt)
                                 : (uint32_t)((st->R_cur + gpt - 1) / gpt);
    }
  }
  uint32_t total;
  const uint32_t ex = block_exscan(units, s_u, &total);
  if (p < np) b->unit_prefix[p] = (int)ex;
  if (p == 0) {
    b->unit_prefix[np] = (int)total;
    b->work_next = 0;
  }
}

// --------------------------------------------------------- run bookkeeping
__global__ void begin_run_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.x;
  st->step = 0;
  st->run += 1;  // -1 at creation: the first run is run 0
  st->R_prev = st->R_cur = st->Rinit;
  st->parity = 0;
  st->error = 0;
  st->Emean = 0.0;  // the first resampling uses Emean = 0 (PAisingSSC.cu:483)
  st->Emin = 0;
  st->sumlnQ = 0.0;
  st->lnQ = 0.0;
  st->q = 0.0;
  st->sE = st->sE2 = st->sM = st->sM2 = 0;
  st->sM4lo = st->sM4hi = 0;
  st->Emin_acc = INT_MAX;
  st->ticket = 0;
  double* row = st->rows;  // beta = 0 row: only betaF and R are defined (PAisingSSC.cu:435,453)
  for (int c = 0; c < kRowCols; ++c) row[c] = 0.0;
  row[6] = st->bf0 / st->N;
  row[8] = (double)st->Rinit;
  st->last_rec = -1;
  st->last_fam = -1;
}

// ------------------------------------------------------ family statistics
// Not written by the reference: with c_f the replicas descended from initial
// replica f and R the population size, every temperature records
//   {families with c_f > 0, rho_t = sum_f c_f^2 / R,
//    S_f = -sum_f (c_f/R) ln(c_f/R) = ln R - (1/R) sum_f c_f ln c_f}.
// Ancestors are initial linear replica indices (MSC: 32 * group + bit) and
// follow every copy the resampling makes.

// After the initial population: every replica is its own family.
__global__ void family_init_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  if (!st->family) return;
  const int n = pop_units(st, st->R_cur), R = st->R_cur;
  int32_t* a = st->anc[st->parity];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) a[j] = j < R ? j : -1;
}

// After the spin gather of a temperature step: new replica slots take the
// ancestor of their source (SSC, and MSC with the native stream: slot s <-
// src[s]; MSC with the reference stream: slot 32 g + b holds offspring
// s = b rg_new + g, PAisingMSC.cu:413-414).
__global__ void family_resample_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  if (!st->family || !pop_stepping(st)) return;
  const int Rn = st->R_cur, n = pop_units(st, Rn);
  const int32_t* old = st->anc[st->parity ^ 1];
  int32_t* neu = st->anc[st->parity];
  const uint32_t* src = st->src;
  const bool transposed = st->coding == kMSC && st->rng_mode == kRefCoords;
  const int rgn = (Rn + kMsb - 1) / kMsb;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int s = transposed ? (j & (kMsb - 1)) * rgn + (j >> 5) : j;
    neu[j] = s < Rn ? old[src[s]] : -1;
  }
}

// After finish_step: count the families of the temperature just finished
// (once per temperature, like the records) ...
__global__ void __launch_bounds__(kResThreads) family_count_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  const int s = st->step - 1;
  if (!st->family || s <= st->last_fam || st->error) return;
  const int n = pop_units(st, st->R_cur);
  const int32_t* a = st->anc[st->parity];
  const uint8_t* act = st->coding == kMSC ? st->active[st->parity] : nullptr;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    if ((!act || act[j]) && a[j] >= 0) atomicAdd(&st->fam_cnt[a[j]], 1u);
}

// ... then reduce the counts (clearing them for the next temperature); the
// last block combines the per-block partial sums in block order.
__global__ void __launch_bounds__(kResThreads) family_reduce_kernel(PopDev* pops) {
  __shared__ double s_d[33];
  PopDev* st = pops + blockIdx.y;
  const int s = st->step - 1;
  if (!st->family || s <= st->last_fam || st->error) return;
  const int nf_bins = st->Rinit;
  double nf = 0.0, c2 = 0.0, clnc = 0.0;
  int lo, hi;
  block_chunk(nf_bins, lo, hi);
  for (int f = lo + (int)threadIdx.x; f < hi; f += blockDim.x) {
    const uint32_t c = st->fam_cnt[f];
    if (!c) continue;
    st->fam_cnt[f] = 0u;
    const double cd = (double)c;
    nf += 1.0;
    c2 += cd * cd;
    clnc += cd * log(cd);
  }
  nf = block_sum(nf, s_d);
  c2 = block_sum(c2, s_d);
  clnc = block_sum(clnc, s_d);
  if (threadIdx.x == 0) {
    st->fam_part[3 * blockIdx.x] = nf;
    st->fam_part[3 * blockIdx.x + 1] = c2;
    st->fam_part[3 * blockIdx.x + 2] = clnc;
  }
  if (last_block(&st->ticket) && threadIdx.x == 0) {
    double a = 0.0, b2 = 0.0, c = 0.0;
    const volatile double* p = st->fam_part;
    for (int k = 0; k < (int)gridDim.x; ++k) { a += p[3 * k]; b2 += p[3 * k + 1]; c += p[3 * k + 2]; }
    const double R = (double)st->R_cur;
    double* row = st->fam_rows + (size_t)s * 3;
    row[0] = a;
    row[1] = b2 / R;
    row[2] = log(R) - c / R;
    st->last_fam = s;
    st->ticket = 0;
  }
}

// ---------------------------------------------- per-temperature records
// After finish_step: the population of temperature step-1, if not recorded
// yet in this run, enters the run's energy histogram (UpdateShistE,
// PAisingSSC.cu:296-302, PAisingMSC.cu:454-460: active replicas only) and/or
// the energy ring (EnergiesPopStore, PAisingSSC.cu:563-578: energies in
// replica order; MSC group-major with the active flags).  The last block to
// finish (ticket) marks the temperature recorded, so every block has tested
// the guard before it changes.
__global__ void __launch_bounds__(kResThreads) record_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  const int s = st->step - 1;
  if (!st->rec || s <= st->last_rec || st->error) return;
  const int R = st->R_cur, n = pop_units(st, R), N = st->N;
  const bool msc = st->coding == kMSC;
  const uint8_t* act = msc ? st->active[st->parity] : nullptr;
  const int32_t* E = st->E;
  int32_t* el = nullptr;
  uint8_t* al = nullptr;
  if (st->rec & kRecEnergies) {
    const size_t stride = msc ? (size_t)st->rgcap * kMsb : (size_t)st->Rcap;
    const size_t slot = (size_t)(s % st->ring) * stride;
    el = st->elog + slot;
    if (msc) al = st->alog + slot;
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int e = E[j];
    const bool a = !act || act[j];
    if ((st->rec & kRecMhr) && a) atomicAdd(&st->mhr_hist[(e + 2 * N) >> 2], 1ull);
    if (el) el[j] = e;
    if (al) al[j] = a ? 1 : 0;
  }
  if (last_block(&st->ticket)) {
    if (threadIdx.x == 0) {
      if (el) st->nlog[s % st->ring] = n;
      st->last_rec = s;
      st->ticket = 0;
    }
  }
}

// After a sweep kernel: observables of the step (PAisingSSC.cu:620-630)
// written to the output row, state advanced to the next temperature.  The
// arithmetic uses explicitly rounded operations so that no multiply-add is
// fused and the row is identical to an unfused host evaluation.
__global__ void finish_step_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.x;
  const int step = st->step;
  if (step > st->nsteps) return;  // this population's schedule is complete
  const bool msc = st->coding == kMSC;
  if (step == 0) {
    const int rg = (st->R_cur + kMsb - 1) / kMsb;
    st->iseq += (unsigned long long)(msc ? rg : st->R_cur) * kRefThreads;  // ReplicaInit draws
    st->Emin = st->Emin_acc;
  } else if (!st->error) {
    const int R = st->R_cur, Rp = st->R_prev, N = st->N;
    const double Rd = (double)R, Nd = (double)N, b = st->betas[step];
    const double E = __ddiv_rn((double)st->sE, Rd);
    const double C = __dmul_rn(__dmul_rn(__dsub_rn(__ddiv_rn((double)st->sE2, Rd), __dmul_rn(E, E)), b), b);
    const double Mv = __ddiv_rn((double)st->sM, Rd);
    const double M2 = __ddiv_rn((double)st->sM2, Rd);
    const double M4 = __ddiv_rn(u128_to_double(st->sM4lo, st->sM4hi), Rd);
    const double lnQ = st->lnQ;
    const double sum = __dsub_rn(st->sumlnQ, lnQ);
    const double BF = __dadd_rn(st->bf0, sum);
    const double S = __dsub_rn(__dmul_rn(b, E), BF);
    double* row = st->rows + (size_t)step * kRowCols;
    row[0] = b;
    row[1] = __ddiv_rn(E, Nd);
    row[2] = __ddiv_rn(C, Nd);
    row[3] = __ddiv_rn(Mv, Nd);
    row[4] = __ddiv_rn(__ddiv_rn(M2, Nd), Nd);
    row[5] = __ddiv_rn(__ddiv_rn(__ddiv_rn(__ddiv_rn(M4, Nd), Nd), Nd), Nd);
    row[6] = __ddiv_rn(BF, Nd);
    row[7] = __ddiv_rn(S, Nd);
    row[8] = Rd;
    row[9] = lnQ;
    st->sumlnQ = sum;
    st->Emean = E;
    st->Emin = st->Emin_acc;
    const int rgp = (Rp + kMsb - 1) / kMsb, rgc = (R + kMsb - 1) / kMsb;
    st->iseq += msc ? (unsigned long long)rgp * kMsb + (unsigned long long)rgc * kRefThreads
                    : (unsigned long long)Rp + (unsigned long long)R * kRefThreads;
    st->R_prev = R;
  }
  st->step = step + 1;
  st->sE = st->sE2 = st->sM = st->sM2 = 0;
  st->sM4lo = st->sM4hi = 0;
  st->Emin_acc = INT_MAX;
}

// ------------------------------------------------- adaptive temperature step
// After temperature step-1 (>= 1) of an adaptive population: the next beta,
// as the reference's AdaptiveStep build chooses it (PAisingSSC.cu:644-660):
// starting from the previous step, grow it by 1.1x while the energy-histogram
// overlap stays >= MaxOverlap (and beta stays below beta_final), otherwise
// bisect between 0 and the step until MinOverlap <= overlap < MaxOverlap,
// and clamp the last step onto beta_final.  The overlap of step dB
// (CalcOverlap, PAisingSSC.cu:316-334) is
//   lnQ = -dB Emean + ln sum_i exp(-dB (E_i - Emean)) - ln R,
//   overlap = (1/R) sum_i min(1, Rinit/R exp(-dB E_i - lnQ)),
// evaluated here over the histogram of the population's energies (energies
// are -2N + 4k), so each evaluation costs a pass over at most N+1 bins
// instead of R replicas; one CTA per population, FP64 throughout.
constexpr int kAdaptThreads = 1024;
constexpr int kMaxBisect = 200;  // the reference bisects without a bound

__global__ void __launch_bounds__(kAdaptThreads) adapt_kernel(PopDev* pops) {
  __shared__ double s_red[32];
  PopDev* st = pops + blockIdx.x;
  const int step = st->step;  // index of the temperature to choose (finish_step has advanced it)
  if (!st->adaptive || step < 2 || step > st->nsteps || st->error) return;
  const int N = st->N, nb = N + 1, R = st->R_cur;
  uint32_t* hist = st->hist;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) hist[i] = 0u;
  __syncthreads();
  const bool msc = st->coding == kMSC;
  const int units = pop_units(st, R);
  const uint8_t* act = msc ? st->active[st->parity] : nullptr;
  for (int i = threadIdx.x; i < units; i += blockDim.x)
    if (!msc || act[i]) atomicAdd(&hist[(st->E[i] + 2 * N) >> 2], 1u);
  __syncthreads();

  const double Em = st->Emean, Rd = (double)R, Rinit = (double)st->Rinit;
  auto overlap = [&](double dB) {
    double q = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      const uint32_t c = hist[i];
      if (c) q += (double)c * exp(-dB * ((double)(4 * i - 2 * N) - Em));
    }
    q = block_sum(q, s_red);
    const double lnQ = -dB * Em + log(q) - log(Rd);
    double o = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      const uint32_t c = hist[i];
      if (c) o += (double)c * fmin(1.0, Rinit / Rd * exp(-dB * (double)(4 * i - 2 * N) - lnQ));
    }
    return block_sum(o, s_red) / Rd;
  };

  const double Bp = st->betas[step - 1], Bfin = st->beta_fin, lo = st->min_ov, hi = st->max_ov;
  double dBmin = 0.0, dBmax = st->dbeta_cur, dBmean, ov;
  for (;;) {
    ov = overlap(dBmax);
    if (ov >= hi && Bp + dBmax < Bfin) dBmax *= 1.1;
    else break;
  }
  if (ov >= lo) {
    dBmean = dBmax;
  } else {
    for (int it = 0;; ++it) {
      dBmean = 0.5 * (dBmin + dBmax);
      ov = overlap(dBmean);
      if (it + 1 >= kMaxBisect) break;
      if (ov < lo) dBmax = dBmean;
      else if (ov >= hi) dBmin = dBmean;
      else break;
    }
  }
  const double dB = (Bp < Bfin && Bp + dBmean > Bfin) ? Bfin - Bp : dBmean;
  const double Bn = Bp + dB;
  if (threadIdx.x == 0) {
    st->dbeta_cur = dB;
    if (!(Bn <= Bfin)) {
      st->nsteps = step - 1;  // the schedule ends with the temperature just computed
    } else if (step >= kNBmax - 1) {
      st->error = kErrTooManySteps;  // PAisingSSC.cu:634-641
    } else {
      st->betas[step] = Bn;
      thresholds(Bn, st->thr + (size_t)step * kThrPerStep);
    }
  }
}

// ------------------------------------------------------------ launchers
int res_blocks(long long units) {
  long long b = (units + kResThreads - 1) / kResThreads;
  if (b > kResBlocksMax) b = kResBlocksMax;
  return (int)(b < 1 ? 1 : b);
}

void geom_to_pop(const SweepGeom& g, PopDev* h) {
  h->Wr = g.Wr;
  h->rpp = g.rpp;
  h->T = g.T;
  h->npass = g.npass;
  h->kconst = g.kconst;
  h->gpt = g.G;
  h->seg = g.seg;
  h->invL = recip32(g.L);
  h->invWr = recip32(g.Wr);
}

cudaError_t sweep_setup(int coding, int rng_mode, int smem, SweepLaunch* out, int fixed_l) {
  out->fixed_l = 0;
  return coding == kMSC ? msc_sweep_setup(rng_mode, smem, out, fixed_l) : ssc_sweep_setup(rng_mode, smem, out);
}

cudaError_t launch_plan(BatchDev* b, int npop, int energy_only, cudaStream_t s) {
  (void)npop;
  plan_kernel<<<1, 1024, 0, s>>>(b, energy_only);
  return cudaGetLastError();
}

cudaError_t launch_sweep(BatchDev* b, int coding, int rng_mode, int energy_only, unsigned long long seed,
                         const SweepLaunch& sl, cudaStream_t s) {
  return coding == kMSC ? launch_msc_sweep(b, rng_mode, energy_only, seed, sl, s)
                        : launch_ssc_sweep(b, rng_mode, energy_only, seed, sl, s);
}

cudaError_t launch_init(PopDev* pops, int npop, int coding, cudaStream_t s) {
  return coding == kMSC ? launch_msc_init(pops, npop, s) : launch_ssc_init(pops, npop, s);
}

cudaError_t launch_resample(BatchDev* b, int coding, int rng_mode, cudaStream_t s) {
  return coding == kMSC ? launch_msc_resample(b, rng_mode, s) : launch_ssc_resample(b, s);
}

cudaError_t launch_q(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  q_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_copy_numbers(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  copy_numbers_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_scatter(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  scatter_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_begin_run(PopDev* pops, int npop, cudaStream_t s) {
  begin_run_kernel<<<npop, 1, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_finish_step(PopDev* pops, int npop, cudaStream_t s) {
  finish_step_kernel<<<npop, 1, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_family_init(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  family_init_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_family_resample(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  family_resample_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_family_stats(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  family_count_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  family_reduce_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_record(PopDev* pops, int npop, int blocks, cudaStream_t s) {
  record_kernel<<<dim3(blocks, npop), kResThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_adapt(PopDev* pops, int npop, cudaStream_t s) {
  adapt_kernel<<<npop, kAdaptThreads, 0, s>>>(pops);
  return cudaGetLastError();
}

}  // namespace pa
