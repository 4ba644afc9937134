// pa_msc.cu -- multi-spin coding: 32 replicas bit-packed per uint32 word.
//
// Replaces, from the reference PAisingMSC.cu (MSbits = 32):
//   ReplicaInit  (PAisingMSC.cu:169-188)  -> msc_init_kernel
//   checkKerALL  (PAisingMSC.cu:191-266)  -> msc_sweep_kernel (group resident in
//   energyKer    (PAisingMSC.cu:268-317)     shared memory for all sweeps; per
//                                            replica energy and magnetisation by
//                                            warp ballots in the epilogue)
//   resampleKer  (PAisingMSC.cu:397-435)  -> msc_resample_kernel (gather: each new
//                                            word assembles its 32 source bits,
//                                            no atomics, no memset)
//
// Layout in HBM: group g occupies N words at spins + g*N (sublattice A words,
// then B); bit k of a word is replica k of the group, 1 == spin +1.
#include <climits>

#include "pa_kernels.h"
#include "pa_msc_core.cuh"

namespace pa {

using namespace msc;

// ------------------------------------------------------------------ init
__global__ void msc_init_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  const int N = st->N, h = N >> 1, R = st->R_cur, rg = (R + kMsb - 1) / kMsb;
  const unsigned long long seed = st->seed, iseq = st->iseq;
  uint32_t* wd = (uint32_t*)st->spins[st->parity];
  uint8_t* act = st->active[st->parity];
  if (st->init_src) {  // caller-supplied population (replica 32g+k at group g, bit k)
    const uint4* src = (const uint4*)st->init_src;
    uint4* dst = (uint4*)wd;
    const long long nv = (long long)rg * N / 4;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x)
      dst[v] = src[v];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)rg * kMsb;
         i += (long long)gridDim.x * blockDim.x)
      act[i] = i < R;
    return;
  }
  // ReplicaInit (PAisingMSC.cu:169-188): reference thread t of block B draws
  // words 2k (gA) and 2k+1 (gB) of subsequence iseq + t + 128 B for idx = t + 128 k
  const long long total = (long long)rg * h;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(e / h), idx = (int)(e - (long long)g * h);
    const int t = idx & (kRefThreads - 1), k = idx >> 7;
    const unsigned long long sub = iseq + (unsigned long long)t + (unsigned long long)kRefThreads * g;
    wd[(size_t)g * N + idx] = ref_word(seed, sub, 2ull * k);
    wd[(size_t)g * N + h + idx] = ref_word(seed, sub, 2ull * k + 1);
    if (idx < kMsb) act[g * kMsb + idx] = (g * kMsb + idx) < R;
  }
}

// ----------------------------------------------------------------- sweep
// Persistent: every CTA takes groups of 32 replicas of any population from
// the batch's work queue and anneals one group at a time, both sublattices
// resident in shared memory.  Thread (rsub, tx) owns site column tx of
// sublattice rows rsub, rsub+rpp, ...
//
// MODE kRefCoords: decisions of checkKerALL exactly -- one draw per word-site
//   (ctr = sw*2K + hf*K + k of subsequence iseq + t + 128 g) expanded to 32
//   numbers by the LCG and compared with T4 = ceil(2^32 e^-4b), T8.
// MODE kNative: U_i < T/2^32 for the 32 replica bits is decided digit by
//   digit, most significant first, each digit a fresh Philox4x32-10 bit
//   (accept_native); each replica's acceptance probability is exactly
//   T/2^32, as in the reference.  The stream is keyed by stream_seed (one
//   per batch; populations differ in counter word 3).
template <int MODE>
__global__ void __launch_bounds__(kSweepThreads, 5)
    msc_sweep_kernel(BatchDev* b, int energy_only, unsigned long long stream_seed) {
  extern __shared__ __align__(16) uint32_t lat[];  // N words: A then B
  __shared__ int s_unit, s_pop;
  __shared__ int s_cntE[kMsb], s_cntM[kMsb];
  __shared__ uint2 s_dig[kMsb];  // per digit j: (D8_j, D4_j ^ D8_j)
  __shared__ UnitParams P;
  __shared__ BitStats stats;

  const int tid = threadIdx.x, lane = tid & 31;
  const int total = b->unit_prefix[b->npop];
  const PhiloxKeys keys(stream_seed);
  int cur = -1;
  int tx = 0, rsub = 0, txl = 0, txr = 0;
  bool worker = false;
  if (tid < kMsb) stats.reset(tid);

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      const int u = (int)atomicAdd(&b->work_next, 1u);
      int loc = 0;
      const int p = u < total ? queue_pop(b, u, &loc) : -1;
      s_pop = p;
      s_unit = loc;
      if (p >= 0 && p != cur) {  // parameters of a new population
        const PopDev* st = b->pops + p;
        P.L = st->L; P.N = st->N; P.h = st->N >> 1; P.Wr = st->Wr; P.rpp = st->rpp; P.npass = st->npass;
        P.kconst = st->kconst;
        P.step = st->step;
        P.sweeps = energy_only ? 0 : st->sweeps;
        P.nbatch = (st->npass + kKB - 1) / kKB;
        P.tag = kTagMscSweep | (uint32_t)st->pop_id;
        P.T4 = st->thr[(size_t)st->step * kThrPerStep + 10];
        P.T8 = st->thr[(size_t)st->step * kThrPerStep + 11];
        P.seed = st->seed;
        const int rg_prev = (st->R_prev + kMsb - 1) / kMsb;
        P.iseq = st->iseq + (st->step > 0 ? (unsigned long long)rg_prev * kMsb : 0ull);
        P.words = (uint32_t*)st->spins[st->parity];
        P.act = st->active[st->parity];
        P.E = st->E;
        P.M = st->M;
      }
    }
    if (tid < kMsb) { s_cntE[tid] = 0; s_cntM[tid] = 0; }
    __syncthreads();
    const int p = s_pop, gi = s_unit;
    if (p < 0) break;
    if (p != cur) {  // block-uniform
      if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
      cur = p;
      const int Wr = P.Wr;
      worker = tid < Wr * P.rpp;
      tx = worker ? tid % Wr : 0;
      rsub = worker ? tid / Wr : 0;
      txl = (tx == 0 ? Wr - 1 : tx - 1);
      txr = (tx + 1 == Wr ? 0 : tx + 1);
      if (tid < kMsb) {
        const uint32_t d4 = 0u - ((P.T4 >> (31 - tid)) & 1u), d8 = 0u - ((P.T8 >> (31 - tid)) & 1u);
        s_dig[tid] = make_uint2(d8, d4 ^ d8);
      }
    }
    const int N = P.N, h = P.h;
    uint32_t* words = P.words;
    const uint4* gsrc = (const uint4*)(words + (size_t)gi * N);
    uint4* lat4 = (uint4*)lat;
    for (int v = tid; v < (N >> 2); v += blockDim.x) lat4[v] = gsrc[v];
    __syncthreads();

    const int sweeps = P.sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        uint32_t* self = lat + (hf ? h : 0);
        const uint32_t* oth = lat + (hf ? 0 : h);
        const int L = P.L, Wr = P.Wr, rpp = P.rpp, npass = P.npass;
        if (MODE == kRefCoords) {
#pragma unroll 1
          for (int pass = 0; pass < npass; ++pass) {
            const int ty = rsub + pass * rpp;
            const bool valid = worker && ty < L;
            const int tyc = valid ? ty : 0;
            const int row = tyc * Wr, rowu = (tyc == 0 ? L - 1 : tyc - 1) * Wr, rowd = (tyc + 1 == L ? 0 : tyc + 1) * Wr;
            const int idx = row + tx;
            // horizontal neighbour not at the same idx (PAisingMSC.cu:203, 238)
            const bool left = (hf == 0) == ((tyc & 1) == 0);
            const uint32_t s = self[idx];
            const uint32_t n1 = oth[row + (left ? txl : txr)], n2 = oth[idx], n3 = oth[rowu + tx], n4 = oth[rowd + tx];
            uint32_t s0, s1, s2;
            adder4(s ^ n1, s ^ n2, s ^ n3, s ^ n4, s0, s1, s2);
            const int t = idx & (kRefThreads - 1), k = idx >> 7;
            const int K = P.kconst ? P.kconst : (t < h ? (h - t + kRefThreads - 1) / kRefThreads : 0);
            const unsigned long long sub = P.iseq + (unsigned long long)t + (unsigned long long)kRefThreads * gi;
            uint32_t ran = ref_word(P.seed, sub, (unsigned long long)sw * 2 * K + (unsigned long long)hf * K + k);
            const uint32_t T4 = P.T4, T8 = P.T8;
            uint32_t c4 = 0, c8 = 0;
#pragma unroll 8
            for (int i = 0; i < kMsb; ++i) {
              c4 |= (ran < T4 ? 1u : 0u) << i;
              c8 |= (ran < T8 ? 1u : 0u) << i;
              ran = kLcgA * ran + kLcgC;
            }
            const uint32_t hi = s1 | s2;
            const uint32_t acc = hi | (~hi & ((s0 & c4) | (~s0 & c8)));
            if (valid) self[idx] = s ^ acc;
          }
        } else {
          const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
#pragma unroll 1
          for (int p0 = 0; p0 < npass; p0 += kKB) {
            uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
            int ix[kKB];
#pragma unroll
            for (int k = 0; k < kKB; ++k) {
              const int pass = p0 + k;
              const int ty = rsub + pass * rpp;
              const bool valid = worker && pass < npass && ty < L;
              const int tyc = valid ? ty : 0;
              const int row = tyc * Wr, rowu = (tyc == 0 ? L - 1 : tyc - 1) * Wr, rowd = (tyc + 1 == L ? 0 : tyc + 1) * Wr;
              const int idx = row + tx;
              const bool left = (hf == 0) == ((tyc & 1) == 0);
              const uint32_t s = self[idx];
              const uint32_t n1 = oth[row + (left ? txl : txr)], n2 = oth[idx], n3 = oth[rowu + tx], n4 = oth[rowd + tx];
              uint32_t s0, s1, s2;
              adder4(s ^ n1, s ^ n2, s ^ n3, s ^ n4, s0, s1, s2);
              av[k] = s0;
              ac[k] = s1 | s2;
              un[k] = valid ? ~(s1 | s2) : 0u;
              ix[k] = valid ? idx : -1;
              site[k] = (uint32_t)gi * (uint32_t)h + (uint32_t)idx;
            }
            const uint32_t chain = ((uint32_t)gi * blockDim.x + (uint32_t)tid) * (uint32_t)P.nbatch + (uint32_t)(p0 / kKB);
            accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig);
#pragma unroll
            for (int k = 0; k < kKB; ++k)
              if (ix[k] >= 0) self[ix[k]] ^= ac[k];
          }
        }
        __syncthreads();
      }
    }

    // energy and magnetisation per replica bit: the left and up bond of every
    // A and B site (PAisingMSC.cu:272-294), counted per bit with warp ballots.
    int cE = 0, cM = 0;  // lane k accumulates bit k
    {
      const int L = P.L, Wr = P.Wr, rpp = P.rpp, npass = P.npass;
      for (int pass = 0; pass < npass; ++pass) {
        const int ty = rsub + pass * rpp;
        const bool valid = worker && ty < L;
        uint32_t s0 = 0, s1 = 0, s2 = 0, sA = 0, sB = 0;
        if (valid) {
          const int row = ty * Wr, idx = row + tx, iL = row + txl, iU = (ty + 1 == L ? 0 : ty + 1) * Wr + tx;
          sA = lat[idx];
          sB = lat[h + idx];
          uint32_t Ai2, Bi2;
          if (ty & 1) { Ai2 = sB; Bi2 = lat[iL]; }
          else { Ai2 = lat[h + iL]; Bi2 = sA; }
          adder4(sA ^ Ai2, sA ^ lat[h + iU], sB ^ Bi2, sB ^ lat[iU], s0, s1, s2);
        }
#pragma unroll 4
        for (int k = 0; k < kMsb; ++k) {
          const int e = __popc(__ballot_sync(kFull, (s0 >> k) & 1u)) + 2 * __popc(__ballot_sync(kFull, (s1 >> k) & 1u)) +
                        4 * __popc(__ballot_sync(kFull, (s2 >> k) & 1u));
          const int m = __popc(__ballot_sync(kFull, (sA >> k) & 1u)) + __popc(__ballot_sync(kFull, (sB >> k) & 1u));
          if (lane == k) { cE += e; cM += m; }
        }
      }
    }
    atomicAdd(&s_cntE[lane], cE);
    atomicAdd(&s_cntM[lane], cM);
    uint4* gdst = (uint4*)(words + (size_t)gi * N);
    for (int v = tid; v < (N >> 2); v += blockDim.x) gdst[v] = lat4[v];
    __syncthreads();
    if (tid < kMsb) {
      const int E = 2 * s_cntE[tid] - 2 * N, Mg = 2 * s_cntM[tid] - N;
      P.E[gi * kMsb + tid] = E;
      P.M[gi * kMsb + tid] = Mg;
      if (P.act[gi * kMsb + tid]) stats.add(tid, E, Mg);
    }
  }
  if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
}

// -------------------------------------------------------------- resample
// resampleKer places offspring number s (in the scan order of
// (old group, bit)) at new group s % rg_new, bit s / rg_new
// (PAisingMSC.cu:413-414).  Here every new word gathers its 32 bits:
// bit k of new group j comes from old replica src[k*rg_new + j].
__global__ void msc_resample_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  if (!pop_stepping(st)) return;
  const int N = st->N, Rn = st->R_cur, rgn = (Rn + kMsb - 1) / kMsb;
  const uint32_t* old = (const uint32_t*)st->spins[st->parity ^ 1];
  uint32_t* neu = (uint32_t*)st->spins[st->parity];
  uint8_t* act = st->active[st->parity];
  const uint32_t* src = st->src;
  const long long total = (long long)rgn * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / N), t = (int)(e - (long long)j * N);
    uint32_t w = 0;
#pragma unroll 4
    for (int k = 0; k < kMsb; ++k) {
      const int s = k * rgn + j;
      if (s < Rn) {
        const uint32_t lin = src[s];
        w |= ((old[(size_t)(lin >> 5) * N + t] >> (lin & 31u)) & 1u) << k;
      }
    }
    neu[e] = w;
    if (t < kMsb) act[j * kMsb + t] = (t * rgn + j) < Rn;
  }
}

// -------------------------------------------------------------- geometry
static int pick_rpp(int L, int Wr) {
  int best = 1;
  for (int r = 1; r <= L; ++r)
    if (L % r == 0 && Wr * r <= kSweepThreads) best = r;
  return best;
}

bool msc_geom(int L, SweepGeom* g) {
  if (L < 8 || L % 2 != 0 || L > 128) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 2;
  g->rpp = pick_rpp(L, g->Wr);
  g->T = g->Wr * g->rpp;
  g->npass = (L + g->rpp - 1) / g->rpp;
  g->kconst = (g->half % kRefThreads == 0) ? g->half / kRefThreads : 0;
  g->smem = g->N * 4;
  return true;
}

// -------------------------------------------------------------- launchers
static const void* msc_sweep_fn(int rng_mode) {
  return rng_mode == kRefCoords ? (const void*)msc_sweep_kernel<kRefCoords> : (const void*)msc_sweep_kernel<kNative>;
}

cudaError_t msc_sweep_setup(int rng_mode, int smem, SweepLaunch* out) {
  return persistent_launch(msc_sweep_fn(rng_mode), kSweepThreads, smem, out);
}

cudaError_t launch_msc_sweep(BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                             const SweepLaunch& sl, cudaStream_t s) {
  if (rng_mode == kRefCoords)
    msc_sweep_kernel<kRefCoords><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  else
    msc_sweep_kernel<kNative><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  return cudaGetLastError();
}

cudaError_t launch_msc_init(PopDev* pops, int npop, cudaStream_t s) {
  msc_init_kernel<<<dim3(256, npop), 256, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_msc_resample(PopDev* pops, int npop, cudaStream_t s) {
  int dev, nsm;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int x = (nsm * 8 + npop - 1) / npop;
  msc_resample_kernel<<<dim3(x < 16 ? 16 : x, npop), 256, 0, s>>>(pops);
  return cudaGetLastError();
}

}  // namespace pa
