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

#include "pa_device.cuh"
#include "pa_kernels.h"

namespace pa {

namespace {

constexpr uint32_t kLcgA = 1664525u;     // PAisingMSC.cu:53
constexpr uint32_t kLcgC = 1013904223u;  // PAisingMSC.cu:54

// Bitsliced count of anti-parallel neighbours (4 inputs -> 3 bit planes),
// the adder of PAisingMSC.cu:212-218.
__device__ __forceinline__ void adder4(uint32_t I1, uint32_t I2, uint32_t I3, uint32_t I4, uint32_t& s0,
                                       uint32_t& s1, uint32_t& s2) {
  const uint32_t x12 = I1 ^ I2, x34 = I3 ^ I4, a12 = I1 & I2, a34 = I3 & I4;
  s0 = x12 ^ x34;
  s1 = (x12 & x34) ^ a12 ^ a34;
  s2 = a12 & a34;
}

// One binary digit of the comparison U < T/2^32 done for 32 bits at once:
// U's digit j is bit i of the random word u for replica bit i, T's digit j
// is selected per bit from T4 (bits in s0: one anti-parallel neighbour,
// dE = 4) or T8 (no anti-parallel neighbour, dE = 8).  dg = (D8_j, D4_j ^ D8_j)
// with D_j = all ones iff digit j of the threshold is 1.  Bits decided at this
// digit leave `und` (a subtraction, since they are a subset of it); those
// decided "less" enter `lt`.
__device__ __forceinline__ void digit_step(uint32_t u, uint32_t s0, uint2 dg, uint32_t& und, uint32_t& lt) {
  const uint32_t p = (s0 & dg.y) ^ dg.x;
  const uint32_t dec = und & (p ^ u);
  lt |= dec & p;
  und -= dec;
}

}  // namespace

// ------------------------------------------------------------------ init
__global__ void msc_init_kernel(PopDev* st) {
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
// One CTA anneals one group of 32 replicas at a time (dynamic work counter),
// both sublattices resident in shared memory.  Thread (rsub, tx) owns site
// column tx of sublattice rows rsub, rsub+rpp, ...
//
// MODE kRefCoords: decisions of checkKerALL exactly -- one draw per word-site
//   (ctr = sw*2K + hf*K + k of subsequence iseq + t + 128 g) expanded to 32
//   numbers by the LCG and compared with T4 = ceil(2^32 e^-4b), T8.
// MODE kNative: U_i < T/2^32 for the 32 replica bits is decided digit by
//   digit, most significant first; digit j of every U_i comes from one fresh
//   Philox4x32-10 output word, and the warp stops drawing once every bit of
//   every lane is decided (on average ~11 of the 32 possible digits).  Each
//   replica's acceptance probability is exactly T/2^32, as in the reference.
template <int MODE>
__global__ void __launch_bounds__(256, 5) msc_sweep_kernel(PopDev* st, SweepGeom g, int sweeps) {
  extern __shared__ __align__(16) uint32_t lat[];  // N words: A then B
  __shared__ int s_unit;
  __shared__ int s_cntE[kMsb], s_cntM[kMsb];
  __shared__ uint2 s_dig[kMsb];  // per digit j: (D8_j, D4_j ^ D8_j)

  const int tid = threadIdx.x, lane = tid & 31;
  const int L = g.L, N = g.N, h = g.half, Wr = g.Wr;
  const int R = st->R_cur, step = st->step;
  const int rg = (R + kMsb - 1) / kMsb;
  const unsigned long long seed = st->seed;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const uint32_t tag = kTagMscSweep | (uint32_t)st->pop_id;
  const int rg_prev = (st->R_prev + kMsb - 1) / kMsb;
  const unsigned long long iseq = st->iseq + (step > 0 ? (unsigned long long)rg_prev * kMsb : 0ull);
  const uint32_t T4 = st->thr[(size_t)step * kThrPerStep + 10], T8 = st->thr[(size_t)step * kThrPerStep + 11];
  uint32_t* words = (uint32_t*)st->spins[st->parity];
  const uint8_t* act = st->active[st->parity];
  if (tid < kMsb) {
    const uint32_t d4 = 0u - ((T4 >> (31 - tid)) & 1u), d8 = 0u - ((T8 >> (31 - tid)) & 1u);
    s_dig[tid] = make_uint2(d8, d4 ^ d8);
  }

  const bool worker = tid < g.T;
  const int tx = worker ? tid % Wr : 0, rsub = worker ? tid / Wr : 0;
  const int txl = (tx == 0 ? Wr - 1 : tx - 1), txr = (tx + 1 == Wr ? 0 : tx + 1);

  long long sE = 0, sE2 = 0, sM = 0, sM2 = 0;
  U128 m4{0, 0};
  int emin = INT_MAX;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_unit = (int)atomicAdd(&st->work_next, 1u);
    if (tid < kMsb) { s_cntE[tid] = 0; s_cntM[tid] = 0; }
    __syncthreads();
    const int gi = s_unit;
    if (gi >= rg) break;
    const uint4* gsrc = (const uint4*)(words + (size_t)gi * N);
    uint4* lat4 = (uint4*)lat;
    for (int v = tid; v < (N >> 2); v += blockDim.x) lat4[v] = gsrc[v];
    __syncthreads();

    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        uint32_t* self = lat + (hf ? h : 0);
        const uint32_t* oth = lat + (hf ? 0 : h);
#pragma unroll 1
        for (int pass = 0; pass < g.npass; ++pass) {
          const int ty = rsub + pass * g.rpp;
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
          uint32_t acc;
          if (MODE == kRefCoords) {
            const int t = idx & (kRefThreads - 1), k = idx >> 7;
            const int K = g.kconst ? g.kconst : (t < h ? (h - t + kRefThreads - 1) / kRefThreads : 0);
            const unsigned long long sub = iseq + (unsigned long long)t + (unsigned long long)kRefThreads * gi;
            uint32_t ran = ref_word(seed, sub, (unsigned long long)sw * 2 * K + (unsigned long long)hf * K + k);
            uint32_t c4 = 0, c8 = 0;
#pragma unroll 8
            for (int i = 0; i < kMsb; ++i) {
              c4 |= (ran < T4 ? 1u : 0u) << i;
              c8 |= (ran < T8 ? 1u : 0u) << i;
              ran = kLcgA * ran + kLcgC;
            }
            const uint32_t hi = s1 | s2;
            acc = hi | (~hi & ((s0 & c4) | (~s0 & c8)));
          } else {
            uint32_t und = valid ? ~(s1 | s2) : 0u, lt = 0;
            const uint32_t c0 = (uint32_t)gi * (uint32_t)h + (uint32_t)idx;
            const uint32_t cbase = (uint32_t)((sw * 2 + hf) << 3);
#pragma unroll 1
            for (int c = 0; c < 8; ++c) {
              if (!__any_sync(0xffffffffu, und != 0u)) break;
              const U4 rn = philox10(c0, cbase | (uint32_t)c, (uint32_t)step, tag, k0, k1);
              digit_step(rn.x, s0, s_dig[4 * c + 0], und, lt);
              digit_step(rn.y, s0, s_dig[4 * c + 1], und, lt);
              digit_step(rn.z, s0, s_dig[4 * c + 2], und, lt);
              digit_step(rn.w, s0, s_dig[4 * c + 3], und, lt);
            }
            acc = (s1 | s2) | lt;
          }
          if (valid) self[idx] = s ^ acc;
        }
        __syncthreads();
      }
    }

    // energy and magnetisation per replica bit: the left and up bond of every
    // A and B site (PAisingMSC.cu:272-294), counted per bit with warp ballots.
    int cE = 0, cM = 0;  // lane k accumulates bit k
    for (int pass = 0; pass < g.npass; ++pass) {
      const int ty = rsub + pass * g.rpp;
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
        const int e = __popc(__ballot_sync(0xffffffffu, (s0 >> k) & 1u)) +
                      2 * __popc(__ballot_sync(0xffffffffu, (s1 >> k) & 1u)) +
                      4 * __popc(__ballot_sync(0xffffffffu, (s2 >> k) & 1u));
        const int m = __popc(__ballot_sync(0xffffffffu, (sA >> k) & 1u)) + __popc(__ballot_sync(0xffffffffu, (sB >> k) & 1u));
        if (lane == k) { cE += e; cM += m; }
      }
    }
    atomicAdd(&s_cntE[lane], cE);
    atomicAdd(&s_cntM[lane], cM);
    uint4* gdst = (uint4*)(words + (size_t)gi * N);
    for (int v = tid; v < (N >> 2); v += blockDim.x) gdst[v] = lat4[v];
    __syncthreads();
    if (tid < kMsb) {
      const int E = 2 * s_cntE[tid] - 2 * N, Mg = 2 * s_cntM[tid] - N;
      st->E[gi * kMsb + tid] = E;
      st->M[gi * kMsb + tid] = Mg;
      if (act[gi * kMsb + tid]) {
        const long long am = Mg < 0 ? -(long long)Mg : (long long)Mg;
        sE += E;
        sE2 += (long long)E * E;
        sM += am;
        sM2 += am * am;
        unsigned long long lo, hi;
        m4_of(Mg, lo, hi);
        u128_add(m4, lo, hi);
        emin = E < emin ? E : emin;
      }
    }
  }
  // flush the statistics of this CTA (warp 0 holds them, one lane per bit)
  if (tid < kMsb) {
    sE = warp_sum(sE);
    sE2 = warp_sum(sE2);
    sM = warp_sum(sM);
    sM2 = warp_sum(sM2);
    emin = warp_min(emin);
    // 128-bit sum across the warp: reduce lo with carries into hi
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long lo = __shfl_xor_sync(0xffffffffu, m4.lo, o);
      const unsigned long long hi = __shfl_xor_sync(0xffffffffu, m4.hi, o);
      u128_add(m4, lo, hi);
    }
    if (tid == 0 && emin != INT_MAX) {
      atomicAdd((unsigned long long*)&st->sE, (unsigned long long)sE);
      atomicAdd((unsigned long long*)&st->sE2, (unsigned long long)sE2);
      atomicAdd((unsigned long long*)&st->sM, (unsigned long long)sM);
      atomicAdd((unsigned long long*)&st->sM2, (unsigned long long)sM2);
      u128_atomic_add(&st->sM4lo, &st->sM4hi, m4.lo, m4.hi);
      atomicMin(&st->Emin_acc, emin);
    }
  }
}

// -------------------------------------------------------------- resample
// resampleKer places offspring number s (in the scan order of
// (old group, bit)) at new group s % rg_new, bit s / rg_new
// (PAisingMSC.cu:413-414).  Here every new word gathers its 32 bits:
// bit k of new group j comes from old replica src[k*rg_new + j].
__global__ void msc_resample_kernel(PopDev* st) {
  if (st->error) return;
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

// -------------------------------------------------------------- launchers
static int pick_rpp(int L, int Wr, int max_threads) {
  int best = 1;
  for (int r = 1; r <= L; ++r)
    if (L % r == 0 && Wr * r <= max_threads) best = r;
  return best;
}

bool msc_geom(int L, int max_threads, SweepGeom* g) {
  if (L < 8 || L % 2 != 0 || L > 128) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 2;
  g->rpp = pick_rpp(L, g->Wr, max_threads);
  g->T = g->Wr * g->rpp;
  g->block = (g->T + 31) / 32 * 32;
  g->npass = (L + g->rpp - 1) / g->rpp;
  g->kconst = (g->half % kRefThreads == 0) ? g->half / kRefThreads : 0;
  g->smem = g->N * 4;
  g->grid = 0;
  return true;
}

cudaError_t msc_sweep_setup(SweepGeom* g, int rng_mode) {
  const void* fn = rng_mode == kRefCoords ? (const void*)msc_sweep_kernel<kRefCoords> : (const void*)msc_sweep_kernel<kNative>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g->smem);
  if (e != cudaSuccess) return e;
  int dev, nsm, per;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, g->block, g->smem);
  if (e != cudaSuccess) return e;
  g->grid = nsm * (per > 0 ? per : 1);
  return cudaSuccess;
}

cudaError_t launch_msc_init(PopDev* st, const PopDev& h, cudaStream_t s) {
  const int rg = (h.Rinit + kMsb - 1) / kMsb;
  long long total = (long long)rg * (h.N / 2);
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  msc_init_kernel<<<blocks, 256, 0, s>>>(st);
  return cudaGetLastError();
}

cudaError_t launch_msc_sweep(PopDev* st, const SweepGeom& g, int rng_mode, int sweeps, cudaStream_t s) {
  if (rng_mode == kRefCoords)
    msc_sweep_kernel<kRefCoords><<<g.grid, g.block, g.smem, s>>>(st, g, sweeps);
  else
    msc_sweep_kernel<kNative><<<g.grid, g.block, g.smem, s>>>(st, g, sweeps);
  return cudaGetLastError();
}

cudaError_t launch_msc_resample(PopDev* st, const PopDev& h, cudaStream_t s) {
  int dev, nsm;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  msc_resample_kernel<<<nsm * 8, 256, 0, s>>>(st);
  return cudaGetLastError();
}

}  // namespace pa
